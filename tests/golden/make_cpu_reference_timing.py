"""Times the reference's own VCMTracer (oracle/_ref/vcm_driver, built from the reference
sources by oracle/ref/Makefile) on the VCM benchmark scene at its full size: the Cornell
room with the homogeneous-medium sphere at 512 x 512, depth 16, r0 0.0963, alpha 0.75,
for a few iterations, and records the wall time per iteration with the thread count and
the machine in cpu_reference_vcm_512.json. The reference ties its light paths to the
pixel count (width x height = 262,144 per iteration, src/VCMTracer.cpp:41-52); the GPU
section of the benchmark traces 2^20 per iteration.

The reference's sources are only on the build machine, so this runs there, not on the
GPU machine; bench.py reports the recorded figure beside the GPU's with that provenance.

    python tests/golden/make_cpu_reference_timing.py [iterations] [threads]
"""
import json
import os
import platform
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    from renderx_gb300 import scenes, sceneio
    iters = int(sys.argv[1]) if len(sys.argv) > 1 else 2
    threads = int(sys.argv[2]) if len(sys.argv) > 2 else os.cpu_count()
    driver = os.path.join(ROOT, "oracle", "_ref", "vcm_driver")
    if not os.path.exists(driver):
        sys.exit(f"{driver} missing: build it with make -C oracle/ref REF=<reference checkout>")
    res, depth, r0, alpha = 512, 16, 0.0963, 0.75
    sc = scenes.medium_scene(res, res)
    with tempfile.TemporaryDirectory() as td:
        cfg = sceneio.write_config(sc, td, "VCM", depth, radius=r0)
        pre = os.path.join(td, "out")
        out = subprocess.run([driver, cfg, str(iters), "0", str(r0), str(alpha), pre, str(threads)], check=True,
                             capture_output=True, text=True, cwd=td).stdout.strip().splitlines()[-1].split()
    secs = float(out[-1])
    rec = {"workload": f"VCMTracer, Cornell room + homogeneous-medium sphere, {res}x{res}, depth {depth}, "
                       f"r0 {r0}, alpha {alpha}",
           "implementation": "the reference's own VCMTracer::renderPixels, built from its sources (-O2 -fopenmp)",
           "light_paths_per_iteration": res * res, "iterations": iters, "seconds": secs,
           "ms_per_iteration": secs / iters * 1e3, "threads": threads,
           "machine": f"{platform.machine()} build machine ({os.cpu_count()} cores), not the GPU machine"}
    path = os.path.join(HERE, "cpu_reference_vcm_512.json")
    with open(path, "w") as f:
        json.dump(rec, f, indent=1)
    print(path, json.dumps(rec))


if __name__ == "__main__":
    main()
