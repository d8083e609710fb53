"""Seeded synthetic scenes for the light-transport path.

The reference ships no scene data (its data/ folder is git-ignored), so the workloads
are authored here from their numeric descriptions:

* ``cornell_box()``: the 36-triangle Cornell box in a 5.56^3 room (5 walls x 2, light
  x 2, two boxes x 12), y up, camera looking down +z.
* ``sphere_field()``: the Cornell box plus N seed-placed icospheres (subdivision 5 =
  20480 triangles each) with value-noise radial displacement; 200 spheres give
  4,096,036 triangles.
* ``hit_rays()``: seeded closest-hit batches, origins uniform in the room and
  directions uniform on the sphere (z = 1-2u, phi = 2 pi u).

A scene is a list of objects. Each object holds world-space float32 vertices, uint32
triangle vertex indices local to the object, optional per-vertex normals and a material
record. Objects are concatenated in list order into one triangle list, the way
Scene::buildKDTree concatenates them (reference src/Scene.cpp:248-285), so a global
triangle id is the object's triangle offset plus its local triangle id.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

ROOM = 5.56

# Material kinds; the numeric values are the ABI's material codes.
DIFFUSE, GLOSSY, REFRACTIVE, EMISSIVE, PHONG, REFLECTIVE, VPM = 0, 1, 2, 3, 4, 5, 6


@dataclass
class Material:
    kind: int
    color: tuple = (0.0, 0.0, 0.0)     # albedo / glossy colour / emission / surface colour
    coeff: float = 1.0                 # glossy exponent
    ior: float = 1.5                   # refractive index (negative: mirror)
    diffuse_color: tuple = (0.0, 0.0, 0.0)  # Phong: diffuse component
    sigma_s: tuple = (0.0, 0.0, 0.0)   # homogeneous medium
    sigma_a: tuple = (0.0, 0.0, 0.0)
    g: float = 0.0
    decay: tuple = (1.0, 1.0, 1.0)     # refractive decayColor (per unit length)
    step_size: float = 0.0005          # medium: PhotonMap ray-marching step (SceneVPMObject::stepSize)


@dataclass
class Obj:
    name: str
    verts: np.ndarray                  # (nv, 3) float32, world space
    tris: np.ndarray                   # (nt, 3) uint32, local indices
    material: Material
    normals: np.ndarray | None = None  # (nv, 3) float32 per-vertex normals or None


@dataclass
class Camera:
    """Pinhole camera with the reference's integer ``sightDist`` (pixels), Camera.h:16."""
    width: int
    height: int
    sight_dist: int
    position: tuple
    focus: tuple
    up: tuple = (0.0, 1.0, 0.0)


@dataclass
class Scene:
    objects: list = field(default_factory=list)
    camera: Camera | None = None

    # -- flattening -------------------------------------------------------------------
    def flatten(self):
        """Concatenate objects: returns dict with verts (nv,3) f32, tris (nt,3) u32
        (global vertex indices), tri_obj (nt,) u32, tri_local (nt,) u32,
        normals (nv,3) f32 (zeros where an object has none), has_normals (nobj,) u8."""
        vs, ts, to, tl, ns, hn = [], [], [], [], [], []
        voff = 0
        for oi, o in enumerate(self.objects):
            vs.append(np.asarray(o.verts, np.float32))
            ts.append(np.asarray(o.tris, np.uint32) + np.uint32(voff))
            nt = len(o.tris)
            to.append(np.full(nt, oi, np.uint32))
            tl.append(np.arange(nt, dtype=np.uint32))
            if o.normals is None:
                ns.append(np.zeros((len(o.verts), 3), np.float32))
                hn.append(0)
            else:
                ns.append(np.asarray(o.normals, np.float32))
                hn.append(1)
            voff += len(o.verts)
        return dict(
            verts=np.ascontiguousarray(np.concatenate(vs)),
            tris=np.ascontiguousarray(np.concatenate(ts)),
            tri_obj=np.concatenate(to),
            tri_local=np.concatenate(tl),
            normals=np.ascontiguousarray(np.concatenate(ns)),
            has_normals=np.asarray(hn, np.uint8),
        )

    @property
    def num_triangles(self) -> int:
        return int(sum(len(o.tris) for o in self.objects))


# ------------------------------------------------------------------------------------
# Cornell box
# ------------------------------------------------------------------------------------
def _quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3); the face normal is (p1-p0)x(p2-p0)."""
    v = np.array([p0, p1, p2, p3], np.float32)
    t = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    return v, t


def _oriented_quad(center, u, v, normal):
    """Quad centred at ``center`` spanned by half-extents u, v, wound so that its face
    normal points along ``normal``."""
    c, u, v = np.asarray(center, np.float64), np.asarray(u, np.float64), np.asarray(v, np.float64)
    p = [c - u - v, c + u - v, c + u + v, c - u + v]
    if np.dot(np.cross(p[1] - p[0], p[2] - p[0]), normal) < 0:
        p = p[::-1]
    return _quad(*p)


def _box(center, size, angle_deg):
    """Axis box of ``size`` rotated about the vertical axis by ``angle_deg``, outward
    normals, 12 triangles."""
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)
    ex = np.array([ca, 0.0, -sa]) * size[0] / 2
    ey = np.array([0.0, 1.0, 0.0]) * size[1] / 2
    ez = np.array([sa, 0.0, ca]) * size[2] / 2
    c = np.asarray(center, np.float64)
    verts, tris = [], []
    for axis, (e1, e2) in ((ex, (ey, ez)), (ey, (ez, ex)), (ez, (ex, ey))):
        for sgn in (1.0, -1.0):
            n = sgn * axis / np.linalg.norm(axis)
            v, t = _oriented_quad(c + sgn * axis, e1, e2, n)
            tris.append(t + len(verts) * 4)
            verts.append(v)
    return np.concatenate(verts).astype(np.float32), np.concatenate(tris).astype(np.uint32)


def cornell_box(width: int = 256, height: int = 256, fov_deg: float = 40.0, light_scale: float = 1.0) -> Scene:
    """The 36-triangle Cornell box. Walls diffuse 0.73 (floor, ceiling, back), left
    wall (0.63,0.065,0.05), right wall (0.14,0.45,0.091), ceiling light 1.3x1.05 with
    emission (17,12,4); tall box 1.65x1.65x3.3 rotated 15 deg, short box 1.65^3
    rotated -18 deg. ``light_scale`` scales the light's area (1% ceiling-area light:
    light_scale = sqrt(0.01*5.56^2/(1.3*1.05)))."""
    R = ROOM
    h = R / 2
    white = Material(DIFFUSE, (0.73, 0.73, 0.73))
    objs = []

    def wall(name, center, u, v, n, mat):
        vv, tt = _oriented_quad(center, u, v, np.asarray(n, np.float64))
        objs.append(Obj(name, vv, tt, mat))

    wall("floor", (h, 0, h), (h, 0, 0), (0, 0, h), (0, 1, 0), white)
    wall("ceiling", (h, R, h), (h, 0, 0), (0, 0, h), (0, -1, 0), white)
    wall("back", (h, h, R), (h, 0, 0), (0, h, 0), (0, 0, -1), white)
    # camera right vector is front x up = -x, so the image's left wall sits at x = R
    wall("left", (R, h, h), (0, h, 0), (0, 0, h), (-1, 0, 0), Material(DIFFUSE, (0.63, 0.065, 0.05)))
    wall("right", (0, h, h), (0, h, 0), (0, 0, h), (1, 0, 0), Material(DIFFUSE, (0.14, 0.45, 0.091)))
    lw, ld = 1.3 * light_scale / 2, 1.05 * light_scale / 2
    wall("light", (h, R - 0.01, h), (lw, 0, 0), (0, 0, ld), (0, -1, 0), Material(EMISSIVE, (17.0, 12.0, 4.0)))
    bv, bt = _box((3.68, 1.65, 3.51), (1.65, 3.3, 1.65), 15.0)
    objs.append(Obj("tallbox", bv, bt, white))
    bv, bt = _box((1.85, 0.825, 1.69), (1.65, 1.65, 1.65), -18.0)
    objs.append(Obj("shortbox", bv, bt, white))
    cam = cornell_camera(width, height, fov_deg)
    return Scene(objs, cam)


def cornell_camera(width: int, height: int, fov_deg: float = 40.0) -> Camera:
    # integer sightDist = round((height/2)/tan(fov/2)) pixels (Camera.h:16 stores an int)
    sd = int(round((height / 2) / math.tan(math.radians(fov_deg) / 2)))
    return Camera(width, height, sd, (2.78, 2.73, -8.0), (2.78, 2.73, 0.0), (0.0, 1.0, 0.0))


# ------------------------------------------------------------------------------------
# Icospheres with value-noise displacement
# ------------------------------------------------------------------------------------
_ICO_CACHE: dict = {}


def icosphere(subdiv: int):
    """Unit icosphere: (verts (nv,3) f64, faces (nf,3) int64), outward winding."""
    if subdiv in _ICO_CACHE:
        return _ICO_CACHE[subdiv]
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        es = np.sort(e, axis=1)
        key = es[:, 0] * (len(v) + 1) + es[:, 1]
        uk, inv = np.unique(key, return_inverse=True)
        a, b = uk // (len(v) + 1), uk % (len(v) + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1).T + len(v)  # midpoints of edges (01,12,20)
        v = np.concatenate([v, mid])
        f = np.concatenate([
            np.stack([f[:, 0], m[:, 0], m[:, 2]], 1),
            np.stack([f[:, 1], m[:, 1], m[:, 0]], 1),
            np.stack([f[:, 2], m[:, 2], m[:, 1]], 1),
            np.stack([m[:, 0], m[:, 1], m[:, 2]], 1)])
    _ICO_CACHE[subdiv] = (v, f)
    return v, f


def _value_noise(p: np.ndarray, lattice: np.ndarray) -> np.ndarray:
    """Smooth 3D value noise in [-1,1] on a periodic integer lattice."""
    n = lattice.shape[0]
    i0 = np.floor(p).astype(np.int64)
    fr = p - i0
    w = fr * fr * (3 - 2 * fr)
    out = np.zeros(len(p))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                c = lattice[(i0[:, 0] + dx) % n, (i0[:, 1] + dy) % n, (i0[:, 2] + dz) % n]
                wt = (w[:, 0] if dx else 1 - w[:, 0]) * (w[:, 1] if dy else 1 - w[:, 1]) * (w[:, 2] if dz else 1 - w[:, 2])
                out += wt * c
    return out


def vertex_normals(verts: np.ndarray, faces: np.ndarray) -> np.ndarray:
    """Area-weighted vertex normals (unit length)."""
    v = verts.astype(np.float64)
    fn = np.cross(v[faces[:, 1]] - v[faces[:, 0]], v[faces[:, 2]] - v[faces[:, 0]])
    vn = np.zeros_like(v)
    for k in range(3):
        np.add.at(vn, faces[:, k], fn)
    vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-30)
    return vn


def sphere_field(n_spheres: int = 200, subdiv: int = 5, seed: int = 1, width: int = 1024, height: int = 1024,
                 glossy_frac: float = 0.3, diffuse_frac: float = 0.5, glossy_exp=(10.0, 1000.0),
                 light_scale: float = 1.0, displacement: float = 0.05) -> Scene:
    """Cornell box plus ``n_spheres`` seed-placed displaced icospheres. Radius
    U[0.1,0.4]; materials diffuse (albedo U[0.2,0.8]) / Phong-lobe glossy (exponent
    log-U[glossy_exp]) / dielectric (IOR 1.5) with fractions diffuse_frac /
    glossy_frac / rest. Spheres do not overlap one another or the two boxes."""
    rng = np.random.default_rng(seed)
    sc = cornell_box(width, height, light_scale=light_scale)
    uv, uf = icosphere(subdiv)
    lattice = rng.uniform(-1.0, 1.0, size=(32, 32, 32))
    boxes = [((3.68, 1.65, 3.51), 1.2, 3.3), ((1.85, 0.825, 1.69), 1.2, 1.65)]  # centre, xz radius, height
    placed = []
    tries = 0
    while len(placed) < n_spheres:
        tries += 1
        if tries > 200000:
            raise RuntimeError("could not place spheres")
        r = rng.uniform(0.1, 0.4)
        m = r + displacement + 0.02
        c = rng.uniform(m, ROOM - m, size=3)
        if c[1] > ROOM - 0.6 - m:      # keep clear of the light plane
            continue
        ok = all(np.linalg.norm(c - pc) > r + pr + 2 * displacement + 0.02 for pc, pr in placed)
        if ok:
            for bc, br, bh in boxes:
                dxz = math.hypot(c[0] - bc[0], c[2] - bc[2])
                if dxz < br + m and c[1] - m < bh:
                    ok = False
                    break
        if ok:
            placed.append((c, r))
    lg0, lg1 = math.log(glossy_exp[0]), math.log(glossy_exp[1])
    for si, (c, r) in enumerate(placed):
        u = rng.uniform()
        if u < diffuse_frac:
            mat = Material(DIFFUSE, tuple(rng.uniform(0.2, 0.8, 3)))
        elif u < diffuse_frac + glossy_frac:
            mat = Material(GLOSSY, tuple(rng.uniform(0.2, 0.8, 3)), coeff=float(math.exp(rng.uniform(lg0, lg1))))
        else:
            mat = Material(REFRACTIVE, (1.0, 1.0, 1.0), ior=1.5)
        off = rng.uniform(0, 32, 3)
        d = displacement * _value_noise(uv * (2.5 / max(r, 0.1)) + off, lattice)
        p = c[None, :] + (r + d)[:, None] * uv
        vn = vertex_normals(p, uf)
        sc.objects.append(Obj(f"sphere{si}", p.astype(np.float32), uf.astype(np.uint32), mat, vn.astype(np.float32)))
    return sc


GUIDING_LIGHT_SCALE = math.sqrt(0.01 * ROOM * ROOM / (1.3 * 1.05))  # light = 1% of the ceiling


def guiding_scene(width: int = 1024, height: int = 1024, n_spheres: int = 200, subdiv: int = 5,
                  seed: int = 1) -> Scene:
    """The glossy workload of the learned-guiding comparison: the sphere field with 60%
    Phong-lobe glossy spheres (exponent log-U[100,1000]), 30% diffuse, 10% dielectric,
    and the ceiling light shrunk to 1% of the ceiling area."""
    return sphere_field(n_spheres, subdiv, seed, width, height, glossy_frac=0.6, diffuse_frac=0.3,
                        glossy_exp=(100.0, 1000.0), light_scale=GUIDING_LIGHT_SCALE)


def batch_variants(n: int = 64, seed: int = 1, n_medium: int = 8, resolutions=(128, 256, 512, 1024),
                   spp_range=(4, 64)):
    """The batching workload: ``n`` seeded variants of the sphere field. Triangle counts
    log-U[1k, 2M] (sphere subdivision 2..5 and sphere count chosen to match),
    resolution drawn from ``resolutions`` (squared), spp U{spp_range}, depth cap 16,
    Russian roulette from depth 3; the first ``n_medium`` carry the homogeneous-medium
    sphere of ``medium_scene``. Returns a list of (Scene, options dict)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        target = math.exp(rng.uniform(math.log(1e3), math.log(2e6)))
        d = 5
        while d > 2 and 20 * 4 ** d * 4 > target:
            d -= 1
        ns = int(max(1, min(400, round((target - 36) / (20 * 4 ** d)))))
        res = int(rng.choice(list(resolutions)))
        spp = int(rng.integers(spp_range[0], spp_range[1] + 1))
        sc = sphere_field(ns, d, seed=1000 + k, width=res, height=res)
        if k < n_medium:
            med = medium_scene(res, res).objects[-1]
            sc.objects.append(med)
        out.append((sc, dict(spp=spp, max_depth=16, rr_mode=1, nee=False, seed=k + 1)))
    return out


def hit_rays(n: int, seed: int = 7, lo: float = 0.0, hi: float = ROOM):
    """Closest-hit batch: origins U[lo,hi]^3, directions uniform on S^2 with
    z = 1-2u, phi = 2 pi u. Returns (origins (n,3) f32, dirs (n,3) f32)."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    z = 1.0 - 2.0 * rng.uniform(size=n)
    phi = 2.0 * math.pi * rng.uniform(size=n)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    d = np.stack([s * np.cos(phi), s * np.sin(phi), z], 1).astype(np.float32)
    return o, d


def material_spheres(width: int = 64, height: int = 64, subdiv: int = 2) -> Scene:
    """The Cornell room with five smooth-shaded icospheres (vertex normals), one per
    material: diffuse, Phong-lobe glossy, dielectric (IOR 1.5), Phong (glossy +
    diffuse) and mirror."""
    sc = cornell_box(width, height)
    uv, uf = icosphere(subdiv)
    specs = [((0.8, 0.5, 3.5), 0.5, Material(DIFFUSE, (0.7, 0.35, 0.2))),
             ((1.85, 2.2, 1.69), 0.5, Material(GLOSSY, (0.8, 0.8, 0.6), coeff=60.0)),
             ((4.3, 0.8, 1.4), 0.8, Material(REFRACTIVE, (1.0, 1.0, 1.0), ior=1.5)),
             ((3.1, 0.4, 0.45), 0.4, Material(PHONG, (0.5, 0.5, 0.5), coeff=30.0, diffuse_color=(0.2, 0.4, 0.6))),
             ((4.0, 4.0, 1.2), 0.5, Material(REFLECTIVE, (0.9, 0.9, 0.9), ior=-1.0))]
    for k, (c, r, m) in enumerate(specs):
        p = np.asarray(c)[None, :] + r * uv
        sc.objects.append(Obj(f"ball{k}", p.astype(np.float32), uf.astype(np.uint32), m, uv.astype(np.float32)))
    return sc


def medium_scene(width: int = 512, height: int = 512) -> Scene:
    """The Cornell room plus a dielectric sphere (r=1.0, IOR 1.5) filled with a
    homogeneous medium sigma_s=0.5, sigma_a=0.05 per unit, HG g=0.7."""
    sc = cornell_box(width, height)
    uv, uf = icosphere(4)
    c = np.array([2.78, 3.0, 1.5])
    p = c[None, :] + 1.0 * uv
    mat = Material(VPM, (1.0, 1.0, 1.0), ior=1.5, sigma_s=(0.5, 0.5, 0.5), sigma_a=(0.05, 0.05, 0.05), g=0.7)
    sc.objects.append(Obj("medium", p.astype(np.float32), uf.astype(np.uint32), mat, uv.astype(np.float32)))
    return sc
