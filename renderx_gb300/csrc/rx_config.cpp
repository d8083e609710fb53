// Scene ingest from the reference's own files: the config / scene XML that
// ConfigManager::load reads (reference src/ConfigManager.cpp:25-405) and the OBJ / .shp
// meshes of SimpleShape::loadShape (src/SimpleShape.cpp:44-313), straight into a
// context's geometry and object table. Host C++; no dependency beyond the C library.
//
// Covered: <Config> with <Scene><path/><name/><camera/></Scene>, <Renderer> (<type>,
// <maxDepth>, <spp>, <radius>), <time>, <savePath>; scene files with <Object Name>
// (<filePath>, optional <transform>, a <Material> inline or referenced by <path>/<name>),
// <GroupObject> (one OBJ split into named shapes by its "g" lines, unitized, with the
// group's <transform>; its <Object Name> children pick the shapes) and <Camera Name>;
// materials Diffuse, Glossy, Phong, Refractive, Reflective, Emissive, VPM (<stepsize>).
// Not covered (RX_ERR_UNSUPPORTED): textures, bump maps, GridVolume, ParallelLight.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <array>
#include <atomic>
#include <exception>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rx_internal.h"

namespace {

// ---- a small XML reader: elements, attributes, text (no DTD, no entities beyond the basic five) ----
struct XNode {
  std::string tag, text;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::vector<std::unique_ptr<XNode>> kids;
  const XNode* first(const char* t) const {
    for (auto& k : kids)
      if (k->tag == t) return k.get();
    return nullptr;
  }
  const char* attr(const char* name) const {
    for (auto& a : attrs)
      if (a.first == name) return a.second.c_str();
    return nullptr;
  }
  const char* value(const char* t) const {  // text of the first child <t>, or null
    const XNode* n = first(t);
    return n ? n->text.c_str() : nullptr;
  }
};

struct XParser {
  const char* p;
  const char* end;
  std::string err;
  void skip_ws() {
    while (p < end && (unsigned char)*p <= ' ') p++;
  }
  bool starts(const char* s) const { return (size_t)(end - p) >= strlen(s) && strncmp(p, s, strlen(s)) == 0; }
  void skip_misc() {  // comments, declarations, processing instructions
    for (;;) {
      skip_ws();
      if (starts("<!--")) {
        const char* q = strstr(p, "-->");
        p = q ? q + 3 : end;
      } else if (starts("<?") || starts("<!")) {
        const char* q = strchr(p, '>');
        p = q ? q + 1 : end;
      } else {
        return;
      }
    }
  }
  static std::string unescape(const std::string& s) {
    std::string o;
    for (size_t i = 0; i < s.size(); i++) {
      if (s[i] == '&') {
        static const char* ent[5][2] = {{"&lt;", "<"}, {"&gt;", ">"}, {"&amp;", "&"}, {"&quot;", "\""}, {"&apos;", "'"}};
        bool done = false;
        for (auto& e : ent)
          if (s.compare(i, strlen(e[0]), e[0]) == 0) {
            o += e[1];
            i += strlen(e[0]) - 1;
            done = true;
            break;
          }
        if (!done) o += s[i];
      } else {
        o += s[i];
      }
    }
    return o;
  }
  std::unique_ptr<XNode> element() {
    skip_misc();
    if (p >= end || *p != '<') {
      err = "expected an element";
      return nullptr;
    }
    p++;
    auto n = std::make_unique<XNode>();
    while (p < end && !isspace((unsigned char)*p) && *p != '>' && *p != '/') n->tag += *p++;
    for (;;) {
      skip_ws();
      if (p >= end) {
        err = "unterminated tag <" + n->tag + ">";
        return nullptr;
      }
      if (*p == '/') {  // <tag ... />
        p += 2;
        return n;
      }
      if (*p == '>') {
        p++;
        break;
      }
      std::string name, val;
      while (p < end && *p != '=' && !isspace((unsigned char)*p)) name += *p++;
      skip_ws();
      if (p >= end || *p != '=') {
        err = "bad attribute in <" + n->tag + ">";
        return nullptr;
      }
      p++;
      skip_ws();
      char q = p < end ? *p : 0;
      if (q != '"' && q != '\'') {
        err = "unquoted attribute in <" + n->tag + ">";
        return nullptr;
      }
      p++;
      while (p < end && *p != q) val += *p++;
      p++;
      n->attrs.emplace_back(name, unescape(val));
    }
    for (;;) {
      const char* t0 = p;
      while (p < end && *p != '<') p++;
      n->text += std::string(t0, p);
      if (p >= end) {
        err = "unterminated element <" + n->tag + ">";
        return nullptr;
      }
      if (starts("</")) {
        const char* q = strchr(p, '>');
        p = q ? q + 1 : end;
        break;
      }
      if (starts("<!--") || starts("<?") || starts("<!")) {
        skip_misc();
        continue;
      }
      auto k = element();
      if (!k) return nullptr;
      n->kids.push_back(std::move(k));
    }
    n->text = unescape(n->text);
    size_t a = n->text.find_first_not_of(" \t\r\n"), b = n->text.find_last_not_of(" \t\r\n");
    n->text = a == std::string::npos ? std::string() : n->text.substr(a, b - a + 1);
    return n;
  }
};

// A parsed file: its top-level elements (rapidxml-style documents can hold several).
struct XDoc {
  std::string text;
  std::vector<std::unique_ptr<XNode>> roots;
};

bool read_file(const std::string& path, std::string& out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
  fclose(f);
  return true;
}

// (x, y, z) as readVec (src/xmlHelper.cpp:18-23): the three numbers in parentheses.
bool read_vec(const char* s, float v[3]) {
  if (!s) return false;
  return sscanf(s, " (%f , %f , %f )", &v[0], &v[1], &v[2]) == 3 || sscanf(s, "%f %f %f", &v[0], &v[1], &v[2]) == 3;
}

struct Loader {
  std::string root;  // folder of the config file
  std::unordered_map<std::string, std::unique_ptr<XDoc>> docs;
  std::string err;

  std::string resolve(const std::string& p) const {
    FILE* f = fopen(p.c_str(), "rb");
    if (f) {
      fclose(f);
      return p;
    }
    return root + "/" + p;
  }
  XDoc* doc(const std::string& path) {
    std::string full = resolve(path);
    auto it = docs.find(full);
    if (it != docs.end()) return it->second.get();
    auto d = std::make_unique<XDoc>();
    if (!read_file(full, d->text)) {
      err = "cannot read " + full;
      return nullptr;
    }
    XParser ps{d->text.data(), d->text.data() + d->text.size(), {}};
    for (;;) {
      ps.skip_misc();
      if (ps.p >= ps.end) break;
      auto n = ps.element();
      if (!n) {
        err = full + ": " + ps.err;
        return nullptr;
      }
      d->roots.push_back(std::move(n));
    }
    XDoc* r = d.get();
    docs[full] = std::move(d);
    return r;
  }
  // ConfigManager::findNode: the first <tag> whose Name matches (or any, if unnamed).
  static const XNode* find(const std::vector<std::unique_ptr<XNode>>& v, const char* tag, const std::string& name) {
    for (auto& n : v)
      if (n->tag == tag) {
        const char* a = n->attr("Name");
        if (!a || name.empty() || name == a) return n.get();
      }
    return nullptr;
  }
};

// World-space transform from <transform> as readMatrix (src/xmlHelper.cpp:4-16): four
// bracketed rows; the vertex transform is that matrix applied to (x, y, z, 1).
bool read_matrix(const char* s, float m[4][4]) {
  float v[16];
  if (!s || sscanf(s, " [%f , %f , %f , %f ] [%f , %f , %f , %f ] [%f , %f , %f , %f ] [%f , %f , %f , %f ]", v, v + 1,
                   v + 2, v + 3, v + 4, v + 5, v + 6, v + 7, v + 8, v + 9, v + 10, v + 11, v + 12, v + 13, v + 14,
                   v + 15) != 16)
    return false;
  for (int r = 0; r < 4; r++)
    for (int k = 0; k < 4; k++) m[r][k] = v[4 * r + k];
  return true;
}

struct Mesh {
  std::vector<float> v, n;         // positions, normals (per vertex after re-indexing)
  std::vector<uint32_t> f;         // triangles
};

// Indexed mesh from parsed OBJ data: corners whose normal index differs from an
// earlier corner's at the same position get their own vertex.
bool finish_mesh(const std::vector<float>& pos, const std::vector<float>& nrm, const std::vector<int>& corner_v,
                 const std::vector<int>& corner_n, const std::string& path, Mesh& m, std::string& err) {
  const int nv = (int)pos.size() / 3, nn = (int)nrm.size() / 3;
  bool has_n = nn > 0;
  for (size_t i = 0; i < corner_v.size() && has_n; i++) has_n = corner_n[i] >= 0 && corner_n[i] < nn;
  m.v = pos;
  if (has_n) m.n.assign(pos.size(), 0.0f);
  std::vector<int> vnorm(nv, -1);
  std::unordered_map<uint64_t, uint32_t> split;
  for (size_t i = 0; i < corner_v.size(); i++) {
    int a = corner_v[i];
    if (a < 0 || a >= nv) return err = "face index out of range in " + path, false;
    uint32_t idx = (uint32_t)a;
    if (has_n) {
      int b = corner_n[i];
      if (vnorm[a] < 0 || vnorm[a] == b) {
        vnorm[a] = b;
        for (int q = 0; q < 3; q++) m.n[3 * a + q] = nrm[3 * b + q];
      } else {  // the same position with another normal: its own vertex
        uint64_t key = ((uint64_t)a << 32) | (uint32_t)b;
        auto it = split.find(key);
        if (it == split.end()) {
          idx = (uint32_t)(m.v.size() / 3);
          for (int q = 0; q < 3; q++) m.v.push_back(pos[3 * a + q]), m.n.push_back(nrm[3 * b + q]);
          split[key] = idx;
        } else {
          idx = it->second;
        }
      }
    }
    m.f.push_back(idx);
  }
  return true;
}

// SimpleShape::loadShape for .obj (v / vn / f with v, v//n, v/t/n, quads split (0,1,2),
// (0,2,3); normals normalised on load) and .shp (int count, floats, int count, uints).
// Corners whose normal index differs from the vertex index get their own vertex.
bool load_mesh(const std::string& path, Mesh& m, std::string& err) {
  if (path.size() >= 4 && path.compare(path.size() - 4, 4, ".shp") == 0) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return err = "cannot read " + path, false;
    int nv = 0, nf = 0;
    bool ok = fread(&nv, 4, 1, f) == 1 && nv >= 0;
    if (ok) m.v.resize(nv), ok = fread(m.v.data(), 4, nv, f) == (size_t)nv;
    if (ok) ok = fread(&nf, 4, 1, f) == 1 && nf >= 0;
    if (ok) m.f.resize(nf), ok = fread(m.f.data(), 4, nf, f) == (size_t)nf;
    fclose(f);
    if (!ok || nv % 3 || nf % 3) return err = "malformed " + path, false;
    return true;
  }
  std::string text;
  if (!read_file(path, text)) return err = "cannot read " + path, false;
  std::vector<float> pos, nrm;
  std::vector<int> corner_v, corner_n;
  pos.reserve(text.size() / 12);
  corner_v.reserve(text.size() / 8);
  corner_n.reserve(text.size() / 8);
  const char* p = text.c_str();
  const char* const end = p + text.size();
  auto space = [](char ch) { return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\v' || ch == '\f'; };
  while (p < end) {
    const char* eol = static_cast<const char*>(memchr(p, '\n', (size_t)(end - p)));
    if (!eol) eol = end;
    // the line's first token (the tag), as sscanf's %s
    const char* t = p;
    while (t < eol && space(*t)) t++;
    const char* te = t;
    while (te < eol && !space(*te)) te++;
    const size_t tl = (size_t)(te - t);
    const char* rest = te;
    p = eol + 1;
    if (tl == 0 || *t == '#') continue;
    // numbers as strtof / strtol read them (what sscanf's %f / %d convert with); the
    // text is NUL-terminated, so a number never reads past the buffer, and one that
    // runs into the next line means the line held too few
    if ((tl == 1 && t[0] == 'v') || (tl == 2 && t[0] == 'v' && t[1] == 'n')) {
      float x[3];
      int k = 0;
      for (; k < 3; k++) {
        char* ne;
        x[k] = strtof(rest, &ne);
        if (ne == rest || ne > eol) break;
        rest = ne;
      }
      if (k != 3) continue;
      if (tl == 2) {
        float l = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        if (l > 0) x[0] /= l, x[1] /= l, x[2] /= l;
        nrm.insert(nrm.end(), {x[0], x[1], x[2]});
      } else {
        pos.insert(pos.end(), {x[0], x[1], x[2]});
      }
    } else if (tl == 1 && t[0] == 'f') {
      // corners "a", "a/b", "a/b/c", "a//c": a/b/c and a//c carry a normal, the rest
      // only a position (the sscanf forms %d/%d/%d, %d//%d, %d tried in that order)
      int vi[4], ni[4], k = 0;
      while (k < 4) {
        while (rest < eol && space(*rest)) rest++;
        if (rest >= eol) break;
        const char* tok_end = rest;
        while (tok_end < eol && !space(*tok_end)) tok_end++;
        char* ne;
        long a = strtol(rest, &ne, 10);
        if (ne == rest || ne > tok_end) break;
        const char* q = ne;
        long c = 0;
        bool has_c = false;
        if (q + 1 < tok_end && q[0] == '/' && q[1] == '/') {
          c = strtol(q + 2, &ne, 10);
          has_c = ne != q + 2 && ne <= tok_end && !space(q[2]);
        } else if (q < tok_end && q[0] == '/') {
          strtol(q + 1, &ne, 10);
          if (ne != q + 1 && ne < tok_end && !space(q[1]) && ne[0] == '/') {
            const char* r = ne + 1;
            c = strtol(r, &ne, 10);
            has_c = ne != r && ne <= tok_end && !space(*r);
          }
        }
        vi[k] = (int)a - 1;
        ni[k] = has_c ? (int)c - 1 : -1;
        k++;
        rest = tok_end;
      }
      if (k < 3) continue;
      int tri[2][3] = {{0, 1, 2}, {0, 2, 3}};
      for (int f = 0; f < (k == 4 ? 2 : 1); f++)
        for (int q = 0; q < 3; q++) {
          corner_v.push_back(vi[tri[f][q]]);
          corner_n.push_back(ni[tri[f][q]]);
        }
    }
  }
  return finish_mesh(pos, nrm, corner_v, corner_n, path, m, err);
}

// SimpleShape::loadShape(path, true, &shapes) for a <GroupObject> (src/SimpleShape.cpp:
// 44-313): every "g name" line starts a shape that takes the vertices, normals and
// triangles that follow it (indices relative to where it starts; quads stay with the
// file only, as there); then every shape is unitized by the whole file's bounding box
// (centre to the origin, largest extent to 2: SimpleShape::unitize, applied as the
// transposed matrix it returns). Shapes by name.
bool load_group(const std::string& path, std::unordered_map<std::string, Mesh>& out, std::string& err) {
  std::string text;
  if (!read_file(path, text)) return err = "cannot read " + path, false;
  struct Part {
    std::string name;
    std::vector<float> pos, nrm;
    std::vector<int> cv, cn;
  };
  std::vector<Part> parts;
  std::vector<float> all;  // every vertex of the file (the unitize box)
  int v_base = 0, n_base = 0, nv_all = 0, nn_all = 0;
  const char* p = text.c_str();
  while (*p) {
    const char* eol = strchr(p, '\n');
    std::string line(p, eol ? eol : p + strlen(p));
    p = eol ? eol + 1 : p + strlen(p);
    char tag[8] = {0};
    int off = 0;
    if (sscanf(line.c_str(), "%7s%n", tag, &off) != 1 || tag[0] == '#') continue;
    const char* rest = line.c_str() + off;
    if (!strcmp(tag, "g")) {
      char name[256] = {0};
      sscanf(rest, "%255s", name);
      parts.push_back(Part{name, {}, {}, {}, {}});
      v_base = nv_all;
      n_base = nn_all;
    } else if (!strcmp(tag, "v") || !strcmp(tag, "vn")) {
      float x, y, z;
      if (sscanf(rest, "%f %f %f", &x, &y, &z) != 3) continue;
      if (tag[1] == 'n') {
        float l = std::sqrt(x * x + y * y + z * z);
        if (l > 0) x /= l, y /= l, z /= l;
        nn_all++;
        if (!parts.empty()) parts.back().nrm.insert(parts.back().nrm.end(), {x, y, z});
      } else {
        nv_all++;
        all.insert(all.end(), {x, y, z});
        if (!parts.empty()) parts.back().pos.insert(parts.back().pos.end(), {x, y, z});
      }
    } else if (!strcmp(tag, "f") && !parts.empty()) {
      int vi[4], ni[4], k = 0;
      char tok[64];
      int used = 0;
      while (k < 4 && sscanf(rest, "%63s%n", tok, &used) == 1) {
        rest += used;
        int a = 0, b = 0, c = 0;
        ni[k] = -1;
        if (sscanf(tok, "%d/%d/%d", &a, &b, &c) == 3) vi[k] = a - 1, ni[k] = c - 1;
        else if (sscanf(tok, "%d//%d", &a, &c) == 2) vi[k] = a - 1, ni[k] = c - 1;
        else if (sscanf(tok, "%d", &a) == 1) vi[k] = a - 1;
        else break;
        k++;
      }
      if (k != 3) continue;  // quads are not split into the shapes (loadShape: "not dealt with")
      for (int q = 0; q < 3; q++) {
        parts.back().cv.push_back(vi[q] - v_base);
        parts.back().cn.push_back(ni[q] < 0 ? -1 : ni[q] - n_base);
      }
    }
  }
  if (all.empty()) return err = "no vertices in " + path, false;
  float lo[3] = {all[0], all[1], all[2]}, hi[3] = {all[0], all[1], all[2]};
  for (size_t i = 0; i < all.size(); i += 3)
    for (int q = 0; q < 3; q++) lo[q] = std::min(lo[q], all[i + q]), hi[q] = std::max(hi[q], all[i + q]);
  float len = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
  const float sc = 2 / len, neg = -2 / len;
  float tr[3];
  for (int q = 0; q < 3; q++) tr[q] = neg * ((lo[q] + hi[q]) / 2);
  for (Part& part : parts) {
    for (size_t i = 0; i < part.pos.size(); i += 3)
      for (int q = 0; q < 3; q++) part.pos[i + q] = sc * part.pos[i + q] + tr[q];
    Mesh m;
    if (!finish_mesh(part.pos, part.nrm, part.cv, part.cn, path, m, err)) return false;
    out[part.name] = std::move(m);
  }
  return true;
}

bool material(const XNode* nm, rx_object& o, std::string& err) {
  const char* type = nm->value("type");
  if (!type) return err = "material without <type>", false;
  std::string t = type;
  auto vec = [&](const XNode* n, const char* tag, float* dst) {
    const char* s = n ? n->value(tag) : nullptr;
    if (s) read_vec(s, dst);
  };
  auto num = [&](const XNode* n, const char* tag, float& dst) {
    const char* s = n ? n->value(tag) : nullptr;
    if (s) dst = (float)atof(s);
  };
  if (nm->first("Texture") || nm->first("ColorTexture") || nm->first("CoeffTexture") || nm->first("BumpTexture"))
    return err = "textured materials are not supported", false;
  for (int k = 0; k < 3; k++) o.color[k] = o.diffuse_color[k] = o.decay[k] = 1.0f;
  o.coeff = 1.0f;
  o.ior = 1.5f;
  if (t == "Diffuse") {
    o.material = RX_MAT_DIFFUSE;
    vec(nm, "color", o.color);
  } else if (t == "Glossy") {
    o.material = RX_MAT_GLOSSY;
    vec(nm, "color", o.color);
    num(nm, "coeff", o.coeff);
  } else if (t == "Phong") {
    o.material = RX_MAT_PHONG;
    vec(nm->first("GlossyComponent"), "color", o.color);
    num(nm->first("GlossyComponent"), "coeff", o.coeff);
    vec(nm->first("DiffuseComponent"), "color", o.diffuse_color);
  } else if (t == "Refractive") {
    o.material = RX_MAT_REFRACTIVE;
    num(nm, "coeff", o.ior);
    vec(nm, "surfColor", o.color);
    vec(nm, "decayColor", o.decay);
  } else if (t == "Reflective") {
    o.material = RX_MAT_REFLECTIVE;
    o.ior = -1.0f;
    vec(nm, "color", o.color);
  } else if (t == "Emissive") {
    o.material = RX_MAT_EMISSIVE;
    vec(nm, "color", o.color);
  } else if (t == "VPM") {
    o.material = RX_MAT_VPM;
    if (!nm->first("sigma_s") || !nm->first("sigma_a") || !nm->first("inrate") || !nm->first("g"))
      return err = "VPM material needs sigma_s, sigma_a, inrate and g", false;
    vec(nm, "sigma_s", o.sigma_s);
    vec(nm, "sigma_a", o.sigma_a);
    num(nm, "inrate", o.ior);
    num(nm, "g", o.g);
    if (nm->first("stepsize")) num(nm, "stepsize", o.step_size);  // ConfigManager.cpp:69-70
  } else {
    return err = "material type " + t + " is not supported", false;
  }
  return true;
}

}  // namespace

struct rx_host_scene {
  std::vector<float> verts, norms;
  std::vector<uint32_t> tris, tri_obj, tri_local;
  std::vector<rx_object> objs;
  bool any_normals = false;
};

namespace {
void set_err(char* dst, size_t len, const char* m) {
  if (dst && len) snprintf(dst, len, "%s", m);
}
void set_err(char* dst, size_t len, const std::string& m) { set_err(dst, len, m.c_str()); }

rx_status read_config(const char* config_path, rx_host_scene& H, rx_config_info& in, std::string& err) {
  Loader L;
  L.root = ".";
  std::string cp = config_path;
  size_t sl = cp.find_last_of('/');
  L.root = sl == std::string::npos ? "." : cp.substr(0, sl);
  XDoc* cd = L.doc(cp);
  if (!cd) return err = L.err, RX_ERR_INVALID;
  const XNode* cfg = Loader::find(cd->roots, "Config", "");
  if (!cfg) return err = "no <Config> in " + cp, RX_ERR_INVALID;
  const XNode* sc = cfg->first("Scene");
  if (!sc || !sc->value("camera")) return err = "<Config> needs <Scene> with <camera>", RX_ERR_INVALID;
  std::string scene_path = sc->value("path") ? sc->value("path") : "";
  std::string scene_name = sc->value("name") ? sc->value("name") : "";
  const XNode* scene = nullptr;
  if (!scene_path.empty()) {
    XDoc* sd = L.doc(scene_path);
    if (!sd) return err = L.err, RX_ERR_INVALID;
    scene = Loader::find(sd->roots, "Scene", scene_name);
  }
  if (!scene) scene = Loader::find(cd->roots, "Scene", scene_name);
  if (!scene) return err = "scene not found", RX_ERR_INVALID;
  // one scene object: material from <Material> (a <path>/<name> reference into another
  // file or this scene, else inline), mesh, optional transform (ConfigManager.cpp:166-246)
  auto resolve = [&](const XNode* k, rx_object& o) -> rx_status {
    const XNode* mref = k->first("Material");
    if (!mref) return err = "object without <Material>", RX_ERR_INVALID;
    const XNode* nm = nullptr;
    std::string mpath = mref->value("path") ? mref->value("path") : scene_path;
    std::string mname = mref->value("name") ? mref->value("name") : "";
    if (mref->first("name") || mref->first("path")) {
      XDoc* md = mpath.empty() ? nullptr : L.doc(mpath);
      if (md) nm = Loader::find(md->roots, "Material", mname);
      if (!nm && mref->first("name")) nm = Loader::find(scene->kids, "Material", mname);
    }
    if (!nm) nm = mref;
    o = rx_object{};
    return material(nm, o, err) ? RX_OK : RX_ERR_UNSUPPORTED;
  };
  auto add_object = [&](rx_object o, const Mesh& m, const char* xform) -> rx_status {
    float M[4][4];
    bool xf = xform != nullptr;
    if (xf && !read_matrix(xform, M)) return err = "bad <transform>", RX_ERR_INVALID;
    uint32_t base = (uint32_t)(H.verts.size() / 3);
    for (size_t i = 0; i < m.v.size(); i += 3) {
      float x = m.v[i], y = m.v[i + 1], z = m.v[i + 2];
      if (xf) {  // matrix x (x, y, z, 1), row by row
        float w[3];
        for (int r = 0; r < 3; r++) w[r] = M[r][0] * x + M[r][1] * y + M[r][2] * z + M[r][3];
        x = w[0], y = w[1], z = w[2];
      }
      H.verts.insert(H.verts.end(), {x, y, z});
    }
    bool has_n = !m.n.empty();
    H.any_normals |= has_n;
    for (size_t i = 0; i < m.v.size(); i += 3) {
      float nx = has_n ? m.n[i] : 0.0f, ny = has_n ? m.n[i + 1] : 0.0f, nz = has_n ? m.n[i + 2] : 0.0f;
      if (has_n && xf) {  // inverse transpose of the linear part (cofactor matrix, normalised)
        float a = M[0][0], b = M[0][1], cc = M[0][2], d = M[1][0], e = M[1][1], f = M[1][2], g = M[2][0],
              h = M[2][1], ii = M[2][2];
        float A = e * ii - f * h, B = -(d * ii - f * g), C = d * h - e * g;
        float D = -(b * ii - cc * h), E = a * ii - cc * g, F = -(a * h - b * g);
        float G = b * f - cc * e, Hh = -(a * f - cc * d), I = a * e - b * d;
        float tx = A * nx + B * ny + C * nz, ty = D * nx + E * ny + F * nz, tz = G * nx + Hh * ny + I * nz;
        float l = std::sqrt(tx * tx + ty * ty + tz * tz);
        if (l > 0) nx = tx / l, ny = ty / l, nz = tz / l;
      }
      H.norms.insert(H.norms.end(), {nx, ny, nz});
    }
    o.tri_begin = (uint32_t)(H.tris.size() / 3);
    o.tri_count = (uint32_t)(m.f.size() / 3);
    o.has_vertex_normals = has_n ? 1u : 0u;
    for (size_t i = 0; i < m.f.size(); i++) H.tris.push_back(base + m.f[i]);
    for (uint32_t t = 0; t < o.tri_count; t++) {
      H.tri_obj.push_back((uint32_t)H.objs.size());
      H.tri_local.push_back(t);
    }
    H.objs.push_back(o);
    return RX_OK;
  };
  // <GroupObject>s first (ConfigManager.cpp:193-224): one OBJ split into named shapes, each
  // <Object Name=...> inside taking its shape with the group's transform
  for (auto& g : scene->kids) {
    if (g->tag != "GroupObject") continue;
    const char* fp = g->value("filePath");
    if (!fp) return err = "<GroupObject> without <filePath>", RX_ERR_INVALID;
    std::unordered_map<std::string, Mesh> shapes;
    if (!load_group(L.resolve(fp), shapes, err)) return RX_ERR_INVALID;
    const char* xform = g->first("transform") ? g->value("transform") : nullptr;
    for (auto& k : g->kids) {
      if (k->tag != "Object") continue;
      rx_object o;
      rx_status st = resolve(k.get(), o);
      if (st != RX_OK) return st;
      const char* nm = k->attr("Name");
      auto it = nm ? shapes.find(nm) : shapes.end();
      if (it == shapes.end()) return err = std::string("group shape ") + (nm ? nm : "?") + " not in " + fp, RX_ERR_INVALID;
      if ((st = add_object(o, it->second, xform)) != RX_OK) return st;
    }
  }
  // the <Object> meshes are read by a pool of threads, then added in document order
  // (errors as a sequential reader meets them: an object's material before its mesh)
  std::vector<const XNode*> objs;
  for (auto& k : scene->kids)
    if (k->tag == "Object") objs.push_back(k.get());
  std::vector<Mesh> meshes(objs.size());
  std::vector<std::string> mesh_err(objs.size());
  std::vector<char> mesh_ok(objs.size(), 0);
  // a worker that meets an exception records it here without allocating (no exception
  // leaves a worker thread); the message is built on the calling thread afterwards
  enum : char { kNoExc = 0, kOutOfMemory = 1, kOtherExc = 2 };
  std::vector<char> mesh_exc(objs.size(), kNoExc);
  std::vector<std::array<char, 160>> mesh_what(objs.size());
  {
    std::atomic<size_t> next{0};
    auto work = [&]() noexcept {
      for (size_t i; (i = next.fetch_add(1)) < objs.size();) {
        const char* fp = objs[i]->value("filePath");
        try {
          if (fp) mesh_ok[i] = load_mesh(L.resolve(fp), meshes[i], mesh_err[i]);
        } catch (const std::bad_alloc&) {
          mesh_ok[i] = 0;
          mesh_exc[i] = kOutOfMemory;
        } catch (const std::exception& ex) {
          mesh_ok[i] = 0;
          mesh_exc[i] = kOtherExc;
          std::strncpy(mesh_what[i].data(), ex.what(), mesh_what[i].size() - 1);
          mesh_what[i].back() = 0;
        } catch (...) {
          mesh_ok[i] = 0;
          mesh_exc[i] = kOtherExc;
          std::strncpy(mesh_what[i].data(), "unknown exception", mesh_what[i].size() - 1);
          mesh_what[i].back() = 0;
        }
      }
    };
    const size_t nt = std::min<size_t>(objs.size(), std::max(1u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nt; t++) {
      try {
        pool.emplace_back(work);
      } catch (const std::exception&) {
        break;  // fewer threads: the calling thread reads the rest
      }
    }
    work();
    for (auto& th : pool) th.join();
  }
  for (size_t i = 0; i < objs.size(); i++) {
    const XNode* k = objs[i];
    rx_object o;
    rx_status st = resolve(k, o);
    if (st != RX_OK) return st;
    if (!k->value("filePath")) return err = "object without <filePath>", RX_ERR_INVALID;
    if (mesh_exc[i] == kOutOfMemory) return err = "out of host memory reading " + std::string(k->value("filePath")), RX_ERR_OOM;
    if (mesh_exc[i] == kOtherExc)
      return err = "error reading " + std::string(k->value("filePath")) + ": " + mesh_what[i].data(), RX_ERR_INVALID;
    if (!mesh_ok[i]) return err = mesh_err[i], RX_ERR_INVALID;
    if ((st = add_object(o, meshes[i], k->first("transform") ? k->value("transform") : nullptr)) != RX_OK) return st;
    meshes[i] = Mesh();  // release as we go
  }
  if (H.objs.empty()) return err = "scene has no objects", RX_ERR_INVALID;
  const XNode* cam = Loader::find(scene->kids, "Camera", sc->value("camera"));
  if (!cam) return err = "camera not found", RX_ERR_INVALID;
  in = rx_config_info{};
  in.camera.width = (uint32_t)atoi(cam->value("width") ? cam->value("width") : "0");
  in.camera.height = (uint32_t)atoi(cam->value("height") ? cam->value("height") : "0");
  in.camera.sight_dist = (uint32_t)atoi(cam->value("sightDist") ? cam->value("sightDist") : "0");
  if (!read_vec(cam->value("focus"), in.camera.focus) || !read_vec(cam->value("position"), in.camera.position) ||
      !read_vec(cam->value("up"), in.camera.up))
    return err = "camera needs focus, position and up", RX_ERR_INVALID;
  // renderer (ConfigManager.cpp:277-388: a <Renderer> block wins over the older flat tags)
  in.estimator = -1;
  in.max_depth = 20;  // MCRenderer's default
  const XNode* rn = cfg->first("Renderer");
  std::string type = rn && rn->value("type") ? rn->value("type") : (cfg->value("renderer") ? cfg->value("renderer") : "");
  snprintf(in.renderer, sizeof in.renderer, "%s", type.c_str());
  if (type == "PathTracer" || type == "PT") in.estimator = 0;
  if (type == "PTtest") in.estimator = 1;
  if (type == "VCMTracer" || type == "VCM") in.estimator = 2;
  if (type == "BidirectionalPathTracer" || type == "BPT") in.estimator = 3;
  if (type == "PhotonMap" || type == "PM") in.estimator = 4;
  const char* md = rn ? rn->value("maxDepth") : cfg->value("maxDepth");
  if (md) in.max_depth = (uint32_t)atoi(md);
  const char* spp = rn ? rn->value("spp") : nullptr;
  if (spp) in.spp = (uint32_t)atoi(spp);
  const char* rad = rn ? rn->value("radius") : cfg->value("radius");
  if (rad) in.radius = (float)atof(rad);
  if (const XNode* tn = cfg->first("time")) {
    double rt = 0;
    if (tn->value("hours")) rt += 3600.0 * atoi(tn->value("hours"));
    if (tn->value("minutes")) rt += 60.0 * atoi(tn->value("minutes"));
    in.runtime_s = rt;
  }
  if (cfg->value("savePath")) snprintf(in.save_path, sizeof in.save_path, "%s", cfg->value("savePath"));
  in.num_objects = (uint32_t)H.objs.size();
  in.num_triangles = (uint32_t)(H.tris.size() / 3);
  return RX_OK;
}
}  // namespace

extern "C" rx_status rx_config_read(const char* config_path, rx_host_scene** out, rx_config_info* info, char* err,
                                    size_t err_len) {
  if (!config_path || !out) return set_err(err, err_len, "null argument"), RX_ERR_INVALID;
  *out = nullptr;
  std::unique_ptr<rx_host_scene> H;
  rx_config_info in{};
  std::string e;
  rx_status s;
  try {  // no exception crosses the C ABI
    H.reset(new rx_host_scene());
    s = read_config(config_path, *H, in, e);
  } catch (const std::bad_alloc&) {
    set_err(err, err_len, "out of host memory");
    return RX_ERR_OOM;
  } catch (const std::exception& ex) {
    set_err(err, err_len, ex.what());
    return RX_ERR_INVALID;
  }
  if (s != RX_OK) {
    set_err(err, err_len, e);
    return s;
  }
  *out = H.release();
  if (info) *info = in;
  return RX_OK;
}

extern "C" void rx_host_scene_free(rx_host_scene* h) { delete h; }

extern "C" rx_status rx_host_scene_arrays(const rx_host_scene* h, const float** verts, uint32_t* nv,
                                          const uint32_t** tris, uint32_t* nt, const uint32_t** tri_obj,
                                          const uint32_t** tri_local, const float** vnormals, const rx_object** objs,
                                          uint32_t* nobj) {
  if (!h) return RX_ERR_INVALID;
  if (verts) *verts = h->verts.data();
  if (nv) *nv = (uint32_t)(h->verts.size() / 3);
  if (tris) *tris = h->tris.data();
  if (nt) *nt = (uint32_t)(h->tris.size() / 3);
  if (tri_obj) *tri_obj = h->tri_obj.data();
  if (tri_local) *tri_local = h->tri_local.data();
  if (vnormals) *vnormals = h->any_normals ? h->norms.data() : nullptr;
  if (objs) *objs = h->objs.data();
  if (nobj) *nobj = (uint32_t)h->objs.size();
  return RX_OK;
}

extern "C" rx_status rx_scene_load_config(rx_context* c, const char* config_path, rx_config_info* info) {
  if (!c) return RX_ERR_INVALID;
  if (!config_path) return c->fail(RX_ERR_INVALID, "null path");
  rx_host_scene H;
  rx_config_info in{};
  std::string err;
  rx_status s;
  try {  // no exception crosses the C ABI
    s = read_config(config_path, H, in, err);
  } catch (const std::bad_alloc&) {
    return c->fail(RX_ERR_OOM, "out of host memory reading the config");
  } catch (const std::exception& ex) {
    return c->fail(RX_ERR_INVALID, ex.what());
  }
  if (s != RX_OK) return c->fail(s, err);
  s = rx_scene_set_geometry(c, H.verts.data(), (uint32_t)(H.verts.size() / 3), H.tris.data(),
                            (uint32_t)(H.tris.size() / 3), H.tri_obj.data(), H.tri_local.data(),
                            H.any_normals ? H.norms.data() : nullptr);
  if (s != RX_OK) return s;
  if ((s = rx_scene_set_objects(c, H.objs.data(), (uint32_t)H.objs.size())) != RX_OK) return s;
  if (info) *info = in;
  return RX_OK;
}

// MCRenderer::saveImagePFM (reference src/MCRenderer.cpp:556-574): "PF", width height,
// -1 (little endian), float RGB rows from the bottom up.
extern "C" rx_status rx_write_pfm(const char* path, uint32_t width, uint32_t height, const double* rgb) {
  if (!path || !rgb || width == 0 || height == 0) return RX_ERR_INVALID;
  FILE* f = fopen(path, "wb");
  if (!f) return RX_ERR_INVALID;
  fprintf(f, "PF\n%u %u\n-1.000000\n", width, height);
  std::vector<float> row(3 * (size_t)width);
  for (uint32_t j = height; j-- > 0;) {
    for (size_t i = 0; i < 3 * (size_t)width; i++) row[i] = (float)rgb[3 * (size_t)j * width + i];
    fwrite(row.data(), sizeof(float), row.size(), f);
  }
  bool ok = fclose(f) == 0;
  return ok ? RX_OK : RX_ERR_INVALID;
}
