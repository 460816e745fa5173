// loaders.cpp - scene files to the C scene description, on the host.
//
// PBRT: the subset parser of pkg/loaders/pbrt.go (statement accumulation
// over continuation lines, the tokenizer, AttributeBegin/End blocks with the
// graphics-state stack of the current material and area light) and the
// conversion of scene.NewPBRTScene (pkg/scene/pbrt_scene.go): camera, film,
// diffuse / conductor / dielectric materials, sphere / bilinearPatch /
// trianglemesh / box shapes, area lights on shapes inside attribute blocks,
// point / distant / infinite / infinite-gradient lights.  The result is a
// gprt_scene_desc whose arrays the loaded handle owns, so a scene file goes
// straight to gprt_scene_create (and to the device BVH builder).
//
// PLY: the binary little-endian reader of pkg/loaders/ply.go (vertex x, y, z
// and optional normals / colours / texture coordinates, triangular faces),
// returning arrays that feed gprt_mesh_desc directly.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/gprt.h"

struct gprt_loaded {
  std::vector<gprt_material_desc> materials;
  std::vector<gprt_shape_desc> shapes;
  std::vector<gprt_mesh_desc> meshes;
  std::vector<gprt_light_desc> lights;
  std::vector<std::unique_ptr<std::vector<double>>> vertex_arrays;
  std::vector<std::unique_ptr<std::vector<uint32_t>>> index_arrays;
  gprt_scene_desc desc{};
};

struct gprt_ply {
  std::vector<double> vertices, normals, colors, texcoords;
  std::vector<uint32_t> indices;
  gprt_ply_info info{};
};

namespace gprt {
namespace {

// ------------------------------------------------------------ PBRT parsing
struct Param {
  std::string type;
  std::vector<std::string> values;
};

// PBRTStatement (pbrt.go:14-19)
struct Statement {
  std::string type, subtype;
  std::map<std::string, Param> params;
  int material_index = -1;

  bool number(const std::string& s, double& out) const {
    const char* b = s.c_str();
    char* e = nullptr;
    errno = 0;
    out = std::strtod(b, &e);
    return e != b && *e == 0 && errno == 0;
  }
  // GetFloatParam / GetRGBParam / GetPoint3Param / GetStringParam (pbrt.go:649-705)
  bool float_param(const std::string& name, double& v) const {
    auto it = params.find(name);
    return it != params.end() && !it->second.values.empty() && number(it->second.values[0], v);
  }
  bool vec3_param(const std::string& name, double v[3]) const {
    auto it = params.find(name);
    if (it == params.end() || it->second.values.size() < 3) return false;
    for (int k = 0; k < 3; k++)
      if (!number(it->second.values[k], v[k])) return false;
    return true;
  }
  bool area_light() const {  // IsAreaLight (pbrt.go:677-681)
    auto it = params.find("_areaLight");
    return it != params.end() && !it->second.values.empty() && it->second.values[0] == "true";
  }
};

// AttributeBlock (pbrt.go:41-47)
struct Block {
  std::vector<Statement> materials, shapes, lights;
};

// PBRTScene (pbrt.go:22-38); transforms are parsed and ignored, as there
struct Parsed {
  std::unique_ptr<Statement> camera, film;
  bool has_look = false;
  double look[9] = {0};
  std::vector<Statement> materials, shapes, lights;
  std::vector<Block> blocks;  // in completion order
};

// tokenizePBRT (pbrt.go:492-556): quoted strings and bracketed arrays are
// single tokens
std::vector<std::string> tokenize(const std::string& line) {
  std::vector<std::string> out;
  std::string cur;
  bool q = false, br = false;
  for (char c : line) {
    if (c == '"') {
      if (!br) {
        cur += c;
        if (q) {
          out.push_back(cur);
          cur.clear();
          q = false;
        } else {
          q = true;
        }
      } else {
        cur += c;
      }
    } else if (c == '[') {
      if (!q) {
        if (!cur.empty()) {
          out.push_back(cur);
          cur.clear();
        }
        cur += c;
        br = true;
      } else {
        cur += c;
      }
    } else if (c == ']') {
      cur += c;
      if (!q && br) {
        out.push_back(cur);
        cur.clear();
        br = false;
      }
    } else if (c == ' ' || c == '\t') {
      if (q || br) {
        cur += c;
      } else if (!cur.empty()) {
        out.push_back(cur);
        cur.clear();
      }
    } else {
      cur += c;
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

std::vector<std::string> fields(const std::string& s) {
  std::vector<std::string> out;
  std::istringstream in(s);
  std::string w;
  while (in >> w) out.push_back(w);
  return out;
}

bool starts_with(const std::string& s, const std::string& p) { return s.compare(0, p.size(), p) == 0; }
bool ends_with(const std::string& s, const std::string& p) {
  return s.size() >= p.size() && s.compare(s.size() - p.size(), p.size(), p) == 0;
}
std::string trim(const std::string& s, const char* set) {
  size_t a = s.find_first_not_of(set);
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(set);
  return s.substr(a, b - a + 1);
}

// parseStatement (pbrt.go:558-647)
bool parse_statement(const std::string& line, Statement& st, std::string& err) {
  st = Statement();
  for (const char* kw : {"LookAt", "Translate", "Rotate", "Scale", "Transform"}) {
    if (starts_with(line, kw)) {
      st.type = kw;
      st.params["values"] = Param{"float", fields(line.substr(std::strlen(kw)))};
      return true;
    }
  }
  std::vector<std::string> parts = tokenize(line);
  if (parts.size() < 2) {
    err = "invalid statement format";
    return false;
  }
  st.type = parts[0];
  size_t i = 1;
  if (starts_with(parts[1], "\"") && ends_with(parts[1], "\"")) {
    st.subtype = trim(parts[1], "\"");
    i = 2;
  }
  while (i < parts.size()) {
    if (!starts_with(parts[i], "\"")) {
      i++;
      continue;
    }
    std::vector<std::string> def = fields(trim(parts[i], "\""));
    if (def.size() != 2) {
      i++;
      continue;
    }
    i++;
    Param p{def[0], {}};
    if (i < parts.size()) {
      if (starts_with(parts[i], "[") && ends_with(parts[i], "]")) p.values = fields(trim(parts[i], "[] "));
      else p.values = {parts[i]};
      i++;
    }
    st.params[def[1]] = p;
  }
  return true;
}

// isStatementStart (pbrt.go:707-722)
bool statement_start(const std::string& line) {
  for (const char* kw : {"Camera", "Film", "Sampler", "Integrator", "LookAt", "Material", "Shape", "LightSource",
                         "AreaLightSource", "Translate", "Rotate", "Scale", "Transform", "ReverseOrientation",
                         "Attribute"}) {
    std::string k(kw);
    if (line == k || starts_with(line, k + " ")) return true;
  }
  return false;
}

// PBRTParser (pbrt.go:100-271)
struct Parser {
  struct State {
    int material_index;
    const Statement* area_light;  // kept alive in area_lights
  };
  Parsed scene;
  std::vector<std::unique_ptr<Block>> attr;
  std::vector<State> states;
  std::vector<std::unique_ptr<Statement>> area_lights;  // the statements the states point to
  int current_material = -1;
  bool in_world = false;
  std::vector<std::string> lines;

  bool flush(std::string& err) {  // processAccumulatedStatement (pbrt.go:140-154)
    if (lines.empty()) return true;
    std::string full;
    for (size_t k = 0; k < lines.size(); k++) full += (k ? " " : "") + lines[k];
    lines.clear();
    Statement st;
    if (!parse_statement(full, st, err)) {
      err = "error parsing statement '" + full + "': " + err;
      return false;
    }
    return route(st, err);
  }

  // the area light the graphics state holds copies its L / power onto a shape
  void mark_area(Statement& st) {
    if (states.empty() || !states.back().area_light) return;
    st.params["_areaLight"] = Param{"bool", {"true"}};
    for (const auto& kv : states.back().area_light->params)
      if (kv.first == "L" || kv.first == "power") st.params[kv.first] = kv.second;
  }

  // routeStatement (pbrt.go:272-389)
  bool route(Statement& st, std::string& err) {
    if (st.type == "LookAt") {  // parseLookAt (pbrt.go:435-490)
      auto it = st.params.find("values");
      if (st.params.size() != 1 || it == st.params.end() || it->second.values.size() != 9) {
        err = "error parsing LookAt: LookAt requires 9 values";
        return false;
      }
      for (int k = 0; k < 9; k++)
        if (!st.number(it->second.values[k], scene.look[k])) {
          err = "error parsing LookAt: invalid value '" + it->second.values[k] + "'";
          return false;
        }
      scene.has_look = true;
      return true;
    }
    Block* cur = attr.empty() ? nullptr : attr.back().get();
    if (cur) {
      if (st.type == "Material") {
        cur->materials.push_back(st);
      } else if (st.type == "Shape") {
        int local = (int)cur->materials.size() - 1;
        st.material_index = local >= 0 ? local : current_material;
        mark_area(st);
        cur->shapes.push_back(st);
      } else if (st.type == "LightSource") {
        cur->lights.push_back(st);
      } else if (st.type == "AreaLightSource") {
        area_lights.push_back(std::make_unique<Statement>(st));
        if (!states.empty()) states.back().area_light = area_lights.back().get();
        cur->lights.push_back(st);
      }
      return true;
    }
    if (!in_world) {
      if (st.type == "Camera") scene.camera = std::make_unique<Statement>(st);
      else if (st.type == "Film") scene.film = std::make_unique<Statement>(st);
      return true;  // Sampler and Integrator are kept by the reference but not used
    }
    if (st.type == "Material") {
      scene.materials.push_back(st);
      current_material = (int)scene.materials.size() - 1;
    } else if (st.type == "Shape") {
      st.material_index = current_material;
      mark_area(st);
      scene.shapes.push_back(st);
    } else if (st.type == "LightSource") {
      scene.lights.push_back(st);
    } else if (st.type == "AreaLightSource") {
      area_lights.push_back(std::make_unique<Statement>(st));
      if (!states.empty()) states.back().area_light = area_lights.back().get();
      scene.lights.push_back(st);
    }
    return true;
  }

  // processLine (pbrt.go:227-265)
  bool line(std::string l, std::string& err) {
    l = trim(l, " \t\r\n");
    if (l.empty() || l[0] == '#') return true;
    if (l == "WorldBegin" || l == "WorldEnd") {
      if (!flush(err)) return false;
      in_world = l == "WorldBegin";
      return true;
    }
    if (l == "AttributeBegin") {  // processAttributeBegin (pbrt.go:174-203)
      if (!flush(err)) return false;
      State s{current_material, states.empty() ? nullptr : states.back().area_light};
      states.push_back(s);
      attr.push_back(std::make_unique<Block>());
      return true;
    }
    if (l == "AttributeEnd") {  // processAttributeEnd (pbrt.go:205-225)
      if (!flush(err)) return false;
      if (!attr.empty()) {
        scene.blocks.push_back(*attr.back());
        attr.pop_back();
      }
      if (!states.empty()) {
        current_material = states.back().material_index;
        states.pop_back();
      }
      return true;
    }
    if (statement_start(l)) {
      if (!flush(err)) return false;
      lines = {l};
      return true;
    }
    if (lines.empty()) {
      err = "unexpected continuation line: " + l;
      return false;
    }
    lines.push_back(l);
    return true;
  }
};

// ------------------------------------------------------------ conversion
struct Converter {
  gprt_loaded& out;
  std::string& err;

  gprt_material_desc mat_zero() {
    gprt_material_desc m;
    std::memset(&m, 0, sizeof(m));
    return m;
  }

  // convertMaterial (pbrt_scene.go:160-202)
  bool material(const Statement& st, gprt_material_desc& m) {
    m = mat_zero();
    double v[3], f;
    if (st.subtype == "diffuse") {
      m.kind = GPRT_MAT_LAMBERTIAN;
      if (!st.vec3_param("reflectance", v)) v[0] = v[1] = v[2] = 0.7;
      std::memcpy(m.albedo, v, sizeof(v));
    } else if (st.subtype == "conductor") {
      m.kind = GPRT_MAT_METAL;
      if (!st.vec3_param("eta", v)) {
        v[0] = 0.7;
        v[1] = 0.6;
        v[2] = 0.5;
      }
      std::memcpy(m.albedo, v, sizeof(v));
      m.fuzz = 0.0;
      if (st.float_param("roughness", f)) {
        if (f < 0 || f > 1) {
          err = "failed to convert material: invalid metal roughness: must be between 0 and 1";
          return false;
        }
        m.fuzz = f;
      }
    } else if (st.subtype == "dielectric") {
      m.kind = GPRT_MAT_DIELECTRIC;
      m.ior = 1.5;
      if (st.float_param("eta", f)) {
        if (f <= 0) {
          err = "failed to convert material: invalid dielectric IOR: must be positive";
          return false;
        }
        m.ior = f;
      }
    } else {
      err = "failed to convert material: unsupported material type: " + st.subtype;
      return false;
    }
    return true;
  }

  uint32_t add_material(const gprt_material_desc& m) {
    out.materials.push_back(m);
    return (uint32_t)out.materials.size() - 1;
  }

  // convertShape (pbrt_scene.go:204-305); returns the shape's index
  bool shape(const Statement& st, uint32_t mat, int& index) {
    gprt_shape_desc d;
    std::memset(&d, 0, sizeof(d));
    d.material = mat;
    double v[3];
    if (st.subtype == "sphere") {
      double r = 1.0, c[3] = {0, 0, 0};
      double f;
      if (st.float_param("radius", f)) {
        if (f <= 0) {
          err = "invalid sphere radius: must be positive";
          return false;
        }
        r = f;
      }
      st.vec3_param("center", c);
      d.kind = GPRT_SHAPE_SPHERE;
      std::memcpy(d.p, c, sizeof(c));
      d.p[3] = r;
    } else if (st.subtype == "bilinearPatch") {
      double p00[3], p01[3], p10[3], p11[3];
      if (!st.vec3_param("P00", p00) || !st.vec3_param("P01", p01) || !st.vec3_param("P10", p10) ||
          !st.vec3_param("P11", p11)) {
        err = "bilinearPatch missing corner points";
        return false;
      }
      d.kind = GPRT_SHAPE_QUAD;
      for (int k = 0; k < 3; k++) {
        d.p[k] = p00[k];
        d.p[3 + k] = p01[k] - p00[k];
        d.p[6 + k] = p10[k] - p00[k];
      }
    } else if (st.subtype == "trianglemesh") {
      auto P = st.params.find("P");
      if (P == st.params.end() || P->second.values.size() % 3 != 0) {
        err = "trianglemesh missing or invalid vertices";
        return false;
      }
      auto verts = std::make_unique<std::vector<double>>(P->second.values.size());
      for (size_t k = 0; k < verts->size(); k++)
        if (!st.number(P->second.values[k], (*verts)[k])) {
          err = "invalid vertex coordinate '" + P->second.values[k] + "'";
          return false;
        }
      auto I = st.params.find("indices");
      if (I == st.params.end() || I->second.values.size() % 3 != 0) {
        err = "trianglemesh missing or invalid indices";
        return false;
      }
      auto idx = std::make_unique<std::vector<uint32_t>>(I->second.values.size());
      size_t nv = verts->size() / 3;
      for (size_t k = 0; k < idx->size(); k++) {
        long x = std::strtol(I->second.values[k].c_str(), nullptr, 10);  // strconv.Atoi, errors ignored as there
        if (x < 0 || (size_t)x >= nv) {
          err = "trianglemesh index out of range";  // NewTriangleMesh panics (triangle_mesh.go:73-76)
          return false;
        }
        (*idx)[k] = (uint32_t)x;
      }
      gprt_mesh_desc md;
      std::memset(&md, 0, sizeof(md));
      md.vertices = verts->data();
      md.indices = idx->data();
      md.n_vertices = (uint32_t)nv;
      md.n_triangles = (uint32_t)(idx->size() / 3);
      out.vertex_arrays.push_back(std::move(verts));
      out.index_arrays.push_back(std::move(idx));
      d.kind = GPRT_SHAPE_MESH;
      d.mesh = (uint32_t)out.meshes.size();
      out.meshes.push_back(md);
    } else if (st.subtype == "box") {
      double c[3] = {0, 0, 0}, s[3] = {1, 1, 1}, r[3] = {0, 0, 0};
      st.vec3_param("center", c);
      st.vec3_param("size", s);
      st.vec3_param("rotation", r);
      d.kind = GPRT_SHAPE_BOX;
      std::memcpy(d.p, c, sizeof(c));
      std::memcpy(d.p + 3, s, sizeof(s));
      std::memcpy(d.p + 6, r, sizeof(r));
    } else {
      err = "unsupported shape type: " + st.subtype;
      return false;
    }
    (void)v;
    out.shapes.push_back(d);
    index = (int)out.shapes.size() - 1;
    return true;
  }

  gprt_light_desc light_zero() {
    gprt_light_desc l;
    std::memset(&l, 0, sizeof(l));
    l.weight = 1.0;
    return l;
  }

  // convertLight (pbrt_scene.go:338-395)
  bool light(const Statement& st) {
    gprt_light_desc l = light_zero();
    double v[3];
    if (st.subtype == "point") {  // a 0.1-radius sphere light that is not a scene shape
      l.kind = GPRT_LIGHT_SPHERE;
      l.shape = GPRT_NO_SHAPE;
      double I[3] = {10, 10, 10}, from[3] = {0, 5, 0};
      st.vec3_param("I", I);
      st.vec3_param("from", from);
      std::memcpy(l.color_a, I, sizeof(I));
      std::memcpy(l.from, from, sizeof(from));
      l.radius = 0.1;
    } else if (st.subtype == "distant" || st.subtype == "infinite") {
      l.kind = GPRT_LIGHT_UNIFORM_INFINITE;
      double d = st.subtype == "distant" ? 3.0 : 1.0;
      if (!st.vec3_param("L", v)) v[0] = v[1] = v[2] = d;
      std::memcpy(l.color_a, v, sizeof(v));
    } else if (st.subtype == "infinite-gradient") {
      l.kind = GPRT_LIGHT_GRADIENT_INFINITE;
      double top[3] = {0.5, 0.7, 1.0}, bottom[3] = {1.0, 1.0, 1.0};
      st.vec3_param("topColor", top);
      st.vec3_param("bottomColor", bottom);
      std::memcpy(l.color_a, top, sizeof(top));
      std::memcpy(l.color_b, bottom, sizeof(bottom));
    } else if (st.subtype == "diffuse") {
      err = "failed to convert light: AreaLightSource should be handled as graphics state, not converted as "
            "standalone light";
      return false;
    } else {
      err = "failed to convert light: unsupported light type: " + st.subtype;
      return false;
    }
    out.lights.push_back(l);
    return true;
  }

  // convertAreaLight (pbrt_scene.go:307-336): a quad or sphere light on the
  // shape just converted
  bool area_light(const Statement& st, int shape_index) {
    double L[3];
    if (!st.vec3_param("L", L)) {
      err = "failed to convert area light: area light missing emission parameter 'L'";
      return false;
    }
    const gprt_shape_desc& d = out.shapes[shape_index];
    gprt_light_desc l = light_zero();
    if (d.kind == GPRT_SHAPE_QUAD) l.kind = GPRT_LIGHT_QUAD;
    else if (d.kind == GPRT_SHAPE_SPHERE) l.kind = GPRT_LIGHT_SPHERE;
    else {
      err = "failed to convert area light: shape type is not supported as an area light";
      return false;
    }
    l.shape = (uint32_t)shape_index;
    out.lights.push_back(l);
    return true;
  }

  // NewPBRTScene (pbrt_scene.go:15-78)
  bool convert(const Parsed& ps, const gprt_camera_desc* override) {
    // createDefaultPBRTSamplingConfig (:80-91) and convertCamera (:93-158)
    gprt_sampling_desc& sm = out.desc.sampling;
    sm.width = 400;
    sm.height = 400;
    sm.samples_per_pixel = 150;
    sm.max_depth = 5;
    sm.rr_min_bounces = 16;
    sm.adaptive_min_samples = 0.20;
    sm.adaptive_threshold = 0.005;
    gprt_camera_desc& c = out.desc.camera;
    double center[3] = {0, 0, 0}, look[3] = {0, 0, -1}, up[3] = {0, 1, 0};
    double width = 400, aspect = 1.0, vfov = 90.0, aperture = 0.0, focus = 1.0;
    if (ps.has_look) {
      std::memcpy(center, ps.look, sizeof(center));
      std::memcpy(look, ps.look + 3, sizeof(look));
      std::memcpy(up, ps.look + 6, sizeof(up));
    }
    double f;
    if (ps.camera && ps.camera->subtype == "perspective" && ps.camera->float_param("fov", f)) {
      if (f <= 0 || f >= 180) {
        err = "failed to convert camera: invalid camera FOV: must be between 0 and 180 degrees";
        return false;
      }
      vfov = f;
    }
    if (ps.film) {
      if (ps.film->float_param("xresolution", f)) {
        if (f <= 0 || f > 8192) {
          err = "failed to convert camera: invalid image width: must be between 1 and 8192";
          return false;
        }
        width = (double)(int)f;
        sm.width = (uint32_t)(int)f;
      }
      if (ps.film->float_param("yresolution", f)) {
        if (f <= 0 || f > 8192) {
          err = "failed to convert camera: invalid image height: must be between 1 and 8192";
          return false;
        }
        sm.height = (uint32_t)(int)f;
        aspect = width / f;
      }
    }
    if (override) {  // MergeCameraConfig (camera.go:320-349): non-zero fields win
      auto nz = [](const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) != 0; };
      if (override->width) width = override->width;
      if (override->aspect_ratio != 0) aspect = override->aspect_ratio;
      if (nz(override->center)) std::memcpy(center, override->center, sizeof(center));
      if (nz(override->look_at)) std::memcpy(look, override->look_at, sizeof(look));
      if (nz(override->up)) std::memcpy(up, override->up, sizeof(up));
      if (override->vfov_deg != 0) vfov = override->vfov_deg;
      if (override->aperture != 0) aperture = override->aperture;
      if (override->focus_distance != 0) focus = override->focus_distance;
      if (override->width > 0) {
        sm.width = override->width;
        sm.height = (uint32_t)(int)((double)override->width / aspect);
      }
    }
    std::memcpy(c.center, center, sizeof(center));
    std::memcpy(c.look_at, look, sizeof(look));
    std::memcpy(c.up, up, sizeof(up));
    c.width = (uint32_t)width;
    c.aspect_ratio = aspect;
    c.vfov_deg = vfov;
    c.aperture = aperture;
    c.focus_distance = focus;
    // top-level materials, shapes (never area lights here) and lights
    std::vector<uint32_t> global;
    for (const Statement& m : ps.materials) {
      gprt_material_desc md;
      if (!material(m, md)) return false;
      global.push_back(add_material(md));
    }
    for (const Statement& s : ps.shapes) {
      if (s.material_index < 0 || s.material_index >= (int)global.size()) {
        err = "shape has no valid material";
        return false;
      }
      int idx;
      if (!shape(s, global[s.material_index], idx)) {
        err = "failed to convert shape: " + err;
        return false;
      }
    }
    for (const Statement& l : ps.lights)
      if (!light(l)) return false;
    // attribute blocks (processAttributeBlock, :397-468)
    for (const Block& b : ps.blocks) {
      std::vector<uint32_t> local;
      for (const Statement& m : b.materials) {
        gprt_material_desc md;
        if (!material(m, md)) return false;
        local.push_back(add_material(md));
      }
      std::vector<int> shape_of(b.shapes.size(), -1);
      for (size_t k = 0; k < b.shapes.size(); k++) {
        const Statement& s = b.shapes[k];
        uint32_t mat;
        if (s.material_index >= 0 && s.material_index < (int)local.size()) mat = local[s.material_index];
        else if (s.material_index >= 0 && s.material_index < (int)global.size()) mat = global[s.material_index];
        else {
          err = "failed to process attribute block: shape has no valid material";
          return false;
        }
        double L[3];
        if (s.area_light() && s.vec3_param("L", L)) {
          gprt_material_desc em = mat_zero();
          em.kind = GPRT_MAT_EMISSIVE;
          std::memcpy(em.emission, L, sizeof(L));
          mat = add_material(em);
        }
        if (!shape(s, mat, shape_of[k])) {
          err = "failed to process attribute block: failed to convert shape in attribute block: " + err;
          return false;
        }
      }
      for (size_t k = 0; k < b.shapes.size(); k++)
        if (b.shapes[k].area_light() && !area_light(b.shapes[k], shape_of[k])) return false;
      for (const Statement& l : b.lights)
        if (l.type != "AreaLightSource" && !light(l)) return false;
    }
    out.desc.materials = out.materials.data();
    out.desc.shapes = out.shapes.data();
    out.desc.meshes = out.meshes.data();
    out.desc.lights = out.lights.data();
    out.desc.n_materials = (uint32_t)out.materials.size();
    out.desc.n_shapes = (uint32_t)out.shapes.size();
    out.desc.n_meshes = (uint32_t)out.meshes.size();
    out.desc.n_lights = (uint32_t)out.lights.size();
    return true;
  }
};

void set_err(char* buf, size_t len, const std::string& msg) {
  if (!buf || !len) return;
  std::snprintf(buf, len, "%s", msg.c_str());
}

int parse_text(const std::string& text, const gprt_camera_desc* override, gprt_loaded** out, char* errbuf,
               size_t err_len) {
  if (!out) return GPRT_E_INVALID;
  *out = nullptr;
  Parser p;
  std::string err;
  std::istringstream in(text);
  std::string l;
  while (std::getline(in, l))
    if (!p.line(l, err)) {
      set_err(errbuf, err_len, "failed to parse PBRT: " + err);
      return GPRT_E_INVALID;
    }
  if (!p.flush(err)) {  // finalize (pbrt.go:267-270)
    set_err(errbuf, err_len, "failed to parse PBRT: " + err);
    return GPRT_E_INVALID;
  }
  auto ld = std::make_unique<gprt_loaded>();
  Converter cv{*ld, err};
  if (!cv.convert(p.scene, override)) {
    set_err(errbuf, err_len, err);
    return GPRT_E_INVALID;
  }
  *out = ld.release();
  return GPRT_OK;
}

// validateFilePath (pbrt.go:391-433)
bool valid_scene_path(const std::string& path, std::string& err) {
  if (path.empty()) {
    err = "filename cannot be empty";
    return false;
  }
  const char* td = std::getenv("TMPDIR");
  std::string tmp = td && *td ? td : "/tmp";
  bool in_scenes = starts_with(path, "scenes/") || path.find("scenes/") != std::string::npos;
  if (!in_scenes && !starts_with(path, tmp)) {
    err = "file path must be in scenes/ directory";
    return false;
  }
  if (path.find("..") != std::string::npos && path.find("scenes/") == std::string::npos) {
    err = "invalid file path: directory traversal not allowed";
    return false;
  }
  std::string low = path;
  for (char& ch : low) ch = (char)std::tolower((unsigned char)ch);
  if (!ends_with(low, ".pbrt")) {
    err = "invalid file type: only .pbrt files are allowed";
    return false;
  }
  if (path.size() > 512) {
    err = "file path too long: maximum 512 characters allowed";
    return false;
  }
  return true;
}

// ------------------------------------------------------------ PLY
struct PlyProp {
  std::string name, type, list_count, list_data;
  bool list = false;
};

bool known_type(const std::string& t) {
  for (const char* k : {"float", "float32", "double", "float64", "int", "int32", "uint", "uint32", "short", "int16",
                        "ushort", "uint16", "char", "int8", "uchar", "uint8"})
    if (t == k) return true;
  return false;
}

// getTypeSize (ply.go:542-556)
int type_size(const std::string& t) {
  if (t == "double" || t == "float64") return 8;
  if (t == "short" || t == "int16" || t == "ushort" || t == "uint16") return 2;
  if (t == "char" || t == "int8" || t == "uchar" || t == "uint8") return 1;
  return 4;
}

double read_scalar(const unsigned char* p, const std::string& t) {
  auto rd = [&](auto v) {
    std::memcpy(&v, p, sizeof(v));  // the file is little-endian, as the host
    return v;
  };
  if (t == "float" || t == "float32") return rd(float());
  if (t == "double" || t == "float64") return rd(double());
  if (t == "int" || t == "int32") return rd(int32_t());
  if (t == "uint" || t == "uint32") return rd(uint32_t());
  if (t == "short" || t == "int16") return rd(int16_t());
  if (t == "ushort" || t == "uint16") return rd(uint16_t());
  if (t == "char" || t == "int8") return rd(int8_t());
  if (t == "uchar" || t == "uint8") return rd(uint8_t());
  return rd(float());
}

int load_ply(const char* path, gprt_ply** out, std::string& err) {
  *out = nullptr;
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    err = std::string("failed to open PLY file: ") + path;
    return GPRT_E_INVALID;
  }
  std::string fmt, elem;
  uint64_t nv = 0, nf = 0;
  std::vector<PlyProp> vprops, fprops;
  std::string line;
  bool ended = false;
  while (std::getline(f, line)) {  // parsePLYHeader (ply.go:113-227)
    std::string t = trim(line, " \t\r\n");
    if (t == "end_header") {
      ended = true;
      break;
    }
    std::vector<std::string> parts = fields(t);
    if (parts.empty()) continue;
    if (parts[0] == "format" && parts.size() >= 3) {
      fmt = parts[1];
    } else if (parts[0] == "element" && parts.size() >= 3) {
      char* e = nullptr;
      unsigned long long c = std::strtoull(parts[2].c_str(), &e, 10);
      if (!e || *e) {
        err = "failed to parse PLY header: invalid element count: " + parts[2];
        return GPRT_E_INVALID;
      }
      elem = parts[1];
      if (elem == "vertex") nv = c;
      else if (elem == "face") nf = c;
    } else if (parts[0] == "property") {
      PlyProp pr;
      if (parts.size() >= 2 && parts[1] == "list") {
        if (parts.size() < 5) {
          err = "failed to parse PLY header: invalid list property definition";
          return GPRT_E_INVALID;
        }
        pr.list = true;
        pr.list_count = parts[2];
        pr.list_data = parts[3];
        pr.name = parts[4];
      } else {
        if (parts.size() < 3) {
          err = "failed to parse PLY header: invalid property definition";
          return GPRT_E_INVALID;
        }
        pr.type = parts[1];
        pr.name = parts[2];
      }
      if (elem == "vertex") vprops.push_back(pr);
      else if (elem == "face") fprops.push_back(pr);
    }
  }
  if (!ended) {
    err = "failed to parse PLY header: no end_header";
    return GPRT_E_INVALID;
  }
  if (fmt == "binary_big_endian") {
    err = "binary big-endian PLY format not yet implemented";
    return GPRT_E_INVALID;
  }
  if (fmt == "ascii") {
    err = "ASCII PLY format not yet supported";
    return GPRT_E_INVALID;
  }
  if (fmt != "binary_little_endian") {
    err = "unsupported PLY format: " + fmt;
    return GPRT_E_INVALID;
  }
  if (nv > 0xFFFFFFFFull || nf > 0x55555555ull) {
    err = "PLY element counts too large";
    return GPRT_E_INVALID;
  }
  auto ply = std::make_unique<gprt_ply>();
  // vertex properties by name (ply.go:146-186), offsets in the fixed-size record
  int vsize = 0;
  std::vector<int> off(vprops.size());
  int ix = -1, iy = -1, iz = -1, inx = -1, iny = -1, inz = -1, ir = -1, ig = -1, ib = -1, iu = -1, ivv = -1;
  for (size_t k = 0; k < vprops.size(); k++) {
    if (vprops[k].list) continue;  // calculateVertexSize skips lists (ply.go:529-540)
    off[k] = vsize;
    vsize += type_size(vprops[k].type);
    const std::string& n = vprops[k].name;
    int kk = (int)k;
    if (n == "x") ix = kk;
    else if (n == "y") iy = kk;
    else if (n == "z") iz = kk;
    else if (n == "nx") inx = kk;
    else if (n == "ny") iny = kk;
    else if (n == "nz") inz = kk;
    else if (n == "red" || n == "r") ir = kk;
    else if (n == "green" || n == "g") ig = kk;
    else if (n == "blue" || n == "b") ib = kk;
    else if (n == "u" || n == "s" || n == "texture_u") iu = kk;
    else if (n == "v" || n == "t" || n == "texture_v") ivv = kk;
  }
  bool has_n = inx >= 0 || iny >= 0 || inz >= 0, has_c = ir >= 0 || ig >= 0 || ib >= 0, has_t = iu >= 0 || ivv >= 0;
  std::vector<unsigned char> vb((size_t)vsize * nv);
  if (nv && !f.read(reinterpret_cast<char*>(vb.data()), (std::streamsize)vb.size())) {
    err = "failed to read PLY data: failed to read vertex data";
    return GPRT_E_INVALID;
  }
  ply->vertices.resize(3 * nv);
  if (has_n) ply->normals.resize(3 * nv);
  if (has_c) ply->colors.resize(3 * nv);
  if (has_t) ply->texcoords.resize(2 * nv);
  // parseVertexFromBytes (ply.go:570-664): positions, normals and texture
  // coordinates are read only from float properties, colours from uchar ones
  auto fl = [&](const unsigned char* rec, int k) -> double {
    if (k < 0) return 0.0;
    const std::string& t = vprops[k].type;
    if (t != "float" && t != "float32") return 0.0;
    return (double)(float)read_scalar(rec + off[k], t);
  };
  auto uc = [&](const unsigned char* rec, int k) -> double {
    if (k < 0) return 0.0;
    const std::string& t = vprops[k].type;
    if (t != "uchar" && t != "uint8") return 0.0;
    return read_scalar(rec + off[k], t) / 255.0;
  };
  for (uint64_t i = 0; i < nv; i++) {
    const unsigned char* rec = vb.data() + (size_t)i * vsize;
    ply->vertices[3 * i] = fl(rec, ix);
    ply->vertices[3 * i + 1] = fl(rec, iy);
    ply->vertices[3 * i + 2] = fl(rec, iz);
    if (has_n) {
      ply->normals[3 * i] = fl(rec, inx);
      ply->normals[3 * i + 1] = fl(rec, iny);
      ply->normals[3 * i + 2] = fl(rec, inz);
    }
    if (has_c) {
      ply->colors[3 * i] = uc(rec, ir);
      ply->colors[3 * i + 1] = uc(rec, ig);
      ply->colors[3 * i + 2] = uc(rec, ib);
    }
    if (has_t) {
      ply->texcoords[2 * i] = fl(rec, iu);
      ply->texcoords[2 * i + 1] = fl(rec, ivv);
    }
  }
  // faces (ply.go:317-385): triangles only; other face properties skipped
  ply->indices.reserve(3 * nf);
  std::vector<unsigned char> buf(8);
  for (uint64_t i = 0; i < nf; i++) {
    for (const PlyProp& pr : fprops) {
      if (pr.list && pr.name == "vertex_indices") {
        int cs;
        if (pr.list_count == "uchar" || pr.list_count == "uint8") cs = 1;
        else if (pr.list_count == "int" || pr.list_count == "int32") cs = 4;
        else {
          err = "failed to read PLY data: unsupported list count type: " + pr.list_count;
          return GPRT_E_INVALID;
        }
        if (!f.read(reinterpret_cast<char*>(buf.data()), cs)) {
          err = "failed to read PLY data: failed to read face vertex count at face " + std::to_string(i);
          return GPRT_E_INVALID;
        }
        long cnt = (long)read_scalar(buf.data(), pr.list_count);
        if (cnt != 3) {
          err = "failed to read PLY data: only triangular faces supported, got " + std::to_string(cnt) +
                " vertices at face " + std::to_string(i);
          return GPRT_E_INVALID;
        }
        if (pr.list_data != "int" && pr.list_data != "int32" && pr.list_data != "uint" && pr.list_data != "uint32") {
          err = "failed to read PLY data: unsupported face index data type: " + pr.list_data;
          return GPRT_E_INVALID;
        }
        for (int k = 0; k < 3; k++) {
          if (!f.read(reinterpret_cast<char*>(buf.data()), 4)) {
            err = "failed to read PLY data: failed to read face indices at face " + std::to_string(i);
            return GPRT_E_INVALID;
          }
          double x = read_scalar(buf.data(), pr.list_data);
          if (x < 0 || x >= (double)nv) {
            err = "PLY face index out of range at face " + std::to_string(i);
            return GPRT_E_INVALID;
          }
          ply->indices.push_back((uint32_t)x);
        }
      } else if (pr.list) {  // skipPropertyBuffered (ply.go:413-437): uchar counts only
        if (pr.list_count != "uchar" && pr.list_count != "uint8") {
          err = "failed to read PLY data: unsupported list count type: " + pr.list_count;
          return GPRT_E_INVALID;
        }
        if (!known_type(pr.list_data)) {
          err = "failed to read PLY data: unsupported data type: " + pr.list_data;
          return GPRT_E_INVALID;
        }
        if (!f.read(reinterpret_cast<char*>(buf.data()), 1)) {
          err = "failed to read PLY data: failed to skip face property " + pr.name;
          return GPRT_E_INVALID;
        }
        f.seekg((std::streamoff)buf[0] * type_size(pr.list_data), std::ios::cur);
      } else {
        if (!known_type(pr.type)) {
          err = "failed to read PLY data: unsupported data type: " + pr.type;
          return GPRT_E_INVALID;
        }
        f.seekg(type_size(pr.type), std::ios::cur);
      }
      if (!f) {
        err = "failed to read PLY data: truncated face data";
        return GPRT_E_INVALID;
      }
    }
  }
  ply->info.n_vertices = (uint32_t)nv;
  ply->info.n_triangles = (uint32_t)(ply->indices.size() / 3);
  ply->info.has_normals = has_n;
  ply->info.has_colors = has_c;
  ply->info.has_texcoords = has_t;
  *out = ply.release();
  return GPRT_OK;
}

}  // namespace
}  // namespace gprt

extern "C" {

int gprt_pbrt_parse(const char* text, size_t len, const gprt_camera_desc* camera_override, gprt_loaded** out,
                    char* errbuf, size_t err_len) {
  if (!text) return GPRT_E_INVALID;
  try {
    return gprt::parse_text(std::string(text, len), camera_override, out, errbuf, err_len);
  } catch (const std::exception& e) {
    gprt::set_err(errbuf, err_len, e.what());
    return GPRT_E_INVALID;
  }
}

int gprt_pbrt_load(const char* path, const gprt_camera_desc* camera_override, gprt_loaded** out, char* errbuf,
                   size_t err_len) {
  if (!path || !out) return GPRT_E_INVALID;
  *out = nullptr;
  std::string err;
  if (!gprt::valid_scene_path(path, err)) {
    gprt::set_err(errbuf, err_len, "invalid file path: " + err);
    return GPRT_E_INVALID;
  }
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    gprt::set_err(errbuf, err_len, std::string("failed to open PBRT file: ") + path);
    return GPRT_E_INVALID;
  }
  std::ostringstream ss;
  ss << f.rdbuf();
  std::string text = ss.str();
  return gprt_pbrt_parse(text.data(), text.size(), camera_override, out, errbuf, err_len);
}

const gprt_scene_desc* gprt_loaded_desc(const gprt_loaded* l) { return l ? &l->desc : nullptr; }

void gprt_loaded_free(gprt_loaded* l) { delete l; }

int gprt_ply_load(const char* path, gprt_ply** out, char* errbuf, size_t err_len) {
  if (!path || !out) return GPRT_E_INVALID;
  std::string err;
  try {
    int rc = gprt::load_ply(path, out, err);
    if (rc) gprt::set_err(errbuf, err_len, err);
    return rc;
  } catch (const std::exception& e) {
    gprt::set_err(errbuf, err_len, e.what());
    return GPRT_E_INVALID;
  }
}

int gprt_ply_get(const gprt_ply* p, gprt_ply_info* info, const double** vertices, const uint32_t** indices,
                 const double** normals, const double** colors, const double** texcoords) {
  if (!p) return GPRT_E_INVALID;
  if (info) *info = p->info;
  if (vertices) *vertices = p->vertices.empty() ? nullptr : p->vertices.data();
  if (indices) *indices = p->indices.empty() ? nullptr : p->indices.data();
  if (normals) *normals = p->normals.empty() ? nullptr : p->normals.data();
  if (colors) *colors = p->colors.empty() ? nullptr : p->colors.data();
  if (texcoords) *texcoords = p->texcoords.empty() ? nullptr : p->texcoords.data();
  return GPRT_OK;
}

void gprt_ply_free(gprt_ply* p) { delete p; }

}  // extern "C"
