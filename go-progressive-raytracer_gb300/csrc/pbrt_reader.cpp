// pbrt_reader.cpp - PBRT-v4 subset scene files to a gprt_scene_desc, on the
// host (C ABI: gprt_pbrt_parse, gprt_pbrt_load, gprt_loaded_desc,
// gprt_loaded_free).
//
// The accepted language and its meaning are those of the reference's
// loaders.ParsePBRT (pkg/loaders/pbrt.go) and scene.NewPBRTScene
// (pkg/scene/pbrt_scene.go); this reader is organised differently:
//
//   text --(RecordBuilder: per line)--> records: block markers and whole
//         statements (a statement line plus its continuation lines)
//   statement text --(lex: a 4-state machine)--> tokens
//   tokens --(read_directive)--> Directive {name, type, params}
//   directives --(Draft: scopes and the graphics-state stack)--> the
//         world: pre-world singletons, the top-level scope, and the
//         attribute blocks in the order they close
//   Draft --(DescWriter)--> gprt_loaded (a gprt_scene_desc and the arrays
//         it points to)
//
// Rules that decide what a file means, and so are kept as the reference
// has them: a line is a block marker only when it is exactly WorldBegin /
// WorldEnd / AttributeBegin / AttributeEnd; a statement starts on a line
// that begins with a known directive name, and any other non-comment line
// continues it; inside an attribute block a shape takes the last material
// of that block, or else the last top-level material; an AreaLightSource
// applies to the shapes that follow it in its block and in blocks opened
// inside it; the scene lists the top-level shapes, then the top-level
// lights, then each block (its shapes, the area lights made from them, its
// other lights) in the order the blocks close.  Error messages are the
// reference's.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/gprt.h"

struct gprt_loaded {
  gprt_scene_desc desc{};
  std::vector<gprt_material_desc> materials;
  std::vector<gprt_shape_desc> shapes;
  std::vector<gprt_mesh_desc> meshes;
  std::vector<gprt_light_desc> lights;
  std::deque<std::vector<double>> vertex_store;   // stable addresses for the mesh descriptions
  std::deque<std::vector<uint32_t>> index_store;
};

namespace gprt {
namespace pbrt {
namespace {

struct Failure {
  std::string msg;
};

std::string format(const char* fmt, double v) {
  char b[96];
  std::snprintf(b, sizeof(b), fmt, v);
  return b;
}

// ------------------------------------------------------------------ numbers
// A whole token as a float64 (strconv.ParseFloat); false when it is not one.
bool to_double(const std::string& s, double& out) {
  if (s.empty()) return false;
  const char* b = s.c_str();
  char* e = nullptr;
  errno = 0;
  double v = std::strtod(b, &e);
  if (e != b + s.size()) return false;
  out = v;
  return true;
}

// strconv.Atoi with its error ignored, as the reference reads mesh indices:
// a token that is not a decimal integer counts as 0.
long long to_int_or_zero(const std::string& s) {
  if (s.empty()) return 0;
  const char* b = s.c_str();
  char* e = nullptr;
  long long v = std::strtoll(b, &e, 10);
  return e == b + s.size() ? v : 0;
}

// ------------------------------------------------------------------ lexer
// The tokens of one statement.  Whitespace (space, tab) separates tokens
// outside quotes and brackets; a quote opens a token that the next quote
// closes (text before the opening quote stays in it); '[' starts a token
// that the next ']' closes (quotes inside it are plain characters, and a
// second '[' ends the unfinished one).  A token keeps its quotes or
// brackets: `"float radius"`, `[1 2 3]`.
std::vector<std::string> lex(const std::string& text) {
  enum State { Gap, Word, Quote, Bracket } st = Gap;
  std::vector<std::string> out;
  std::string cur;
  auto emit = [&]() {
    if (!cur.empty()) out.push_back(cur);
    cur.clear();
  };
  for (char ch : text) {
    bool blank = ch == ' ' || ch == '\t';
    switch (st) {
      case Gap:
        if (blank) break;
        cur.push_back(ch);
        st = ch == '"' ? Quote : ch == '[' ? Bracket : Word;
        break;
      case Word:
        if (blank) {
          emit();
          st = Gap;
        } else if (ch == '[') {
          emit();
          cur.push_back(ch);
          st = Bracket;
        } else {
          cur.push_back(ch);
          if (ch == '"') st = Quote;
        }
        break;
      case Quote:
        cur.push_back(ch);
        if (ch == '"') {
          emit();
          st = Gap;
        }
        break;
      case Bracket:
        if (ch == '[') {
          emit();
          cur.push_back(ch);
        } else {
          cur.push_back(ch);
          if (ch == ']') {
            emit();
            st = Gap;
          }
        }
        break;
    }
  }
  emit();
  return out;
}

bool quoted(const std::string& t) { return !t.empty() && t.front() == '"' && t.back() == '"'; }
bool bracketed(const std::string& t) { return !t.empty() && t.front() == '[' && t.back() == ']'; }

// `t` without the quotes at either end
std::string unquote(const std::string& t) {
  size_t a = 0, b = t.size();
  while (a < b && t[a] == '"') a++;
  while (b > a && t[b - 1] == '"') b--;
  return t.substr(a, b - a);
}

std::vector<std::string> split_blank(const std::string& s, size_t from = 0) {
  std::vector<std::string> out;
  size_t i = from, n = s.size();
  while (i < n) {
    while (i < n && std::isspace((unsigned char)s[i])) i++;
    size_t j = i;
    while (j < n && !std::isspace((unsigned char)s[j])) j++;
    if (j > i) out.push_back(s.substr(i, j - i));
    i = j;
  }
  return out;
}

// ------------------------------------------------------------------ directives
struct Param {
  std::string decl;  // the declared type ("float", "rgb", ...)
  std::vector<std::string> values;
};

struct Directive {
  std::string name;  // Camera, Shape, LookAt, ...
  std::string type;  // the quoted type after the name ("sphere"), or empty
  std::map<std::string, Param> params;
  int material = -1;        // shapes: the material slot resolved when the shape was read
  bool area_light = false;  // shapes: an AreaLightSource applies to it

  const Param* find(const char* k) const {
    auto it = params.find(k);
    return it == params.end() ? nullptr : &it->second;
  }
  // GetFloatParam / GetRGBParam / GetPoint3Param (pbrt.go:649-704): absent
  // or unparsable values read as "not given"
  bool number(const char* k, double& v) const {
    const Param* p = find(k);
    return p && !p->values.empty() && to_double(p->values[0], v);
  }
  bool triple(const char* k, double v[3]) const {
    const Param* p = find(k);
    if (!p || p->values.size() < 3) return false;
    double t[3];
    for (int i = 0; i < 3; i++)
      if (!to_double(p->values[i], t[i])) return false;
    std::memcpy(v, t, sizeof(t));
    return true;
  }
};

// The directive names that open a statement (isStatementStart, pbrt.go:707-722).
const char* const kStatementNames[] = {"Camera",      "Film",       "Sampler",         "Integrator", "LookAt",
                                       "Material",    "Shape",      "LightSource",     "AreaLightSource",
                                       "Translate",   "Rotate",     "Scale",           "Transform",
                                       "ReverseOrientation",        "Attribute"};

bool opens_statement(const std::string& line) {
  for (const char* n : kStatementNames) {
    size_t k = std::strlen(n);
    if (line.compare(0, k, n) == 0 && (line.size() == k || line[k] == ' ')) return true;
  }
  return false;
}

// One statement's text to a Directive (parseStatement, pbrt.go:558-647).
// The matrix and look-at directives carry their numbers as a "values" list.
Directive read_directive(const std::string& text) {
  Directive d;
  for (const char* n : {"LookAt", "Translate", "Rotate", "Scale", "Transform"}) {
    size_t k = std::strlen(n);
    if (text.compare(0, k, n) == 0) {
      d.name = n;
      d.params["values"] = Param{"float", split_blank(text, k)};
      return d;
    }
  }
  std::vector<std::string> tok = lex(text);
  if (tok.size() < 2) throw Failure{"invalid statement format"};
  d.name = tok[0];
  size_t i = 1;
  if (quoted(tok[1])) {
    d.type = unquote(tok[1]);
    i = 2;
  }
  // "decl name" value-or-[list] pairs; anything else is skipped
  while (i < tok.size()) {
    const std::string& t = tok[i++];
    if (t.empty() || t[0] != '"') continue;
    std::vector<std::string> decl = split_blank(unquote(t));
    if (decl.size() != 2) continue;
    Param p{decl[0], {}};
    if (i < tok.size()) {
      const std::string& v = tok[i++];
      if (bracketed(v)) {
        size_t a = 0, b = v.size();
        while (a < b && (v[a] == '[' || v[a] == ']' || v[a] == ' ')) a++;
        while (b > a && (v[b - 1] == '[' || v[b - 1] == ']' || v[b - 1] == ' ')) b--;
        p.values = split_blank(v.substr(a, b - a));
      } else {
        p.values.push_back(v);
      }
    }
    d.params[decl[1]] = std::move(p);
  }
  return d;
}

// ------------------------------------------------------------------ draft
// The world as read: pre-world singletons, the top-level scope, and the
// attribute blocks in the order they closed.
struct Scope {
  std::vector<Directive> materials, shapes, lights;
};

struct Draft {
  std::unique_ptr<Directive> camera, film;
  bool has_look = false;
  double look[9] = {0};
  Scope top;
  std::vector<Scope> closed;  // completion order
  int top_material = -1;      // slot of the last top-level material

  // open blocks and, per block, the graphics state it restores
  struct Frame {
    Scope scope;
    int saved_material;
    std::shared_ptr<const Directive> area;  // the AreaLightSource in force in this block
  };
  std::vector<Frame> open;
  bool in_world = false;

  void begin_block() {
    Frame f;
    f.saved_material = top_material;
    if (!open.empty()) f.area = open.back().area;  // inherited by nested blocks
    open.push_back(std::move(f));
  }
  void end_block() {
    if (open.empty()) return;  // an unmatched AttributeEnd changes nothing
    closed.push_back(std::move(open.back().scope));
    top_material = open.back().saved_material;
    open.pop_back();
  }

  // parseLookAt (pbrt.go:435-490)
  void look_at(const Directive& d) {
    const Param& p = d.params.at("values");
    if (p.values.size() != 9) throw Failure{"error parsing LookAt: LookAt requires 9 values"};
    static const char* what[9] = {"eye X", "eye Y", "eye Z", "look-at X", "look-at Y", "look-at Z",
                                  "up X",  "up Y",  "up Z"};
    for (int k = 0; k < 9; k++)
      if (!to_double(p.values[k], look[k]))
        throw Failure{"error parsing LookAt: invalid " + std::string(what[k]) + " coordinate '" + p.values[k] +
                      "'"};
    has_look = true;
  }

  // A shape takes the material and area light in force where it appears.
  void place_shape(Directive d) {
    if (!open.empty()) {
      Frame& f = open.back();
      d.material = !f.scope.materials.empty() ? (int)f.scope.materials.size() - 1 : top_material;
      if (f.area) {
        d.area_light = true;
        for (const char* k : {"L", "power"}) {
          const Param* p = f.area->find(k);
          if (p) d.params[k] = *p;
        }
      }
      f.scope.shapes.push_back(std::move(d));
    } else {
      d.material = top_material;
      top.shapes.push_back(std::move(d));
    }
  }

  // routeStatement (pbrt.go:272-389)
  void take(Directive d) {
    if (d.name == "LookAt") {
      look_at(d);
      return;
    }
    const std::string& n = d.name;
    if (!open.empty()) {
      Frame& f = open.back();
      if (n == "Material") f.scope.materials.push_back(std::move(d));
      else if (n == "Shape") place_shape(std::move(d));
      else if (n == "LightSource") f.scope.lights.push_back(std::move(d));
      else if (n == "AreaLightSource") {
        f.area = std::make_shared<const Directive>(d);
        f.scope.lights.push_back(std::move(d));
      }
      return;  // transforms and anything else: no effect on the scene
    }
    if (!in_world) {
      if (n == "Camera") camera = std::make_unique<Directive>(std::move(d));
      else if (n == "Film") film = std::make_unique<Directive>(std::move(d));
      return;  // Sampler, Integrator: read and unused
    }
    if (n == "Material") {
      top.materials.push_back(std::move(d));
      top_material = (int)top.materials.size() - 1;
    } else if (n == "Shape") {
      place_shape(std::move(d));
    } else if (n == "LightSource" || n == "AreaLightSource") {
      top.lights.push_back(std::move(d));
    }
  }
};

// ------------------------------------------------------------------ records
// Groups lines into statements (processLine, pbrt.go:227-265) and feeds the
// draft in file order.
struct RecordBuilder {
  Draft& draft;
  std::vector<std::string> pending;  // the lines of the open statement

  void flush(const char* where) {
    if (pending.empty()) return;
    std::string text;
    for (size_t k = 0; k < pending.size(); k++) {
      if (k) text.push_back(' ');
      text += pending[k];
    }
    pending.clear();
    Directive d;
    try {
      d = read_directive(text);
    } catch (const Failure& f) {
      throw Failure{std::string("error parsing statement ") + where + " '" + text + "': " + f.msg};
    }
    draft.take(std::move(d));
  }

  void line(std::string s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    s = s.substr(a, b - a);
    if (s.empty() || s[0] == '#') return;
    if (s == "WorldBegin") {
      flush("before WorldBegin");
      draft.in_world = true;
    } else if (s == "WorldEnd") {
      flush("before WorldEnd");
      draft.in_world = false;
    } else if (s == "AttributeBegin") {
      flush("before AttributeBegin");
      draft.begin_block();
    } else if (s == "AttributeEnd") {
      flush("before AttributeEnd");
      draft.end_block();
    } else if (opens_statement(s)) {
      flush("");
      pending.push_back(s);
    } else {
      if (pending.empty()) throw Failure{"unexpected continuation line: " + s};
      pending.push_back(s);
    }
  }
};

// ------------------------------------------------------------------ conversion
// NewPBRTScene (pbrt_scene.go:15-78) into the library's scene description.
struct DescWriter {
  gprt_loaded& out;

  static gprt_material_desc blank_material() {
    gprt_material_desc m;
    std::memset(&m, 0, sizeof(m));
    return m;
  }
  static gprt_light_desc blank_light() {
    gprt_light_desc l;
    std::memset(&l, 0, sizeof(l));
    l.weight = 1.0;
    return l;
  }

  // convertMaterial (pbrt_scene.go:160-202): diffuse, conductor, dielectric
  uint32_t material(const Directive& d) {
    gprt_material_desc m = blank_material();
    double v;
    if (d.type == "diffuse") {
      m.kind = GPRT_MAT_LAMBERTIAN;
      m.albedo[0] = m.albedo[1] = m.albedo[2] = 0.7;
      d.triple("reflectance", m.albedo);
    } else if (d.type == "conductor") {
      m.kind = GPRT_MAT_METAL;
      m.albedo[0] = 0.7;
      m.albedo[1] = 0.6;
      m.albedo[2] = 0.5;
      d.triple("eta", m.albedo);
      if (d.number("roughness", v)) {
        if (v < 0 || v > 1) throw Failure{format("invalid metal roughness %f: must be between 0 and 1", v)};
        m.fuzz = v;
      }
    } else if (d.type == "dielectric") {
      m.kind = GPRT_MAT_DIELECTRIC;
      m.ior = 1.5;
      if (d.number("eta", v)) {
        if (v <= 0) throw Failure{format("invalid dielectric IOR %f: must be positive", v)};
        m.ior = v;
      }
    } else {
      throw Failure{"unsupported material type: " + d.type};
    }
    out.materials.push_back(m);
    return (uint32_t)out.materials.size() - 1;
  }

  uint32_t emissive(const double L[3]) {
    gprt_material_desc m = blank_material();
    m.kind = GPRT_MAT_EMISSIVE;
    std::memcpy(m.emission, L, 3 * sizeof(double));
    out.materials.push_back(m);
    return (uint32_t)out.materials.size() - 1;
  }

  // triangle mesh arrays, owned by the loaded handle
  uint32_t mesh(const Directive& d) {
    const Param* P = d.find("P");
    if (!P || P->values.size() % 3 != 0) throw Failure{"trianglemesh missing or invalid vertices"};
    out.vertex_store.emplace_back(P->values.size());
    std::vector<double>& v = out.vertex_store.back();
    static const char* axis[3] = {"X", "Y", "Z"};
    for (size_t k = 0; k < v.size(); k++)
      if (!to_double(P->values[k], v[k]))
        throw Failure{"invalid vertex " + std::string(axis[k % 3]) + " coordinate '" + P->values[k] + "'"};
    const Param* I = d.find("indices");
    if (!I || I->values.size() % 3 != 0) throw Failure{"trianglemesh missing or invalid indices"};
    out.index_store.emplace_back(I->values.size());
    std::vector<uint32_t>& idx = out.index_store.back();
    const long long nv = (long long)(v.size() / 3);
    for (size_t k = 0; k < idx.size(); k++) {
      long long x = to_int_or_zero(I->values[k]);
      // the reference's NewTriangleMesh indexes past its vertices and panics
      if (x < 0 || x >= nv) throw Failure{"trianglemesh index out of range"};
      idx[k] = (uint32_t)x;
    }
    gprt_mesh_desc md;
    std::memset(&md, 0, sizeof(md));
    md.vertices = v.data();
    md.indices = idx.data();
    md.n_vertices = (uint32_t)nv;
    md.n_triangles = (uint32_t)(idx.size() / 3);
    out.meshes.push_back(md);
    return (uint32_t)out.meshes.size() - 1;
  }

  // convertShape (pbrt_scene.go:204-305): sphere, bilinearPatch, trianglemesh, box
  uint32_t shape(const Directive& d, uint32_t mat) {
    gprt_shape_desc s;
    std::memset(&s, 0, sizeof(s));
    s.material = mat;
    if (d.type == "sphere") {
      s.kind = GPRT_SHAPE_SPHERE;
      double r;
      s.p[3] = 1.0;
      if (d.number("radius", r)) {
        if (r <= 0) throw Failure{format("invalid sphere radius %f: must be positive", r)};
        s.p[3] = r;
      }
      d.triple("center", s.p);
    } else if (d.type == "bilinearPatch") {
      double c[4][3];
      const char* names[4] = {"P00", "P01", "P10", "P11"};
      for (int k = 0; k < 4; k++)
        if (!d.triple(names[k], c[k])) throw Failure{"bilinearPatch missing corner points"};
      s.kind = GPRT_SHAPE_QUAD;  // corner P00, u = P01 - P00, v = P10 - P00 (P11 is not used)
      for (int a = 0; a < 3; a++) {
        s.p[a] = c[0][a];
        s.p[3 + a] = c[1][a] - c[0][a];
        s.p[6 + a] = c[2][a] - c[0][a];
      }
    } else if (d.type == "trianglemesh") {
      s.kind = GPRT_SHAPE_MESH;
      s.mesh = mesh(d);
    } else if (d.type == "box") {
      s.kind = GPRT_SHAPE_BOX;
      s.p[3] = s.p[4] = s.p[5] = 1.0;  // half extents
      d.triple("center", s.p);
      d.triple("size", s.p + 3);
      d.triple("rotation", s.p + 6);
    } else {
      throw Failure{"unsupported shape type: " + d.type};
    }
    out.shapes.push_back(s);
    return (uint32_t)out.shapes.size() - 1;
  }

  // convertLight (pbrt_scene.go:338-395)
  void light(const Directive& d) {
    gprt_light_desc l = blank_light();
    if (d.type == "point") {  // a 0.1-radius sphere light that is not a scene shape
      l.kind = GPRT_LIGHT_SPHERE;
      l.shape = GPRT_NO_SHAPE;
      l.color_a[0] = l.color_a[1] = l.color_a[2] = 10.0;
      l.from[1] = 5.0;
      d.triple("I", l.color_a);
      d.triple("from", l.from);
      l.radius = 0.1;
    } else if (d.type == "distant" || d.type == "infinite") {
      l.kind = GPRT_LIGHT_UNIFORM_INFINITE;
      double def = d.type == "distant" ? 3.0 : 1.0;
      l.color_a[0] = l.color_a[1] = l.color_a[2] = def;
      d.triple("L", l.color_a);
    } else if (d.type == "infinite-gradient") {
      l.kind = GPRT_LIGHT_GRADIENT_INFINITE;
      double top[3] = {0.5, 0.7, 1.0};
      std::memcpy(l.color_a, top, sizeof(top));
      l.color_b[0] = l.color_b[1] = l.color_b[2] = 1.0;
      d.triple("topColor", l.color_a);
      d.triple("bottomColor", l.color_b);
    } else if (d.type == "diffuse") {
      throw Failure{"AreaLightSource should be handled as graphics state, not converted as standalone light"};
    } else {
      throw Failure{"unsupported light type: " + d.type};
    }
    out.lights.push_back(l);
  }

  // convertAreaLight (pbrt_scene.go:307-336): a light on a converted quad or sphere
  void area_light(const Directive& d, uint32_t shape_index) {
    double L[3];
    if (!d.triple("L", L)) throw Failure{"area light missing emission parameter 'L'"};
    gprt_light_desc l = blank_light();
    uint32_t kind = out.shapes[shape_index].kind;
    if (kind == GPRT_SHAPE_QUAD) l.kind = GPRT_LIGHT_QUAD;
    else if (kind == GPRT_SHAPE_SPHERE) l.kind = GPRT_LIGHT_SPHERE;
    else
      throw Failure{std::string("shape type ") + (kind == GPRT_SHAPE_BOX ? "*geometry.Box" : "*geometry.TriangleMesh") +
                    " is not supported as an area light"};
    l.shape = shape_index;
    out.lights.push_back(l);
  }

  // convertCamera (pbrt_scene.go:93-158) with createDefaultPBRTSamplingConfig (:80-91)
  void camera(const Draft& w, const gprt_camera_desc* ov) {
    gprt_sampling_desc& sm = out.desc.sampling;
    sm.width = sm.height = 400;
    sm.samples_per_pixel = 150;
    sm.max_depth = 5;
    sm.rr_min_bounces = 16;
    sm.adaptive_min_samples = 0.20;
    sm.adaptive_threshold = 0.005;
    gprt_camera_desc& c = out.desc.camera;
    std::memset(&c, 0, sizeof(c));
    c.look_at[2] = -1.0;
    c.up[1] = 1.0;
    c.width = 400;
    c.aspect_ratio = 1.0;
    c.vfov_deg = 90.0;
    c.focus_distance = 1.0;
    if (w.has_look) {
      std::memcpy(c.center, w.look, 3 * sizeof(double));
      std::memcpy(c.look_at, w.look + 3, 3 * sizeof(double));
      std::memcpy(c.up, w.look + 6, 3 * sizeof(double));
    }
    double v;
    if (w.camera && w.camera->type == "perspective" && w.camera->number("fov", v)) {
      if (v <= 0 || v >= 180) throw Failure{format("invalid camera FOV %f: must be between 0 and 180 degrees", v)};
      c.vfov_deg = v;
    }
    if (w.film) {
      if (w.film->number("xresolution", v)) {
        if (v <= 0 || v > 8192) throw Failure{format("invalid image width %f: must be between 1 and 8192", v)};
        c.width = (uint32_t)(int)v;
        sm.width = c.width;
      }
      if (w.film->number("yresolution", v)) {
        if (v <= 0 || v > 8192) throw Failure{format("invalid image height %f: must be between 1 and 8192", v)};
        sm.height = (uint32_t)(int)v;
        c.aspect_ratio = (double)c.width / v;
      }
    }
    if (ov) {  // MergeCameraConfig (camera.go:320-349): the override's non-zero fields win
      auto given = [](const double* x) { return std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]) != 0; };
      if (given(ov->center)) std::memcpy(c.center, ov->center, 3 * sizeof(double));
      if (given(ov->look_at)) std::memcpy(c.look_at, ov->look_at, 3 * sizeof(double));
      if (given(ov->up)) std::memcpy(c.up, ov->up, 3 * sizeof(double));
      if (ov->width) c.width = ov->width;
      if (ov->aspect_ratio != 0) c.aspect_ratio = ov->aspect_ratio;
      if (ov->vfov_deg != 0) c.vfov_deg = ov->vfov_deg;
      if (ov->aperture != 0) c.aperture = ov->aperture;
      if (ov->focus_distance != 0) c.focus_distance = ov->focus_distance;
      if (ov->width > 0) {
        sm.width = ov->width;
        sm.height = (uint32_t)(int)((double)ov->width / c.aspect_ratio);
      }
    }
  }

  template <class F>
  static void within(const char* ctx, F&& f) {
    try {
      f();
    } catch (const Failure& e) {
      throw Failure{std::string(ctx) + e.msg};
    }
  }

  void write(const Draft& w, const gprt_camera_desc* ov) {
    within("failed to convert camera: ", [&] { camera(w, ov); });
    std::vector<uint32_t> top_mats;
    for (const Directive& m : w.top.materials)
      within("failed to convert material: ", [&] { top_mats.push_back(material(m)); });
    for (const Directive& s : w.top.shapes) {
      if (s.material < 0 || s.material >= (int)top_mats.size())
        throw Failure{"shape has no valid material (MaterialIndex: " + std::to_string(s.material) + ")"};
      within("failed to convert shape: ", [&] { shape(s, top_mats[s.material]); });
    }
    for (const Directive& l : w.top.lights) within("failed to convert light: ", [&] { light(l); });
    for (const Scope& b : w.closed) within("failed to process attribute block: ", [&] { block(b, top_mats); });
    out.desc.materials = out.materials.data();
    out.desc.shapes = out.shapes.data();
    out.desc.meshes = out.meshes.data();
    out.desc.lights = out.lights.data();
    out.desc.n_materials = (uint32_t)out.materials.size();
    out.desc.n_shapes = (uint32_t)out.shapes.size();
    out.desc.n_meshes = (uint32_t)out.meshes.size();
    out.desc.n_lights = (uint32_t)out.lights.size();
  }

  // processAttributeBlock (pbrt_scene.go:397-468)
  void block(const Scope& b, const std::vector<uint32_t>& top_mats) {
    std::vector<uint32_t> local;
    for (const Directive& m : b.materials)
      within("failed to convert material in attribute block: ", [&] { local.push_back(material(m)); });
    std::vector<uint32_t> made(b.shapes.size());
    for (size_t k = 0; k < b.shapes.size(); k++) {
      const Directive& s = b.shapes[k];
      uint32_t mat;
      if (s.material >= 0 && s.material < (int)local.size()) mat = local[s.material];
      else if (s.material >= 0 && s.material < (int)top_mats.size()) mat = top_mats[s.material];
      else
        throw Failure{"shape has no valid material (MaterialIndex: " + std::to_string(s.material) +
                      ", local materials: " + std::to_string(local.size()) +
                      ", global materials: " + std::to_string(top_mats.size()) + ")"};
      double L[3];
      if (s.area_light && s.triple("L", L)) mat = emissive(L);
      within("failed to convert shape in attribute block: ", [&] { made[k] = shape(s, mat); });
    }
    for (size_t k = 0; k < b.shapes.size(); k++)
      if (b.shapes[k].area_light) within("failed to convert area light: ", [&] { area_light(b.shapes[k], made[k]); });
    for (const Directive& l : b.lights)
      if (l.name != "AreaLightSource") within("failed to convert light in attribute block: ", [&] { light(l); });
  }
};

// ------------------------------------------------------------------ paths
// Lexical clean of a slash-separated path (what filepath.Clean computes):
// repeated separators and "." elements removed, ".." elements resolved
// against the element before them where there is one.
std::string clean_path(const std::string& p) {
  if (p.empty()) return ".";
  bool rooted = p[0] == '/';
  std::vector<std::string> parts;
  size_t i = 0;
  while (i <= p.size()) {
    size_t j = p.find('/', i);
    if (j == std::string::npos) j = p.size();
    std::string e = p.substr(i, j - i);
    if (e.empty() || e == ".") {
    } else if (e == "..") {
      if (!parts.empty() && parts.back() != "..") parts.pop_back();
      else if (!rooted) parts.push_back("..");
    } else {
      parts.push_back(e);
    }
    i = j + 1;
  }
  std::string out = rooted ? "/" : "";
  for (size_t k = 0; k < parts.size(); k++) {
    if (k) out.push_back('/');
    out += parts[k];
  }
  return out.empty() ? "." : out;
}

// validateFilePath (pbrt.go:391-433): scene files live under a scenes/
// directory (or the temporary directory), end in .pbrt and are at most 512
// bytes long.
void check_scene_path(const std::string& name) {
  if (name.empty()) throw Failure{"filename cannot be empty"};
  std::string p = clean_path(name);
  const char* td = std::getenv("TMPDIR");
  std::string tmp = td && *td ? td : "/tmp";
  bool scenes = p.compare(0, 7, "scenes/") == 0 || p.find("scenes/") != std::string::npos;
  if (!scenes && p.compare(0, tmp.size(), tmp) != 0) throw Failure{"file path must be in scenes/ directory"};
  if (p.find("..") != std::string::npos && !scenes)
    throw Failure{"invalid file path: directory traversal not allowed"};
  std::string low = p;
  for (char& ch : low) ch = (char)std::tolower((unsigned char)ch);
  if (low.size() < 5 || low.compare(low.size() - 5, 5, ".pbrt") != 0)
    throw Failure{"invalid file type: only .pbrt files are allowed"};
  if (p.size() > 512) throw Failure{"file path too long: maximum 512 characters allowed"};
}

void set_err(char* buf, size_t len, const std::string& msg) {
  if (buf && len) std::snprintf(buf, len, "%s", msg.c_str());
}

int read_text(const std::string& text, const gprt_camera_desc* ov, gprt_loaded** out, char* errbuf, size_t err_len) {
  Draft w;
  try {
    RecordBuilder rb{w, {}};
    size_t i = 0;
    while (i < text.size()) {
      size_t j = text.find('\n', i);
      if (j == std::string::npos) j = text.size();
      rb.line(text.substr(i, j - i));
      i = j + 1;
    }
    rb.flush("at end of file");
  } catch (const Failure& f) {
    set_err(errbuf, err_len, "failed to parse PBRT: " + f.msg);
    return GPRT_E_INVALID;
  }
  auto ld = std::make_unique<gprt_loaded>();
  try {
    DescWriter{*ld}.write(w, ov);
  } catch (const Failure& f) {
    set_err(errbuf, err_len, f.msg);
    return GPRT_E_INVALID;
  }
  *out = ld.release();
  return GPRT_OK;
}

}  // namespace
}  // namespace pbrt
}  // namespace gprt

extern "C" {

int gprt_pbrt_parse(const char* text, size_t len, const gprt_camera_desc* camera_override, gprt_loaded** out,
                    char* errbuf, size_t err_len) {
  if (!text || !out) return GPRT_E_INVALID;
  *out = nullptr;
  try {
    return gprt::pbrt::read_text(std::string(text, len), camera_override, out, errbuf, err_len);
  } catch (const std::exception& e) {
    gprt::pbrt::set_err(errbuf, err_len, e.what());
    return GPRT_E_INVALID;
  }
}

int gprt_pbrt_load(const char* path, const gprt_camera_desc* camera_override, gprt_loaded** out, char* errbuf,
                   size_t err_len) {
  if (!path || !out) return GPRT_E_INVALID;
  *out = nullptr;
  try {
    gprt::pbrt::check_scene_path(path);
  } catch (const gprt::pbrt::Failure& f) {
    gprt::pbrt::set_err(errbuf, err_len, "invalid file path: " + f.msg);
    return GPRT_E_INVALID;
  }
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    gprt::pbrt::set_err(errbuf, err_len, std::string("failed to open PBRT file: ") + path);
    return GPRT_E_INVALID;
  }
  std::ostringstream ss;
  ss << f.rdbuf();
  std::string text = ss.str();
  return gprt_pbrt_parse(text.data(), text.size(), camera_override, out, errbuf, err_len);
}

const gprt_scene_desc* gprt_loaded_desc(const gprt_loaded* l) { return l ? &l->desc : nullptr; }

void gprt_loaded_free(gprt_loaded* l) { delete l; }

}  // extern "C"
