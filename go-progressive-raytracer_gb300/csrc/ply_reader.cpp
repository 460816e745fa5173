// ply_reader.cpp - binary little-endian PLY meshes to the arrays of a
// gprt_mesh_desc, on the host (C ABI: gprt_ply_load, gprt_ply_get,
// gprt_ply_free).
//
// Reads what the reference's loaders.LoadPLY reads (pkg/loaders/ply.go:72-
// 370): vertex positions, and when present normals (nx ny nz), colours (red
// green blue as uchar / 255) and texture coordinates (u v, s t or
// texture_u texture_v); triangular faces from a `vertex_indices` list whose
// count is uchar or int and whose items are int or uint.  Other properties
// are skipped.  ASCII and big-endian files are refused with the reference's
// messages.
//
// The file is read into memory once; the header becomes a list of element
// layouts (name, count, properties with their byte sizes), and the body is
// walked with one bounds-checked cursor, element by element in header
// order.  Fixed-size vertex records are decoded by precomputed byte offsets.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/gprt.h"

struct gprt_ply {
  std::vector<double> vertices, normals, colors, texcoords;
  std::vector<uint32_t> indices;
  gprt_ply_info info{};
};

namespace gprt {
namespace ply {
namespace {

struct Failure {
  std::string msg;
};

// Scalar types of the format and their sizes (0: unknown).
int scalar_size(const std::string& t) {
  if (t == "char" || t == "int8" || t == "uchar" || t == "uint8") return 1;
  if (t == "short" || t == "int16" || t == "ushort" || t == "uint16") return 2;
  if (t == "int" || t == "int32" || t == "uint" || t == "uint32" || t == "float" || t == "float32") return 4;
  if (t == "double" || t == "float64") return 8;
  return 0;
}

struct Property {
  std::string name, type;      // scalar property
  bool list = false;
  std::string count_type;      // list: type of the item count
  std::string item_type;       // list: type of the items
};

struct Element {
  std::string name;
  uint64_t count = 0;
  std::vector<Property> props;
};

struct Header {
  std::string format;
  std::vector<Element> elements;
  size_t body = 0;  // byte offset of the first element's data
};

std::vector<std::string> words(const std::string& s) {
  std::vector<std::string> out;
  std::istringstream in(s);
  std::string w;
  while (in >> w) out.push_back(w);
  return out;
}

// The header lines up to end_header (parsePLYHeader, ply.go:113-217).
Header read_header(const std::string& file) {
  Header h;
  size_t pos = 0;
  bool ended = false;
  while (pos < file.size()) {
    size_t nl = file.find('\n', pos);
    size_t next = nl == std::string::npos ? file.size() : nl + 1;
    std::string line = file.substr(pos, (nl == std::string::npos ? file.size() : nl) - pos);
    pos = next;
    std::vector<std::string> w = words(line);
    if (w.size() == 1 && w[0] == "end_header") {
      ended = true;
      break;
    }
    if (w.empty()) continue;
    if (w[0] == "format") {
      if (w.size() >= 3) h.format = w[1];
    } else if (w[0] == "element") {
      if (w.size() >= 3) {
        char* e = nullptr;
        unsigned long long n = std::strtoull(w[2].c_str(), &e, 10);
        if (w[2].empty() || *e || w[2][0] == '-')
          throw Failure{"failed to parse PLY header: invalid element count: " + w[2]};
        Element el;
        el.name = w[1];
        el.count = n;
        h.elements.push_back(el);
      }
    } else if (w[0] == "property") {
      Property p;
      if (w.size() < 3) throw Failure{"failed to parse PLY header: failed to parse property: invalid property definition"};
      if (w[1] == "list") {
        if (w.size() < 5)
          throw Failure{"failed to parse PLY header: failed to parse property: invalid list property definition"};
        p.list = true;
        p.count_type = w[2];
        p.item_type = w[3];
        p.name = w[4];
      } else {
        p.type = w[1];
        p.name = w[2];
      }
      if (!h.elements.empty()) h.elements.back().props.push_back(p);
    }
    // "ply", "comment", "obj_info" and anything else: nothing to keep
  }
  if (!ended) throw Failure{"failed to parse PLY header: no end_header line"};
  h.body = pos;
  return h;
}

// Little-endian reads through one bounds-checked cursor.
struct Cursor {
  const unsigned char* p;
  size_t n, at = 0;
  const unsigned char* take(size_t k, const char* what) {
    if (at + k > n) throw Failure{std::string("failed to read PLY data: ") + what + ": unexpected EOF"};
    const unsigned char* r = p + at;
    at += k;
    return r;
  }
};

uint64_t load_le(const unsigned char* b, int size) {
  uint64_t v = 0;
  for (int k = size - 1; k >= 0; k--) v = (v << 8) | b[k];
  return v;
}

// A scalar of type `t` at `b` as a double (integers by value).
double scalar(const unsigned char* b, const std::string& t) {
  int sz = scalar_size(t);
  uint64_t u = load_le(b, sz);
  if (t == "float" || t == "float32") {
    float f;
    uint32_t w = (uint32_t)u;
    std::memcpy(&f, &w, 4);
    return f;
  }
  if (t == "double" || t == "float64") {
    double d;
    std::memcpy(&d, &u, 8);
    return d;
  }
  if (t == "char" || t == "int8") return (double)(int8_t)u;
  if (t == "short" || t == "int16") return (double)(int16_t)u;
  if (t == "int" || t == "int32") return (double)(int32_t)u;
  return (double)u;  // unsigned types
}

// Where a vertex record holds each attribute (-1: absent).
struct VertexLayout {
  size_t stride = 0;
  int pos[3] = {-1, -1, -1}, nrm[3] = {-1, -1, -1}, col[3] = {-1, -1, -1}, tex[2] = {-1, -1};
  std::string pos_t[3], nrm_t[3], col_t[3], tex_t[2];
  bool normals = false, colors = false, texcoords = false;
};

VertexLayout vertex_layout(const Element& el) {
  VertexLayout L;
  for (const Property& p : el.props) {
    if (p.list) throw Failure{"failed to read PLY data: list property '" + p.name + "' in vertex records"};
    int sz = scalar_size(p.type);
    if (!sz) throw Failure{"failed to read PLY data: unsupported data type: " + p.type};
    int off = (int)L.stride;
    auto set = [&](int* slots, std::string* types, int k) {
      slots[k] = off;
      types[k] = p.type;
    };
    const std::string& n = p.name;
    if (n == "x") set(L.pos, L.pos_t, 0);
    else if (n == "y") set(L.pos, L.pos_t, 1);
    else if (n == "z") set(L.pos, L.pos_t, 2);
    else if (n == "nx") set(L.nrm, L.nrm_t, 0), L.normals = true;
    else if (n == "ny") set(L.nrm, L.nrm_t, 1), L.normals = true;
    else if (n == "nz") set(L.nrm, L.nrm_t, 2), L.normals = true;
    else if (n == "red" || n == "r") set(L.col, L.col_t, 0), L.colors = true;
    else if (n == "green" || n == "g") set(L.col, L.col_t, 1), L.colors = true;
    else if (n == "blue" || n == "b") set(L.col, L.col_t, 2), L.colors = true;
    else if (n == "u" || n == "s" || n == "texture_u") set(L.tex, L.tex_t, 0), L.texcoords = true;
    else if (n == "v" || n == "t" || n == "texture_v") set(L.tex, L.tex_t, 1), L.texcoords = true;
    L.stride += (size_t)sz;
  }
  return L;
}

void read_vertices(Cursor& c, const Element& el, gprt_ply& out) {
  VertexLayout L = vertex_layout(el);
  const unsigned char* base = c.take(L.stride * el.count, "failed to read vertex data");
  size_t n = (size_t)el.count;
  out.vertices.assign(3 * n, 0.0);
  if (L.normals) out.normals.assign(3 * n, 0.0);
  if (L.colors) out.colors.assign(3 * n, 0.0);
  if (L.texcoords) out.texcoords.assign(2 * n, 0.0);
  for (size_t i = 0; i < n; i++) {
    const unsigned char* r = base + i * L.stride;
    for (int k = 0; k < 3; k++) {
      if (L.pos[k] >= 0) out.vertices[3 * i + k] = scalar(r + L.pos[k], L.pos_t[k]);
      if (L.normals && L.nrm[k] >= 0) out.normals[3 * i + k] = scalar(r + L.nrm[k], L.nrm_t[k]);
      if (L.colors && L.col[k] >= 0) {
        double v = scalar(r + L.col[k], L.col_t[k]);
        bool byte = L.col_t[k] == "uchar" || L.col_t[k] == "uint8";
        out.colors[3 * i + k] = byte ? v / 255.0 : v;
      }
    }
    for (int k = 0; k < 2; k++)
      if (L.texcoords && L.tex[k] >= 0) out.texcoords[2 * i + k] = scalar(r + L.tex[k], L.tex_t[k]);
  }
}

// Skips one property value (a scalar, or a uchar-counted list).
void skip(Cursor& c, const Property& p, const char* what) {
  if (!p.list) {
    int sz = scalar_size(p.type);
    if (!sz) throw Failure{"failed to read PLY data: unsupported data type: " + p.type};
    c.take((size_t)sz, what);
    return;
  }
  if (p.count_type != "uchar" && p.count_type != "uint8")
    throw Failure{"failed to read PLY data: unsupported list count type: " + p.count_type};
  int isz = scalar_size(p.item_type);
  if (!isz) throw Failure{"failed to read PLY data: unsupported data type: " + p.item_type};
  size_t k = *c.take(1, what);
  c.take(k * (size_t)isz, what);
}

void read_faces(Cursor& c, const Element& el, gprt_ply& out) {
  out.indices.reserve((size_t)std::min<uint64_t>(3 * el.count, (c.n - c.at) / 4));
  for (uint64_t f = 0; f < el.count; f++) {
    for (const Property& p : el.props) {
      if (!(p.list && p.name == "vertex_indices")) {
        skip(c, p, "failed to skip face property");
        continue;
      }
      uint64_t n;
      if (p.count_type == "uchar" || p.count_type == "uint8") n = *c.take(1, "failed to read face vertex count");
      else if (p.count_type == "int" || p.count_type == "int32")
        n = (uint64_t)(int64_t)(int32_t)load_le(c.take(4, "failed to read face vertex count"), 4);
      else throw Failure{"failed to read PLY data: unsupported list count type: " + p.count_type};
      if (n != 3)
        throw Failure{"failed to read PLY data: only triangular faces supported, got " +
                      std::to_string((int64_t)n) + " vertices at face " + std::to_string(f)};
      bool sgn = p.item_type == "int" || p.item_type == "int32";
      if (!sgn && p.item_type != "uint" && p.item_type != "uint32")
        throw Failure{"failed to read PLY data: unsupported face index data type: " + p.item_type};
      const unsigned char* b = c.take(12, "failed to read face indices");
      for (int k = 0; k < 3; k++) {
        uint32_t w = (uint32_t)load_le(b + 4 * k, 4);
        int64_t idx = sgn ? (int64_t)(int32_t)w : (int64_t)w;
        if (idx < 0 || (uint64_t)idx >= out.info.n_vertices)
          throw Failure{"failed to read PLY data: vertex index out of range at face " + std::to_string(f) + ": " +
                        std::to_string(idx) + " of " + std::to_string(out.info.n_vertices) + " vertices"};
        out.indices.push_back((uint32_t)idx);
      }
    }
  }
}

std::unique_ptr<gprt_ply> load(const char* path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw Failure{std::string("failed to open PLY file: ") + path + ": no such file or not readable"};
  std::ostringstream ss;
  ss << in.rdbuf();
  const std::string file = ss.str();
  Header h = read_header(file);
  if (h.format == "binary_big_endian") throw Failure{"binary big-endian PLY format not yet implemented"};
  if (h.format == "ascii") throw Failure{"ASCII PLY format not yet supported"};
  if (h.format != "binary_little_endian") throw Failure{"unsupported PLY format: " + h.format};
  auto out = std::make_unique<gprt_ply>();
  Cursor c{reinterpret_cast<const unsigned char*>(file.data()), file.size(), h.body};
  bool have_vertices = false;
  for (const Element& el : h.elements) {
    if (el.name == "vertex") {
      read_vertices(c, el, *out);
      out->info.n_vertices = (uint32_t)el.count;
      have_vertices = true;
    } else if (el.name == "face") {
      if (!have_vertices && el.count) throw Failure{"failed to read PLY data: faces before vertices"};
      read_faces(c, el, *out);
    } else {
      for (uint64_t k = 0; k < el.count; k++)
        for (const Property& p : el.props) skip(c, p, "failed to skip element");
    }
  }
  gprt_ply_info& info = out->info;
  info.n_triangles = (uint32_t)(out->indices.size() / 3);
  info.has_normals = out->normals.empty() ? 0u : 1u;
  info.has_colors = out->colors.empty() ? 0u : 1u;
  info.has_texcoords = out->texcoords.empty() ? 0u : 1u;
  return out;
}

}  // namespace
}  // namespace ply
}  // namespace gprt

extern "C" {

int gprt_ply_load(const char* path, gprt_ply** out, char* errbuf, size_t err_len) {
  if (!path || !out) return GPRT_E_INVALID;
  *out = nullptr;
  try {
    *out = gprt::ply::load(path).release();
    return GPRT_OK;
  } catch (const gprt::ply::Failure& f) {
    if (errbuf && err_len) std::snprintf(errbuf, err_len, "%s", f.msg.c_str());
  } catch (const std::exception& e) {
    if (errbuf && err_len) std::snprintf(errbuf, err_len, "%s", e.what());
  }
  return GPRT_E_INVALID;
}

int gprt_ply_get(const gprt_ply* p, gprt_ply_info* info, const double** vertices, const uint32_t** indices,
                 const double** normals, const double** colors, const double** texcoords) {
  if (!p) return GPRT_E_INVALID;
  auto ptr = [](const auto& v) { return v.empty() ? nullptr : v.data(); };
  if (info) *info = p->info;
  if (vertices) *vertices = ptr(p->vertices);
  if (indices) *indices = ptr(p->indices);
  if (normals) *normals = ptr(p->normals);
  if (colors) *colors = ptr(p->colors);
  if (texcoords) *texcoords = ptr(p->texcoords);
  return GPRT_OK;
}

void gprt_ply_free(gprt_ply* p) { delete p; }

}  // extern "C"
