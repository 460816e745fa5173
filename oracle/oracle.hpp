// oracle.hpp - CPU restatement (C++17, float64) of go-progressive-raytracer's
// rendering hot path.  TEST INFRASTRUCTURE ONLY: this code is the checker for
// the GB300 library; only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline use it, and the product never links or calls it.
//
// Every function follows the reference Go code cited beside it (paths are
// relative to the reference project root).  Arithmetic is float64 like the
// reference (core.Vec3, pkg/core/vec3.go:9-11).  The only deliberate
// difference is the random source: the reference draws from Go's math/rand,
// whose source is not available here, so the oracle's samplers are a PCG32
// stream per 64x64 tile (consumed in the reference's order) and the injected
// test sampler of pkg/integrator/bdpt_test.go:17-74.  Parity of rendered
// images is therefore statistical; parity of every deterministic function is
// pinned by the reference's own known-answer tests (oracle/kat.cpp).
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace ref {

constexpr double kPi = 3.14159265358979323846;
constexpr double kInf = std::numeric_limits<double>::infinity();

// ---------------------------------------------------------------------------
// core.Vec3 / Vec2 / Ray  (pkg/core/vec3.go:9-218)
// ---------------------------------------------------------------------------
struct Vec2 {
  double x = 0, y = 0;
  Vec2() = default;
  Vec2(double a, double b) : x(a), y(b) {}
  Vec2 add(Vec2 o) const { return {x + o.x, y + o.y}; }
  Vec2 mul(double s) const { return {x * s, y * s}; }
};

struct Vec3 {
  double x = 0, y = 0, z = 0;
  Vec3() = default;
  Vec3(double a, double b, double c) : x(a), y(b), z(c) {}
  Vec3 add(const Vec3& o) const { return {x + o.x, y + o.y, z + o.z}; }
  Vec3 sub(const Vec3& o) const { return {x - o.x, y - o.y, z - o.z}; }
  Vec3 mul(double s) const { return {x * s, y * s, z * s}; }
  double length() const { return std::sqrt(x * x + y * y + z * z); }
  double lengthSquared() const { return x * x + y * y + z * z; }
  double dot(const Vec3& o) const { return x * o.x + y * o.y + z * o.z; }
  double absDot(const Vec3& o) const { return std::fabs(dot(o)); }
  // Clamp (vec3.go:78-84)
  Vec3 clamp(double lo, double hi) const {
    return {std::max(lo, std::min(hi, x)), std::max(lo, std::min(hi, y)),
            std::max(lo, std::min(hi, z))};
  }
  // GammaCorrect (vec3.go:87-94)
  Vec3 gammaCorrect(double gamma) const {
    double inv = 1.0 / gamma;
    return {std::pow(x, inv), std::pow(y, inv), std::pow(z, inv)};
  }
  // Normalize (vec3.go:97-103): zero vector stays zero
  Vec3 normalize() const {
    double l = length();
    if (l == 0) return {0, 0, 0};
    return {x / l, y / l, z / l};
  }
  Vec3 cross(const Vec3& o) const {
    return {y * o.z - z * o.y, z * o.x - x * o.z, x * o.y - y * o.x};
  }
  Vec3 mulVec(const Vec3& o) const { return {x * o.x, y * o.y, z * o.z}; }
  // Luminance (vec3.go:134-136)
  double luminance() const { return 0.2126 * x + 0.7152 * y + 0.0722 * z; }
  bool isZero() const { return x == 0 && y == 0 && z == 0; }
  Vec3 negate() const { return {-x, -y, -z}; }
  double axis(int a) const { return a == 0 ? x : (a == 1 ? y : z); }
  // Rotate X -> Y -> Z (vec3.go:162-198)
  Vec3 rotate(const Vec3& r) const {
    if (r.x == 0 && r.y == 0 && r.z == 0) return *this;
    Vec3 v = *this;
    if (r.x != 0) {
      double c = std::cos(r.x), s = std::sin(r.x);
      double ny = v.y * c - v.z * s, nz = v.y * s + v.z * c;
      v = {v.x, ny, nz};
    }
    if (r.y != 0) {
      double c = std::cos(r.y), s = std::sin(r.y);
      double nx = v.x * c + v.z * s, nz = -v.x * s + v.z * c;
      v = {nx, v.y, nz};
    }
    if (r.z != 0) {
      double c = std::cos(r.z), s = std::sin(r.z);
      double nx = v.x * c - v.y * s, ny = v.x * s + v.y * c;
      v = {nx, ny, v.z};
    }
    return v;
  }
};

struct Ray {
  Vec3 origin, direction;
  Ray() = default;
  Ray(const Vec3& o, const Vec3& d) : origin(o), direction(d) {}
  Vec3 at(double t) const { return origin.add(direction.mul(t)); }  // vec3.go:216-218
};
// core.NewRayTo (vec3.go:211-213)
inline Ray rayTo(const Vec3& o, const Vec3& target) { return Ray(o, target.sub(o).normalize()); }

// ---------------------------------------------------------------------------
// core.Sampler (pkg/core/sampling.go:10-14) and the oracle's sources
// ---------------------------------------------------------------------------
struct Sampler {
  virtual ~Sampler() = default;
  virtual double get1D() = 0;
  virtual Vec2 get2D() = 0;
  virtual Vec3 get3D() = 0;
};

// PCG32 (O'Neill 2014, "PCG: A Family of Simple Fast Space-Efficient
// Statistically Good Algorithms for Random Number Generation"), XSH-RR output.
// Stands in for the per-tile *rand.Rand of progressive.go:444 and is consumed
// in the same order as RandomSampler (sampling.go:17-39).
struct PcgSampler : Sampler {
  uint64_t state = 0, inc = 1;
  PcgSampler(uint64_t seed, uint64_t stream) {
    inc = (stream << 1u) | 1u;
    state = 0;
    next();
    state += seed;
    next();
  }
  uint32_t next() {
    uint64_t old = state;
    state = old * 6364136223846793005ULL + inc;
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
  }
  // 53-bit double in [0,1) from two outputs (Float64 semantics of math/rand)
  double get1D() override {
    uint64_t hi = next(), lo = next();
    uint64_t v = ((hi << 32) | lo) >> 11;
    return (double)v * (1.0 / 9007199254740992.0);
  }
  Vec2 get2D() override {
    double a = get1D();
    double b = get1D();
    return {a, b};
  }
  Vec3 get3D() override {
    double a = get1D();
    double b = get1D();
    double c = get1D();
    return {a, b, c};
  }
};

// The GPU library's counter-based stream for one pixel sample: draw k is
// word k % 4 of pcg4d(pixel, sample, k / 4, seed word) (Jarzynski & Olano,
// "Hash Functions for GPU Rendering", JCGT 9(3), 2020), the seed word being
// fmix32(seed_lo ^ fmix32(seed_hi ^ 0x9e3779b9)) (MurmurHash3's finalizer),
// mapped to [0,1) as (word >> 8) * 2^-24.  Consumed in the reference's order,
// it gives the oracle the same inputs as the GPU for per-sample comparisons.
struct CounterSampler : Sampler {
  uint32_t k0, k1, k3, pos = 0;
  uint32_t buf[4] = {0, 0, 0, 0};
  static uint32_t fmix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
  }
  CounterSampler(uint64_t seed, uint32_t pixel, uint32_t sample)
      : k0(pixel), k1(sample), k3(fmix32((uint32_t)seed ^ fmix32((uint32_t)(seed >> 32) ^ 0x9e3779b9u))) {}
  static void pcg4d(uint32_t v[4]) {
    for (int i = 0; i < 4; i++) v[i] = v[i] * 1664525u + 1013904223u;
    v[0] += v[1] * v[3];
    v[1] += v[2] * v[0];
    v[2] += v[0] * v[1];
    v[3] += v[1] * v[2];
    for (int i = 0; i < 4; i++) v[i] ^= v[i] >> 16;
    v[0] += v[1] * v[3];
    v[1] += v[2] * v[0];
    v[2] += v[0] * v[1];
    v[3] += v[1] * v[2];
  }
  double get1D() override {
    uint32_t lane = pos & 3u;
    if (lane == 0) {
      buf[0] = k0;
      buf[1] = k1;
      buf[2] = pos >> 2;
      buf[3] = k3;
      pcg4d(buf);
    }
    pos++;
    return (double)(buf[lane] >> 8) * (1.0 / 16777216.0);
  }
  Vec2 get2D() override {
    double a = get1D();
    double b = get1D();
    return {a, b};
  }
  Vec3 get3D() override {
    double a = get1D();
    double b = get1D();
    double c = get1D();
    return {a, b, c};
  }
};

// TestSampler (pkg/integrator/bdpt_test.go:17-74): predetermined values.
struct ListSampler : Sampler {
  std::vector<double> v1;
  std::vector<Vec2> v2;
  std::vector<Vec3> v3;
  size_t i1 = 0, i2 = 0, i3 = 0;
  ListSampler(std::vector<double> a, std::vector<Vec2> b, std::vector<Vec3> c)
      : v1(std::move(a)), v2(std::move(b)), v3(std::move(c)) {}
  double get1D() override {
    if (i1 >= v1.size()) throw std::runtime_error("TestSampler ran out of 1D values");
    return v1[i1++];
  }
  Vec2 get2D() override {
    if (i2 >= v2.size()) throw std::runtime_error("TestSampler ran out of 2D values");
    return v2[i2++];
  }
  Vec3 get3D() override {
    if (i3 >= v3.size()) throw std::runtime_error("TestSampler ran out of 3D values");
    return v3[i3++];
  }
  void reset() { i1 = i2 = i3 = 0; }
};

// ---------------------------------------------------------------------------
// Sampling warps (pkg/core/sampling.go:42-147)
// ---------------------------------------------------------------------------
// SampleCosineHemisphere (sampling.go:42-67)
inline Vec3 sampleCosineHemisphere(const Vec3& normal, Vec2 s) {
  double a = 2.0 * kPi * s.x;
  double z = s.y;
  double r = std::sqrt(z);
  double x = r * std::cos(a);
  double y = r * std::sin(a);
  double zc = std::sqrt(1.0 - z);
  Vec3 nt = std::fabs(normal.x) > 0.1 ? Vec3(0, 1, 0) : Vec3(1, 0, 0);
  Vec3 tangent = nt.cross(normal).normalize();
  Vec3 bitangent = normal.cross(tangent);
  return tangent.mul(x).add(bitangent.mul(y)).add(normal.mul(zc));
}
// SampleCone (sampling.go:70-94)
inline Vec3 sampleCone(const Vec3& direction, double cosTotalWidth, Vec2 s) {
  Vec3 w = direction;
  Vec3 u = std::fabs(w.x) > 0.1 ? Vec3(0, 1, 0) : Vec3(1, 0, 0);
  u = u.cross(w).normalize();
  Vec3 v = w.cross(u);
  double cosTheta = 1.0 - s.x * (1.0 - cosTotalWidth);
  double sinTheta = std::sqrt(std::max(0.0, 1.0 - cosTheta * cosTheta));
  double phi = 2.0 * kPi * s.y;
  return u.mul(sinTheta * std::cos(phi)).add(v.mul(sinTheta * std::sin(phi))).add(w.mul(cosTheta));
}
// SampleOnUnitSphere (sampling.go:97-104)
inline Vec3 sampleOnUnitSphere(Vec2 s) {
  double z = 1.0 - 2.0 * s.x;
  double r = std::sqrt(std::max(0.0, 1.0 - z * z));
  double phi = 2.0 * kPi * s.y;
  return {r * std::cos(phi), r * std::sin(phi), z};
}
// SamplePointInUnitDisk, concentric mapping (sampling.go:108-126)
inline Vec3 samplePointInUnitDisk(Vec2 s) {
  Vec2 u(2 * s.x - 1, 2 * s.y - 1);
  if (u.x == 0 && u.y == 0) return {0, 0, 0};
  double theta, r;
  if (std::fabs(u.x) > std::fabs(u.y)) {
    r = u.x;
    theta = kPi / 4 * (u.y / u.x);
  } else {
    r = u.y;
    theta = kPi / 2 - kPi / 4 * (u.x / u.y);
  }
  return {r * std::cos(theta), r * std::sin(theta), 0};
}
// SamplePointInUnitSphere (sampling.go:130-147)
inline Vec3 samplePointInUnitSphere(Vec3 s) {
  double r = std::pow(s.x, 1.0 / 3.0);
  double phi = 2 * kPi * s.y;
  double cosTheta = 2 * s.z - 1;
  double sinTheta = std::sqrt(1 - cosTheta * cosTheta);
  return {r * sinTheta * std::cos(phi), r * sinTheta * std::sin(phi), r * cosTheta};
}

// ---------------------------------------------------------------------------
// Materials (pkg/material/*.go)
// ---------------------------------------------------------------------------
enum class TransportMode { Radiance, Importance };  // interfaces.go:9-14
struct Material;

// SurfaceInteraction (interfaces.go:48-65).  shape/sub are instrumentation
// (index in scene.Shapes and box face / mesh triangle) used by parity tests.
struct SurfaceInteraction {
  Vec3 point, normal;
  double t = 0;
  bool frontFace = false;
  const Material* material = nullptr;
  Vec2 uv;
  int shape = -1, sub = 0;
  // SetFaceNormal (interfaces.go:58-65)
  void setFaceNormal(const Ray& ray, const Vec3& outward) {
    frontFace = ray.direction.dot(outward) < 0;
    normal = frontFace ? outward : outward.mul(-1);
  }
};

// ScatterResult (interfaces.go:35-45)
struct ScatterResult {
  Ray incoming, scattered;
  Vec3 attenuation;
  double pdf = 0;
  bool isSpecular() const { return pdf <= 0; }
};

struct Material {
  virtual ~Material() = default;
  virtual bool scatter(const Ray& in, const SurfaceInteraction& hit, Sampler& s,
                       ScatterResult& out) const = 0;
  virtual Vec3 evaluateBRDF(const Vec3& in, const Vec3& out, const SurfaceInteraction* hit,
                            TransportMode mode) const = 0;
  // returns pdf, sets isDelta
  virtual double pdf(const Vec3& in, const Vec3& out, const Vec3& normal, bool& isDelta) const = 0;
  // Emitter interface (interfaces.go:30-32)
  virtual bool isEmitter() const { return false; }
  virtual Vec3 emit(const Ray&, const SurfaceInteraction*) const { return {}; }
};

// reflect (metal.go:87-90; dielectric.go:152-155)
inline Vec3 reflectVec(const Vec3& v, const Vec3& n) { return v.sub(n.mul(2 * v.dot(n))); }
// refractVector (dielectric.go:158-163)
inline Vec3 refractVec(const Vec3& uv, const Vec3& n, double etaiOverEtat) {
  double cosTheta = std::min(-uv.dot(n), 1.0);
  Vec3 perp = uv.add(n.mul(cosTheta)).mul(etaiOverEtat);
  Vec3 par = n.mul(-std::sqrt(std::fabs(1.0 - perp.lengthSquared())));
  return perp.add(par);
}
// Reflectance, Schlick (dielectric.go:166-172)
inline double reflectance(double cosine, double ratio) {
  double r0 = (1 - ratio) / (1 + ratio);
  r0 = r0 * r0;
  return r0 + (1 - r0) * std::pow(1 - cosine, 5);
}

// Lambertian with SolidColor albedo (lambertian.go:25-72, color_source.go)
// ImageTexture.Evaluate (image_texture.go:25-52): wrap u and v into [0,1),
// nearest texel with v = 0 at the bottom row, clamped to the image
struct ImageTexture {
  int width = 0, height = 0;
  std::vector<Vec3> pixels;  // row-major, pixels[y * width + x]
  Vec3 evaluate(Vec2 uv) const {
    double u = uv.x - (double)(long long)uv.x, v = uv.y - (double)(long long)uv.y;
    if (u < 0) u += 1.0;
    if (v < 0) v += 1.0;
    long long x = (long long)(u * width), y = (long long)((1.0 - v) * height);
    if (x >= width) x = width - 1;
    if (y >= height) y = height - 1;
    if (x < 0) x = 0;
    if (y < 0) y = 0;
    return pixels[(size_t)y * width + x];
  }
};

// Lambertian (lambertian.go:10-72); the albedo may be a texture
// (NewTexturedLambertian) evaluated at the hit's UV
struct Lambertian : Material {
  Vec3 albedo;
  const ImageTexture* tex = nullptr;
  explicit Lambertian(Vec3 a, const ImageTexture* t = nullptr) : albedo(a), tex(t) {}
  Vec3 albedoAt(const SurfaceInteraction& h) const { return tex ? tex->evaluate(h.uv) : albedo; }
  bool scatter(const Ray& in, const SurfaceInteraction& hit, Sampler& s,
               ScatterResult& out) const override {
    Vec3 dir = sampleCosineHemisphere(hit.normal, s.get2D());
    double c = dir.normalize().dot(hit.normal);
    if (c < 0) c = 0;
    out.incoming = in;
    out.scattered = Ray(hit.point, dir);
    out.attenuation = albedoAt(hit).mul(1.0 / kPi);
    out.pdf = c / kPi;
    return true;
  }
  Vec3 evaluateBRDF(const Vec3&, const Vec3& out, const SurfaceInteraction* hit,
                    TransportMode) const override {
    if (out.dot(hit->normal) <= 0) return {};
    return albedoAt(*hit).mul(1.0 / kPi);
  }
  double pdf(const Vec3&, const Vec3& out, const Vec3& n, bool& isDelta) const override {
    isDelta = false;
    double c = out.dot(n);
    if (c <= 0) return 0.0;
    return c / kPi;
  }
};

// Metal (metal.go:18-90); NewMetal clamps fuzz to [0,1]
struct Metal : Material {
  Vec3 albedo;
  double fuzz;
  const ImageTexture* tex = nullptr;  // NewTexturedMetal (metal.go:25-36)
  Metal(Vec3 a, double f, const ImageTexture* t = nullptr) : albedo(a), fuzz(std::min(1.0, std::max(0.0, f))), tex(t) {}
  Vec3 albedoAt(const SurfaceInteraction& h) const { return tex ? tex->evaluate(h.uv) : albedo; }
  bool scatter(const Ray& in, const SurfaceInteraction& hit, Sampler& s,
               ScatterResult& out) const override {
    Vec3 r = reflectVec(in.direction.normalize(), hit.normal);
    if (fuzz > 0) r = r.add(samplePointInUnitSphere(s.get3D()).mul(fuzz));
    out.incoming = in;
    out.scattered = Ray(hit.point, r);
    out.attenuation = albedoAt(hit);
    out.pdf = 0;
    return out.scattered.direction.dot(hit.normal) > 0;
  }
  Vec3 evaluateBRDF(const Vec3& in, const Vec3& out, const SurfaceInteraction* hit,
                    TransportMode) const override {
    Vec3 r = reflectVec(in.negate(), hit->normal);
    if (out.sub(r).length() < 0.001) return albedoAt(*hit);
    return {};
  }
  double pdf(const Vec3&, const Vec3&, const Vec3&, bool& isDelta) const override {
    isDelta = true;
    return 0.0;
  }
};

// Dielectric (dielectric.go:20-149)
struct Dielectric : Material {
  double ior;
  explicit Dielectric(double i) : ior(i) {}
  bool scatter(const Ray& in, const SurfaceInteraction& hit, Sampler& s,
               ScatterResult& out) const override {
    double ratio = hit.frontFace ? 1.0 / ior : ior;
    Vec3 unit = in.direction.normalize();
    double cosTheta = std::min(-unit.dot(hit.normal), 1.0);
    double sinTheta = std::sqrt(1.0 - cosTheta * cosTheta);
    bool cannotRefract = ratio * sinTheta > 1.0;
    Vec3 dir;
    // Go's || short-circuits: no sample is drawn under total internal reflection
    if (cannotRefract || reflectance(cosTheta, ratio) > s.get1D())
      dir = reflectVec(unit, hit.normal);
    else
      dir = refractVec(unit, hit.normal, ratio);
    out.incoming = in;
    out.scattered = Ray(hit.point, dir);
    out.attenuation = Vec3(1, 1, 1);
    out.pdf = 0;
    return true;
  }
  Vec3 evaluateBRDF(const Vec3& inDir, const Vec3& outDir, const SurfaceInteraction* hit,
                    TransportMode mode) const override {
    Vec3 wi = inDir.normalize(), wo = outDir.normalize(), n = hit->normal.normalize();
    double wiN = wi.dot(n), woN = wo.dot(n);
    bool same = (wiN > 0) == (woN > 0);
    if (!same) {
      Vec3 r = reflectVec(wi, n);
      if (wo.sub(r).length() < 0.001) {
        double ratio = hit->frontFace ? 1.0 / ior : ior;
        double f = reflectance(std::fabs(wiN), ratio);
        return {f, f, f};
      }
    } else {
      double ratio = hit->frontFace ? 1.0 / ior : ior;
      double cosTheta = std::fabs(wiN);
      Vec3 refr = refractVec(wi, n, ratio);
      if (wo.sub(refr).length() < 0.001) {
        double tr = 1.0 - reflectance(cosTheta, ratio);
        if (mode == TransportMode::Radiance) {
          double etap = hit->frontFace ? ior : 1.0 / ior;
          tr /= etap * etap;
        }
        return {tr, tr, tr};
      }
    }
    return {};
  }
  double pdf(const Vec3&, const Vec3&, const Vec3&, bool& isDelta) const override {
    isDelta = true;
    return 0.0;
  }
};

// Emissive (emissive.go:17-44): emits from the front face only
struct Emissive : Material {
  Vec3 emission;
  explicit Emissive(Vec3 e) : emission(e) {}
  bool scatter(const Ray&, const SurfaceInteraction&, Sampler&, ScatterResult&) const override {
    return false;
  }
  Vec3 evaluateBRDF(const Vec3&, const Vec3&, const SurfaceInteraction*,
                    TransportMode) const override {
    return {};
  }
  double pdf(const Vec3&, const Vec3&, const Vec3&, bool& isDelta) const override {
    isDelta = false;
    return 0.0;
  }
  bool isEmitter() const override { return true; }
  Vec3 emit(const Ray&, const SurfaceInteraction* hit) const override {
    if (hit != nullptr && !hit->frontFace) return {};
    return emission;
  }
};

// discSpotLightMaterial (disc_spot_light.go:13-62): emits its base emission
// from the front face, and only towards rays travelling against the spot
// direction (cosine with it below -0.3, the ray direction as given)
struct SpotEmissive : Material {
  Vec3 emission, direction;
  SpotEmissive(Vec3 e, Vec3 d) : emission(e), direction(d) {}
  bool scatter(const Ray&, const SurfaceInteraction&, Sampler&, ScatterResult&) const override { return false; }
  Vec3 evaluateBRDF(const Vec3&, const Vec3&, const SurfaceInteraction*, TransportMode) const override { return {}; }
  double pdf(const Vec3&, const Vec3&, const Vec3&, bool& isDelta) const override {
    isDelta = false;
    return 0.0;
  }
  bool isEmitter() const override { return true; }
  Vec3 emit(const Ray& r, const SurfaceInteraction* hit) const override {
    if (hit != nullptr && !hit->frontFace) return {};
    if (r.direction.dot(direction) > -0.3) return {};
    return emission;
  }
};

// isReflectionPath (layered.go:110-119)
inline bool isReflectionPath(const Vec3& in, const Vec3& out, const Vec3& n) {
  Vec3 inc = in.negate();
  Vec3 r = inc.sub(n.mul(2 * inc.dot(n)));
  return out.sub(r).length() < 0.1;
}

// Layered (layered.go:24-119)
struct Layered : Material {
  const Material* outer;
  const Material* inner;
  Layered(const Material* o, const Material* i) : outer(o), inner(i) {}
  bool scatter(const Ray& in, const SurfaceInteraction& hit, Sampler& s,
               ScatterResult& out) const override {
    SurfaceInteraction oh = hit;
    oh.material = outer;
    ScatterResult orr;
    if (!outer->scatter(in, oh, s, orr)) return false;
    Vec3 sd = orr.scattered.direction.normalize();
    if (!(sd.dot(hit.normal) < 0)) {
      out = orr;
      return true;
    }
    Ray innerRay(hit.point, sd);
    SurfaceInteraction ih = hit;
    ih.material = inner;
    ScatterResult ir;
    if (!inner->scatter(innerRay, ih, s, ir)) {
      out = orr;
      return true;
    }
    out.incoming = in;
    out.scattered = ir.scattered;
    out.attenuation = orr.attenuation.mulVec(ir.attenuation);
    out.pdf = ir.pdf;
    return true;
  }
  Vec3 evaluateBRDF(const Vec3& in, const Vec3& out, const SurfaceInteraction* hit,
                    TransportMode mode) const override {
    if (isReflectionPath(in, out, hit->normal)) return outer->evaluateBRDF(in, out, hit, mode);
    return inner->evaluateBRDF(in, out, hit, mode);
  }
  double pdf(const Vec3& in, const Vec3& out, const Vec3& n, bool& isDelta) const override {
    bool d;
    double p = isReflectionPath(in, out, n) ? outer->pdf(in, out, n, d) : inner->pdf(in, out, n, d);
    isDelta = false;
    return p;
  }
};

// Mix (mix.go:9-59): one uniform number picks the material that scatters
// (material 2 below the ratio); BRDF and pdf are the ratio-weighted blends,
// never delta
struct Mix : Material {
  const Material* m1;
  const Material* m2;
  double ratio;
  Mix(const Material* a, const Material* b, double r) : m1(a), m2(b), ratio(std::max(0.0, std::min(r, 1.0))) {}
  bool scatter(const Ray& in, const SurfaceInteraction& hit, Sampler& s, ScatterResult& out) const override {
    if (s.get1D() < ratio) return m2->scatter(in, hit, s, out);
    return m1->scatter(in, hit, s, out);
  }
  Vec3 evaluateBRDF(const Vec3& in, const Vec3& out, const SurfaceInteraction* hit,
                    TransportMode mode) const override {
    return m1->evaluateBRDF(in, out, hit, mode).mul(1.0 - ratio).add(m2->evaluateBRDF(in, out, hit, mode).mul(ratio));
  }
  double pdf(const Vec3& in, const Vec3& out, const Vec3& n, bool& isDelta) const override {
    bool d;
    double p1 = m1->pdf(in, out, n, d), p2 = m2->pdf(in, out, n, d);
    isDelta = false;
    return p1 * (1.0 - ratio) + p2 * ratio;
  }
};

// ---------------------------------------------------------------------------
// Geometry (pkg/geometry)
// ---------------------------------------------------------------------------
// Work counters of the instrumented traversal (per thread).
struct TraversalCounters {
  uint64_t aabb = 0, prims = 0;
};
inline TraversalCounters& counters() {
  static thread_local TraversalCounters c;
  return c;
}

// AABB (aabb.go:27-171)
struct AABB {
  Vec3 min, max;
  AABB() = default;
  AABB(Vec3 a, Vec3 b) : min(a), max(b) {}
  static AABB fromPoints(const std::vector<Vec3>& pts) {  // NewAABBFromPoints (aabb.go:38-57)
    if (pts.empty()) return {};
    Vec3 mn = pts[0], mx = pts[0];
    for (size_t i = 1; i < pts.size(); i++) {
      mn = {std::min(mn.x, pts[i].x), std::min(mn.y, pts[i].y), std::min(mn.z, pts[i].z)};
      mx = {std::max(mx.x, pts[i].x), std::max(mx.y, pts[i].y), std::max(mx.z, pts[i].z)};
    }
    return {mn, mx};
  }
  // Hit, slab method with the |d|<1e-8 parallel case (aabb.go:43-95)
  bool hit(const Ray& r, double tMin, double tMax) const {
    counters().aabb++;
    for (int a = 0; a < 3; a++) {
      double mn = min.axis(a), mx = max.axis(a), o = r.origin.axis(a), d = r.direction.axis(a);
      if (std::fabs(d) < 1e-8) {
        if (o < mn || o > mx) return false;
        continue;
      }
      double inv = 1.0 / d;
      double t1 = (mn - o) * inv, t2 = (mx - o) * inv;
      if (t1 > t2) std::swap(t1, t2);
      tMin = std::max(tMin, t1);
      tMax = std::min(tMax, t2);
      if (tMin > tMax) return false;
    }
    return true;
  }
  AABB unite(const AABB& o) const {  // Union (aabb.go:98-111)
    return {{std::min(min.x, o.min.x), std::min(min.y, o.min.y), std::min(min.z, o.min.z)},
            {std::max(max.x, o.max.x), std::max(max.y, o.max.y), std::max(max.z, o.max.z)}};
  }
  Vec3 center() const { return min.add(max).mul(0.5); }
  Vec3 size() const { return max.sub(min); }
  int longestAxis() const {  // aabb.go:130-139
    Vec3 s = size();
    if (s.x > s.y && s.x > s.z) return 0;
    if (s.y > s.z) return 1;
    return 2;
  }
};

// Shape interface (interfaces.go:9-12)
struct Shape {
  int id = -1;  // index in scene.Shapes (instrumentation)
  virtual ~Shape() = default;
  virtual bool hit(const Ray& r, double tMin, double tMax, SurfaceInteraction& out) const = 0;
  virtual AABB boundingBox() const = 0;
};

// Sphere (sphere.go:27-90)
struct Sphere : Shape {
  Vec3 center;
  double radius;
  const Material* material;
  Sphere(Vec3 c, double r, const Material* m) : center(c), radius(r), material(m) {}
  bool hit(const Ray& ray, double tMin, double tMax, SurfaceInteraction& out) const override {
    counters().prims++;
    Vec3 oc = ray.origin.sub(center);
    double a = ray.direction.dot(ray.direction);
    double halfB = oc.dot(ray.direction);
    double c = oc.dot(oc) - radius * radius;
    double disc = halfB * halfB - a * c;
    if (disc < 0) return false;
    double sq = std::sqrt(disc);
    double root = (-halfB - sq) / a;
    if (root < tMin || root > tMax) {
      root = (-halfB + sq) / a;
      if (root < tMin || root > tMax) return false;
    }
    Vec3 p = ray.at(root);
    Vec3 on = p.sub(center).mul(1.0 / radius);
    double theta = std::acos(-on.y);
    double phi = std::atan2(-on.z, on.x) + kPi;
    out = SurfaceInteraction();
    out.t = root;
    out.point = p;
    out.material = material;
    out.uv = Vec2(phi / (2.0 * kPi), theta / kPi);
    out.shape = id;
    out.sub = 0;
    out.setFaceNormal(ray, on);
    return true;
  }
  AABB boundingBox() const override {
    Vec3 r(radius, radius, radius);
    return {center.sub(r), center.add(r)};
  }
};

// Quad (quad.go:109-210)
struct Quad : Shape {
  Vec3 corner, u, v, normal, w;
  double d;
  const Material* material;
  int subIndex = 0;  // box face index (instrumentation)
  Quad(Vec3 c, Vec3 uu, Vec3 vv, const Material* m) : corner(c), u(uu), v(vv), material(m) {
    normal = u.cross(v).normalize();
    d = normal.dot(corner);
    Vec3 cr = u.cross(v);
    w = normal.mul(1.0 / normal.dot(cr));
  }
  bool hit(const Ray& ray, double tMin, double tMax, SurfaceInteraction& out) const override {
    counters().prims++;
    double den = ray.direction.dot(normal);
    if (std::fabs(den) < 1e-8) return false;
    double t = (d - ray.origin.dot(normal)) / den;
    if (t < tMin || t > tMax) return false;
    Vec3 p = ray.at(t);
    Vec3 hv = p.sub(corner);
    double alpha = w.dot(hv.cross(v));
    double beta = w.dot(u.cross(hv));
    if (alpha < 0 || alpha > 1 || beta < 0 || beta > 1) return false;
    out = SurfaceInteraction();
    out.t = t;
    out.point = p;
    out.material = material;
    out.uv = Vec2(alpha, beta);
    out.shape = id;
    out.sub = subIndex;
    out.setFaceNormal(ray, normal);
    return true;
  }
  // getAxisAlignment (quad.go:21-41) + createAxisAlignedAABB (quad.go:44-77)
  AABB boundingBox() const override {
    std::vector<Vec3> cs = {corner, corner.add(u), corner.add(v), corner.add(u).add(v)};
    const double th = 0.9999, tol = 0.0001, eps = 0.001;
    int al = 0;
    if (std::fabs(normal.x) > th && std::fabs(normal.y) < tol && std::fabs(normal.z) < tol) al = 1;
    else if (std::fabs(normal.y) > th && std::fabs(normal.x) < tol && std::fabs(normal.z) < tol) al = 2;
    else if (std::fabs(normal.z) > th && std::fabs(normal.x) < tol && std::fabs(normal.y) < tol) al = 3;
    if (al == 0) return AABB::fromPoints(cs);
    auto mm = [&](int a, double& lo, double& hi) {
      lo = hi = cs[0].axis(a);
      for (int i = 1; i < 4; i++) {
        double val = cs[i].axis(a);
        if (val < lo) lo = val;
        if (val > hi) hi = val;
      }
    };
    double lo0, hi0, lo1, hi1;
    if (al == 1) {
      double f = cs[0].x;
      mm(1, lo0, hi0);
      mm(2, lo1, hi1);
      return {{f - eps, lo0, lo1}, {f + eps, hi0, hi1}};
    } else if (al == 2) {
      double f = cs[0].y;
      mm(0, lo0, hi0);
      mm(2, lo1, hi1);
      return {{lo0, f - eps, lo1}, {hi0, f + eps, hi1}};
    }
    double f = cs[0].z;
    mm(0, lo0, hi0);
    mm(1, lo1, hi1);
    return {{lo0, lo1, f - eps}, {hi0, hi1, f + eps}};
  }
};

// Disc (disc.go:11-134): plane hit with |n.d| < 1e-6 rejected, inside when
// |p - c|^2 <= r^2; UV from the right / up frame of NewDisc
struct Disc : Shape {
  Vec3 center, normal, right, up;
  double radius;
  const Material* material;
  Disc(Vec3 c, Vec3 n, double r, const Material* m) : center(c), radius(r), material(m) {
    normal = n.normalize();
    Vec3 rv = std::fabs(normal.x) > 0.1 ? Vec3(0, 1, 0) : Vec3(1, 0, 0);
    right = rv.cross(normal).normalize();
    up = normal.cross(right).normalize();
  }
  bool hit(const Ray& ray, double tMin, double tMax, SurfaceInteraction& out) const override {
    counters().prims++;
    double den = normal.dot(ray.direction);
    if (std::fabs(den) < 1e-6) return false;
    double t = normal.dot(center.sub(ray.origin)) / den;
    if (t < tMin || t > tMax) return false;
    Vec3 p = ray.at(t);
    Vec3 cp = p.sub(center);
    if (cp.lengthSquared() > radius * radius) return false;
    out = SurfaceInteraction();
    out.t = t;
    out.point = p;
    out.material = material;
    out.uv = Vec2((cp.dot(right) / radius + 1.0) / 2.0, (cp.dot(up) / radius + 1.0) / 2.0);
    out.shape = id;
    out.sub = 0;
    out.setFaceNormal(ray, normal);
    return true;
  }
  AABB boundingBox() const override {  // the four corners centre +- r right +- r up
    Vec3 re = right.mul(radius), ue = up.mul(radius);
    std::vector<Vec3> cs = {center.add(re).add(ue), center.add(re).sub(ue), center.sub(re).add(ue),
                            center.sub(re).sub(ue)};
    return AABB::fromPoints(cs);
  }
};

// UV of a point on a cylinder or cone body (cylinder.go:187-205,
// cone.go:234-253): v = height along the axis / length, u = the angle of the
// radial vector in a basis built from the axis and a reference direction
inline Vec2 axialUV(const Vec3& axis, const Vec3& radial, double h, double height) {
  Vec3 ref = std::fabs(axis.y) < 0.9 ? Vec3(0, 1, 0) : Vec3(1, 0, 0);
  Vec3 tangent = axis.cross(ref).normalize();
  Vec3 bitangent = axis.cross(tangent);
  double u = std::atan2(radial.dot(bitangent), radial.dot(tangent));
  return Vec2((u + kPi) / (2.0 * kPi), h / height);
}
// UV of a point on a cap of outward normal n (cylinder.go:241-255, cone.go:322-339)
inline Vec2 capUV(const Vec3& n, const Vec3& center, double radius, const Vec3& p) {
  Vec3 ref = std::fabs(n.y) < 0.9 ? Vec3(0, 1, 0) : Vec3(1, 0, 0);
  Vec3 tangent = n.cross(ref).normalize();
  Vec3 bitangent = n.cross(tangent);
  Vec3 l = p.sub(center);
  return Vec2((l.dot(tangent) / radius + 1.0) / 2.0, (l.dot(bitangent) / radius + 1.0) / 2.0);
}

// Circular cap shared by Cylinder and Cone (cylinder.go:224-266, cone.go:306-350)
inline bool hit_cap(const Ray& ray, const Vec3& center, const Vec3& normal, double radius, double tMin, double tMax,
                    double& t, Vec3& p) {
  double den = ray.direction.dot(normal);
  if (std::fabs(den) < 1e-8) return false;
  t = center.sub(ray.origin).dot(normal) / den;
  if (t < tMin || t > tMax) return false;
  p = ray.at(t);
  return p.sub(center).length() <= radius;
}

// Finite cylinder with optional caps (cylinder.go:24-266)
struct Cylinder : Shape {
  Vec3 base, top, axis;
  double radius, height;
  bool capped;
  const Material* material;
  Cylinder(Vec3 b, Vec3 tp, double r, bool cap, const Material* m)
      : base(b), top(tp), radius(r), capped(cap), material(m) {
    Vec3 av = top.sub(base);
    height = av.length();
    axis = av.normalize();
  }
  bool hit(const Ray& ray, double tMin, double tMax, SurfaceInteraction& out) const override {
    counters().prims++;
    double closest = tMax;
    bool any = false;
    Vec3 outward, point;
    Vec2 uv;
    // body (hitBody, cylinder.go:125-221)
    {
      Vec3 delta = ray.origin.sub(base);
      double DV = ray.direction.dot(axis), dV = delta.dot(axis);
      double a = ray.direction.lengthSquared() - DV * DV;
      double b = 2.0 * (delta.dot(ray.direction) - dV * DV);
      double c = delta.lengthSquared() - dV * dV - radius * radius;
      if (std::fabs(a) >= 1e-8) {
        double disc = b * b - 4 * a * c;
        if (disc >= 0) {
          double sq = std::sqrt(disc);
          double t1 = (-b - sq) / (2 * a), t2 = (-b + sq) / (2 * a);
          double t = t1;
          bool ok = true;
          if (t < tMin || t > closest) {
            t = t2;
            if (t < tMin || t > closest) ok = false;
          }
          if (ok) {
            Vec3 p = ray.at(t);
            double h = p.sub(base).dot(axis);
            if (h < 0 || h > height) {
              ok = false;
              if (t == t1) {
                t = t2;
                if (!(t < tMin || t > closest)) {
                  p = ray.at(t);
                  h = p.sub(base).dot(axis);
                  ok = !(h < 0 || h > height);
                }
              }
            }
            if (ok) {
              Vec3 onAxis = base.add(axis.mul(h));
              outward = p.sub(onAxis).normalize();
              uv = axialUV(axis, p.sub(onAxis), h, height);
              point = p;
              closest = t;
              any = true;
            }
          }
        }
      }
    }
    if (capped) {
      double t;
      Vec3 p;
      if (hit_cap(ray, base, axis.negate(), radius, tMin, closest, t, p)) {
        closest = t;
        point = p;
        outward = axis.negate();
        uv = capUV(outward, base, radius, p);
        any = true;
      }
      if (hit_cap(ray, top, axis, radius, tMin, closest, t, p)) {
        closest = t;
        point = p;
        outward = axis;
        uv = capUV(outward, top, radius, p);
        any = true;
      }
    }
    if (!any) return false;
    out = SurfaceInteraction();
    out.t = closest;
    out.point = point;
    out.uv = uv;
    out.material = material;
    out.shape = id;
    out.sub = 0;
    out.setFaceNormal(ray, outward);
    return true;
  }
  AABB boundingBox() const override {  // segment box widened by r except along an axis-parallel direction
    double e[3];
    for (int k = 0; k < 3; k++) e[k] = std::fabs(axis.axis(k)) > 0.9999 ? 0.0 : radius;
    Vec3 lo(std::min(base.x, top.x) - e[0], std::min(base.y, top.y) - e[1], std::min(base.z, top.z) - e[2]);
    Vec3 hi(std::max(base.x, top.x) + e[0], std::max(base.y, top.y) + e[1], std::max(base.z, top.z) + e[2]);
    return {lo, hi};
  }
};

// Cone or frustum with optional caps (cone.go:27-350)
struct Cone : Shape {
  Vec3 base, top, axis, apex;
  double r0, r1, height, tanAngle;
  bool capped;
  const Material* material;
  Cone(Vec3 b, double br, Vec3 tp, double tr, bool cap, const Material* m)
      : base(b), top(tp), r0(br), r1(tr), capped(cap), material(m) {
    Vec3 av = top.sub(base);
    height = av.length();
    axis = av.normalize();
    tanAngle = (r0 - r1) / height;
    apex = r1 == 0 ? top : top.add(axis.mul(r1 * height / (r0 - r1)));
  }
  // validateIntersection (cone.go:279-303)
  bool valid(const Ray& ray, double t, double tMin, double tMax) const {
    if (t < tMin || t > tMax) return false;
    Vec3 p = ray.at(t);
    double h = p.sub(base).dot(axis);
    if (h < -1e-8 || h > height + 1e-8) return false;
    return p.sub(apex).dot(axis) <= 1e-8;
  }
  bool hit(const Ray& ray, double tMin, double tMax, SurfaceInteraction& out) const override {
    counters().prims++;
    double closest = tMax;
    bool any = false;
    Vec3 outward, point;
    Vec2 uv;
    // body (hitBody, cone.go:180-276)
    {
      Vec3 CO = ray.origin.sub(apex);
      double DV = ray.direction.dot(axis), COV = CO.dot(axis);
      double k = tanAngle * tanAngle;
      double a = ray.direction.lengthSquared() - (1 + k) * DV * DV;
      double b = 2.0 * (ray.direction.dot(CO) - (1 + k) * DV * COV);
      double c = CO.lengthSquared() - (1 + k) * COV * COV;
      if (std::fabs(a) >= 1e-8) {
        double disc = b * b - 4 * a * c;
        if (disc >= 0) {
          double sq = std::sqrt(disc);
          double t = (-b - sq) / (2 * a);
          bool ok = valid(ray, t, tMin, closest);
          if (!ok) {
            t = (-b + sq) / (2 * a);
            ok = valid(ray, t, tMin, closest);
          }
          if (ok) {
            Vec3 p = ray.at(t);
            double h = p.sub(base).dot(axis);
            Vec3 radial = p.sub(base.add(axis.mul(h)));
            outward = radial.add(axis.mul((r0 - r1) / height)).normalize();
            uv = axialUV(axis, radial, h, height);
            point = p;
            closest = t;
            any = true;
          }
        }
      }
    }
    if (capped) {
      double t;
      Vec3 p;
      if (hit_cap(ray, base, axis.negate(), r0, tMin, closest, t, p)) {
        closest = t;
        point = p;
        outward = axis.negate();
        uv = capUV(outward, base, r0, p);
        any = true;
      }
      if (r1 > 0 && hit_cap(ray, top, axis, r1, tMin, closest, t, p)) {
        closest = t;
        point = p;
        outward = axis;
        uv = capUV(outward, top, r1, p);
        any = true;
      }
    }
    if (!any) return false;
    out = SurfaceInteraction();
    out.t = closest;
    out.point = point;
    out.uv = uv;
    out.material = material;
    out.shape = id;
    out.sub = 0;
    out.setFaceNormal(ray, outward);
    return true;
  }
  AABB boundingBox() const override {  // segment box widened by the base radius (cone.go:79-126)
    double e[3];
    for (int k = 0; k < 3; k++) e[k] = std::fabs(axis.axis(k)) > 0.9999 ? 0.0 : r0;
    Vec3 lo(std::min(base.x, top.x) - e[0], std::min(base.y, top.y) - e[1], std::min(base.z, top.z) - e[2]);
    Vec3 hi(std::max(base.x, top.x) + e[0], std::max(base.y, top.y) + e[1], std::max(base.z, top.z) + e[2]);
    return {lo, hi};
  }
};

// Triangle, Moller-Trumbore with epsilon 1e-8 (triangle.go:17-185)
struct Triangle : Shape {
  Vec3 v0, v1, v2, normal;
  const Material* material;
  AABB bbox;
  int subIndex = 0;
  bool hasUVs = false;
  Vec2 uv0, uv1, uv2;  // NewTriangleWithUVs (triangle.go:51-68)
  Triangle(Vec3 a, Vec3 b, Vec3 c, const Material* m) : v0(a), v1(b), v2(c), material(m) {
    normal = v1.sub(v0).cross(v2.sub(v0)).normalize();  // computeNormal (triangle.go:92-99)
    bbox = AABB::fromPoints({v0, v1, v2});
  }
  // NewTriangleWithNormal (triangle.go:35-49): the given normal, normalised
  void setNormal(const Vec3& n) { normal = n.normalize(); }
  bool hit(const Ray& ray, double tMin, double tMax, SurfaceInteraction& out) const override {
    counters().prims++;
    const double eps = 1e-8;
    Vec3 e1 = v1.sub(v0), e2 = v2.sub(v0);
    Vec3 h = ray.direction.cross(e2);
    double a = e1.dot(h);
    if (a > -eps && a < eps) return false;
    double f = 1.0 / a;
    Vec3 s = ray.origin.sub(v0);
    double uu = f * s.dot(h);
    if (uu < 0.0 || uu > 1.0) return false;
    Vec3 q = s.cross(e1);
    double vv = f * ray.direction.dot(q);
    if (vv < 0.0 || uu + vv > 1.0) return false;
    double t = f * e2.dot(q);
    if (t < tMin || t > tMax) return false;
    out = SurfaceInteraction();
    out.t = t;
    out.point = ray.at(t);
    out.material = material;
    // per-vertex UVs interpolated with the barycentrics, else the barycentrics (triangle.go:151-161)
    out.uv = hasUVs ? uv0.mul(1.0 - uu - vv).add(uv1.mul(uu)).add(uv2.mul(vv)) : Vec2(uu, vv);
    out.shape = id;
    out.sub = subIndex;
    out.setFaceNormal(ray, normal);
    return true;
  }
  AABB boundingBox() const override { return bbox; }
};

// BVH (bvh.go:13-239): binary, midpoint split of the longest axis, leaf <= 8
struct BVHNode {
  AABB box;
  std::unique_ptr<BVHNode> left, right;
  std::vector<const Shape*> shapes;
  bool leaf = false;
};

struct BVH {
  std::unique_ptr<BVHNode> root;
  Vec3 center;
  double radius = 0;

  static constexpr size_t kLeafThreshold = 8;  // bvh.go:58

  // NewBVH (bvh.go:26-55)
  explicit BVH(const std::vector<const Shape*>& shapes) {
    if (shapes.empty()) {
      center = {};
      radius = 0;  // NewBVH returns Radius 0 for an empty slice (bvh.go:27-29)
      return;
    }
    std::vector<const Shape*> copy = shapes;
    root = build(copy);
    center = root->box.center();
    radius = root->box.max.sub(center).length();
  }
  // buildBVH (bvh.go:64-109)
  static std::unique_ptr<BVHNode> build(std::vector<const Shape*>& shapes) {
    auto node = std::make_unique<BVHNode>();
    AABB box;
    if (!shapes.empty()) {
      box = shapes[0]->boundingBox();
      for (size_t i = 1; i < shapes.size(); i++) box = box.unite(shapes[i]->boundingBox());
    }
    node->box = box;
    auto makeLeaf = [&]() {
      node->leaf = true;
      node->shapes = shapes;
      return std::move(node);
    };
    if (shapes.size() <= kLeafThreshold) return makeLeaf();
    // findBestSplitSimple (bvh.go:112-134)
    int axis = box.longestAxis();
    double mn = box.min.axis(axis), mx = box.max.axis(axis);
    if (mx <= mn) return makeLeaf();
    double split = (mn + mx) * 0.5;
    // partitionShapesSimple (bvh.go:137-160)
    std::vector<const Shape*> l, r;
    for (const Shape* s : shapes) {
      if (s->boundingBox().center().axis(axis) < split) l.push_back(s);
      else r.push_back(s);
    }
    if (l.empty() || r.empty()) return makeLeaf();
    node->left = build(l);
    node->right = build(r);
    return node;
  }
  // Hit / hitNode (bvh.go:183-239): left then right, closest so far shrinks
  bool hit(const Ray& ray, double tMin, double tMax, SurfaceInteraction& out) const {
    if (!root) return false;
    return hitNode(root.get(), ray, tMin, tMax, out);
  }
  static bool hitNode(const BVHNode* node, const Ray& ray, double tMin, double tMax,
                      SurfaceInteraction& out) {
    if (!node->box.hit(ray, tMin, tMax)) return false;
    bool any = false;
    double closest = tMax;
    SurfaceInteraction tmp;
    if (node->leaf) {
      for (const Shape* s : node->shapes) {
        if (s->hit(ray, tMin, closest, tmp)) {
          any = true;
          closest = tmp.t;
          out = tmp;
        }
      }
      return any;
    }
    if (node->left && hitNode(node->left.get(), ray, tMin, closest, tmp)) {
      any = true;
      closest = tmp.t;
      out = tmp;
    }
    if (node->right && hitNode(node->right.get(), ray, tMin, closest, tmp)) {
      any = true;
      closest = tmp.t;
      out = tmp;
    }
    return any;
  }
  AABB boundingBox() const { return root ? root->box : AABB(); }
};

// Box: 6 quads from scaled, rotated corners (box.go:21-145)
struct Box : Shape {
  Vec3 center, size, rotation;
  const Material* material;
  std::unique_ptr<Quad> faces[6];
  AABB bbox;
  Box(Vec3 c, Vec3 s, Vec3 r, const Material* m) : center(c), size(s), rotation(r), material(m) {
    Vec3 cs[8] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                  {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (auto& p : cs) {
      p = Vec3(p.x * size.x, p.y * size.y, p.z * size.z);
      p = p.rotate(rotation);
      p = p.add(center);
    }
    faces[0] = std::make_unique<Quad>(cs[4], cs[5].sub(cs[4]), cs[7].sub(cs[4]), m);
    faces[1] = std::make_unique<Quad>(cs[1], cs[0].sub(cs[1]), cs[2].sub(cs[1]), m);
    faces[2] = std::make_unique<Quad>(cs[5], cs[1].sub(cs[5]), cs[6].sub(cs[5]), m);
    faces[3] = std::make_unique<Quad>(cs[0], cs[4].sub(cs[0]), cs[3].sub(cs[0]), m);
    faces[4] = std::make_unique<Quad>(cs[3], cs[7].sub(cs[3]), cs[2].sub(cs[3]), m);
    faces[5] = std::make_unique<Quad>(cs[4], cs[0].sub(cs[4]), cs[5].sub(cs[4]), m);
    for (int i = 0; i < 6; i++) faces[i]->subIndex = i;
    bbox = AABB::fromPoints(std::vector<Vec3>(cs, cs + 8));
  }
  void setId(int i) {
    id = i;
    for (auto& f : faces) f->id = i;
  }
  // Box.Hit keeps the first face on equal t (box.go:125-140)
  bool hit(const Ray& ray, double tMin, double tMax, SurfaceInteraction& out) const override {
    bool any = false;
    double closest = tMax;
    SurfaceInteraction tmp;
    for (const auto& f : faces) {
      if (f->hit(ray, tMin, closest, tmp)) {
        if (tmp.t < closest) {
          closest = tmp.t;
          out = tmp;
          any = true;
        }
      }
    }
    return any;
  }
  AABB boundingBox() const override { return bbox; }
};

// TriangleMesh with its own BVH (triangle_mesh.go:33-152)
struct TriangleMesh : Shape {
  std::vector<std::unique_ptr<Triangle>> tris;
  std::unique_ptr<BVH> bvh;
  AABB bbox;
  // TriangleMeshOptions.Normals (one per triangle) and VertexUVs (one per
  // vertex) are optional (triangle_mesh.go:20-26, 95-120)
  TriangleMesh(const std::vector<Vec3>& verts, const std::vector<uint32_t>& idx,
               const std::vector<const Material*>& mats, const double* tri_normals = nullptr,
               const double* vertex_uvs = nullptr) {
    size_t n = idx.size() / 3;
    tris.reserve(n);
    std::vector<const Shape*> shapes;
    shapes.reserve(n);
    for (size_t i = 0; i < n; i++) {
      uint32_t a = idx[3 * i], b = idx[3 * i + 1], c = idx[3 * i + 2];
      if (a >= verts.size() || b >= verts.size() || c >= verts.size())
        throw std::runtime_error("Face index out of bounds");
      tris.push_back(std::make_unique<Triangle>(verts[a], verts[b], verts[c], mats[i]));
      tris.back()->subIndex = (int)i;
      if (tri_normals) tris.back()->setNormal(Vec3(tri_normals[3 * i], tri_normals[3 * i + 1], tri_normals[3 * i + 2]));
      if (vertex_uvs) {
        Triangle& T = *tris.back();
        T.hasUVs = true;
        T.uv0 = Vec2(vertex_uvs[2 * a], vertex_uvs[2 * a + 1]);
        T.uv1 = Vec2(vertex_uvs[2 * b], vertex_uvs[2 * b + 1]);
        T.uv2 = Vec2(vertex_uvs[2 * c], vertex_uvs[2 * c + 1]);
      }
      shapes.push_back(tris.back().get());
    }
    bvh = std::make_unique<BVH>(shapes);
    if (!tris.empty()) {
      bbox = tris[0]->boundingBox();
      for (size_t i = 1; i < tris.size(); i++) bbox = bbox.unite(tris[i]->boundingBox());
    }
  }
  void setId(int i) {
    id = i;
    for (auto& t : tris) t->id = i;
  }
  bool hit(const Ray& ray, double tMin, double tMax, SurfaceInteraction& out) const override {
    return bvh->hit(ray, tMin, tMax, out);
  }
  AABB boundingBox() const override { return bbox; }
};

// ---------------------------------------------------------------------------
// Camera (pkg/geometry/camera.go)
// ---------------------------------------------------------------------------
struct CameraConfig {
  Vec3 center, lookAt, up;
  int width = 400;
  double aspectRatio = 1.0, vfov = 40.0, aperture = 0.0, focusDistance = 0.0;
};

struct CameraSample {
  Ray ray;
  Vec3 weight;
  double pdf = 0;
};

struct Camera {
  Vec3 center, pixel00, du, dv, diskU, diskV, u, v, w, forward;
  double focusDistance, lensRadius, lensArea, totalSensorArea, imagePlaneArea;
  int imageWidth, imageHeight;
  double theta, viewportWidth, viewportHeight, cosTotalWidth;
  // NewCamera (camera.go:70-170)
  explicit Camera(const CameraConfig& c) {
    w = c.center.sub(c.lookAt).normalize();
    u = w.cross(c.up).normalize();
    v = w.cross(u);
    focusDistance = c.focusDistance;
    if (focusDistance <= 0) focusDistance = c.center.sub(c.lookAt).length();
    lensRadius = c.aperture / 2;
    lensArea = kPi * lensRadius * lensRadius;
    if (c.aperture == 0) lensArea = 1.0;
    imageWidth = c.width;
    imageHeight = (int)((double)imageWidth / c.aspectRatio);
    theta = c.vfov * kPi / 180.0;
    double h = std::tan(theta / 2.0);
    viewportHeight = 2.0 * h * focusDistance;
    viewportWidth = viewportHeight * c.aspectRatio;
    double hz = std::tan(theta / 2.0);
    double vh1 = 2.0 * hz * 1.0;
    double vw1 = vh1 * c.aspectRatio;
    imagePlaneArea = vw1 * vh1;
    Vec3 vu = u.mul(viewportWidth), vv = v.mul(viewportHeight);
    du = vu.mul(1.0 / (double)imageWidth);
    dv = vv.mul(1.0 / (double)imageHeight);
    totalSensorArea = du.length() * dv.length() * (double)imageWidth * (double)imageHeight;
    Vec3 ul = c.center.sub(w.mul(focusDistance)).sub(vu.mul(0.5)).sub(vv.mul(0.5));
    pixel00 = ul.add(du.add(dv).mul(0.5));
    diskU = u.mul(c.aperture / 2);
    diskV = v.mul(c.aperture / 2);
    forward = c.lookAt.sub(c.center).normalize();
    Vec3 corner = Vec3(-viewportWidth / 2, -viewportHeight / 2, -focusDistance).normalize();
    cosTotalWidth = corner.dot(Vec3(0, 0, -1));
    center = c.center;
  }
  // GetRay (camera.go:173-190)
  Ray getRay(int i, int j, Vec2 samplePoint, Vec2 jitter) const {
    Vec3 jit(jitter.x - 0.5, jitter.y - 0.5, 0);
    Vec3 ps = pixel00.add(du.mul((double)i + jit.x)).add(dv.mul((double)j + jit.y));
    Vec3 o = center;
    if (diskU.length() > 0) {
      Vec3 p = samplePointInUnitDisk(samplePoint);
      o = center.add(diskU.mul(p.x).add(diskV.mul(p.y)));
    }
    return Ray(o, ps.sub(o).normalize());
  }
  // MapRayToPixel (camera.go:280-316)
  bool mapRayToPixel(const Ray& ray, int& px, int& py) const {
    Vec3 ipc = center.sub(w.mul(focusDistance));
    Vec3 toPlane = ipc.sub(ray.origin);
    double t = toPlane.dot(w) / ray.direction.dot(w);
    if (t <= 0) return false;
    Vec3 hp = ray.origin.add(ray.direction.mul(t));
    Vec3 rel = hp.sub(ipc);
    double planeX = rel.dot(u), planeY = rel.dot(v);
    double nx = (planeX + viewportWidth / 2) / viewportWidth;
    double ny = (planeY + viewportHeight / 2) / viewportHeight;
    int x = (int)(nx * (double)imageWidth), y = (int)(ny * (double)imageHeight);
    if (x >= 0 && x < imageWidth && y >= 0 && y < imageHeight) {
      px = x;
      py = y;
      return true;
    }
    return false;
  }
  // CalculateRayPDFs (camera.go:194-216)
  void calculateRayPDFs(const Ray& ray, double& areaPdf, double& dirPdf) const {
    double cosTheta = ray.direction.dot(forward);
    areaPdf = dirPdf = 0;
    if (cosTheta <= cosTotalWidth) return;
    int x, y;
    if (!mapRayToPixel(ray, x, y)) return;
    areaPdf = 1.0 / lensArea;
    dirPdf = 1.0 / (imagePlaneArea * std::pow(cosTheta, 3));
  }
  // EvaluateRayImportance (camera.go:263-277)
  Vec3 evaluateRayImportance(const Ray& ray) const {
    double cosTheta = ray.direction.dot(forward);
    if (cosTheta < cosTotalWidth) return {};
    double imp = 1.0 / (imagePlaneArea * lensArea * std::pow(cosTheta, 4));
    return {imp, imp, imp};
  }
  // SampleCameraFromPoint (camera.go:226-259); returns false for Go's nil
  bool sampleCameraFromPoint(const Vec3& ref, Vec2 s, CameraSample& out) const {
    Vec3 lens = samplePointInUnitDisk(s).mul(lensRadius);
    Vec3 lp = center.add(u.mul(lens.x)).add(v.mul(lens.y));
    Vec3 dir = ref.sub(lp).normalize();
    double dist = ref.sub(lp).length();
    Ray r(lp, dir);
    double cosTheta = forward.absDot(r.direction);
    double pdf = (dist * dist) / (cosTheta * lensArea);
    Vec3 imp = evaluateRayImportance(r);
    if (imp.luminance() == 0) return false;
    out.ray = r;
    out.weight = imp;
    out.pdf = pdf;
    return true;
  }
};

// ---------------------------------------------------------------------------
// Lights (pkg/lights)
// ---------------------------------------------------------------------------
enum class LightType { Area, Point, Infinite };  // interfaces.go:8-14

struct LightSample {  // interfaces.go:46-53
  Vec3 point, normal, direction;
  double distance = 0;
  Vec3 emission;
  double pdf = 0;
};
struct EmissionSample {  // interfaces.go:56-63
  Vec3 point, normal, direction, emission;
  double areaPdf = 0, directionPdf = 0;
};

struct Light {
  virtual ~Light() = default;
  virtual LightType type() const = 0;
  virtual LightSample sample(const Vec3& p, const Vec3& n, Vec2 s) const = 0;
  virtual double pdf(const Vec3& p, const Vec3& n, const Vec3& dir) const = 0;
  virtual EmissionSample sampleEmission(Vec2 sp, Vec2 sd) const = 0;
  virtual void pdfLe(const Vec3& p, const Vec3& dir, double& pdfPos, double& pdfDir) const = 0;
  virtual Vec3 emit(const Ray& r, const SurfaceInteraction* hit) const = 0;
  virtual void preprocess(const Vec3&, double) {}
};

// SampleEmissionDirection (light_sampling.go:58-80)
inline EmissionSample sampleEmissionDirection(const Vec3& p, const Vec3& n, double areaPdf,
                                              const Material* m, Vec2 s) {
  EmissionSample e;
  Vec3 dir = sampleCosineHemisphere(n, s);
  e.point = p;
  e.normal = n;
  e.direction = dir;
  e.directionPdf = dir.dot(n) / kPi;
  if (m && m->isEmitter()) e.emission = m->emit(Ray(p, dir), nullptr);
  e.areaPdf = areaPdf;
  return e;
}

// SampleInfiniteLight (light_sampling.go:89-115)
inline Ray sampleInfiniteLight(const Vec3& c, double r, Vec2 sp, Vec2 sd, double& areaPdf,
                               double& dirPdf) {
  Vec3 dir = sampleOnUnitSphere(sd);
  Vec3 up = std::fabs(dir.x) > 0.9 ? Vec3(0, 1, 0) : Vec3(1, 0, 0);
  Vec3 right = dir.cross(up).normalize();
  up = right.cross(dir).normalize();
  Vec3 ds = samplePointInUnitDisk(sp);
  Vec3 dp = c.add(right.mul(ds.x * r)).add(up.mul(ds.y * r));
  Vec3 ep = dp.add(dir.mul(-r));
  areaPdf = 1.0 / (kPi * r * r);
  dirPdf = 1.0 / (4.0 * kPi);
  return Ray(ep, dir);
}

// QuadLight (quad_light.go:13-195)
struct QuadLight : Light {
  const Quad* quad;
  double area;
  explicit QuadLight(const Quad* q) : quad(q) { area = q->u.cross(q->v).length(); }
  LightType type() const override { return LightType::Area; }
  Vec3 emit(const Ray& r, const SurfaceInteraction* hit) const override {
    if (quad->material && quad->material->isEmitter()) return quad->material->emit(r, hit);
    return {};
  }
  LightSample sample(const Vec3& p, const Vec3&, Vec2 s) const override {
    LightSample ls;
    Vec3 sp = quad->corner.add(quad->u.mul(s.x)).add(quad->v.mul(s.y));
    Vec3 to = sp.sub(p);
    double dist = to.length();
    Vec3 dir = to.mul(1.0 / dist);
    double pdfA = 1.0 / area;
    double cosTheta = std::fabs(quad->normal.dot(dir.mul(-1)));
    ls.point = sp;
    ls.normal = quad->normal;
    ls.direction = dir;
    ls.distance = dist;
    if (cosTheta < 1e-8) {
      ls.emission = {};
      ls.pdf = 0;
      return ls;
    }
    ls.pdf = pdfA * dist * dist / cosTheta;
    bool front = dir.dot(quad->normal) < 0;
    ls.emission = front ? emit(Ray(p, dir), nullptr) : Vec3();
    return ls;
  }
  double pdf(const Vec3& p, const Vec3&, const Vec3& dir) const override {
    SurfaceInteraction h;
    if (!quad->hit(Ray(p, dir), 0.001, kInf, h)) return 0.0;
    double dist = h.t;
    double cosTheta = std::fabs(quad->normal.dot(dir.mul(-1)));
    if (cosTheta < 1e-8) return 0.0;
    return (1.0 / area) * dist * dist / cosTheta;
  }
  EmissionSample sampleEmission(Vec2 sp, Vec2 sd) const override {
    EmissionSample e;
    e.point = quad->corner.add(quad->u.mul(sp.x)).add(quad->v.mul(sp.y));
    e.direction = sampleCosineHemisphere(quad->normal, sd);
    e.normal = quad->normal;
    e.areaPdf = 1.0 / area;
    e.directionPdf = e.direction.dot(quad->normal) / kPi;
    e.emission = emit(Ray(e.point, e.direction), nullptr);
    return e;
  }
  void pdfLe(const Vec3& p, const Vec3& dir, double& pdfPos, double& pdfDir) const override {
    pdfPos = pdfDir = 0;
    Vec3 tp = p.sub(quad->corner);
    double uu = quad->u.dot(quad->u), vv = quad->v.dot(quad->v), uv = quad->u.dot(quad->v);
    if (uu == 0 || vv == 0) return;
    double det = uu * vv - uv * uv;
    if (std::fabs(det) < 1e-8) return;
    double tu = tp.dot(quad->u), tv = tp.dot(quad->v);
    double alpha = (vv * tu - uv * tv) / det;
    double beta = (uu * tv - uv * tu) / det;
    if (alpha < 0 || alpha > 1 || beta < 0 || beta > 1) return;
    Vec3 rec = quad->corner.add(quad->u.mul(alpha)).add(quad->v.mul(beta));
    if (rec.sub(p).length() > 0.001) return;
    pdfPos = 1.0 / area;
    double c = dir.dot(quad->normal);
    if (c <= 0) return;
    pdfDir = c / kPi;
  }
};

// SphereLight (sphere_light.go:13-224)
struct SphereLight : Light {
  const Sphere* sphere;
  explicit SphereLight(const Sphere* s) : sphere(s) {}
  LightType type() const override { return LightType::Area; }
  Vec3 emit(const Ray& r, const SurfaceInteraction* hit) const override {
    if (sphere->material && sphere->material->isEmitter()) return sphere->material->emit(r, hit);
    return {};
  }
  LightSample sampleUniform(const Vec3& p, Vec2 s) const {
    double z = 1.0 - 2.0 * s.x;
    double r = std::sqrt(std::max(0.0, 1.0 - z * z));
    double phi = 2.0 * kPi * s.y;
    Vec3 ld(r * std::cos(phi), r * std::sin(phi), z);
    Vec3 sp = sphere->center.add(ld.mul(sphere->radius));
    Vec3 d = sp.sub(p);
    LightSample ls;
    ls.point = sp;
    ls.normal = ld;
    ls.direction = d.normalize();
    ls.distance = d.length();
    ls.pdf = 1.0 / (4.0 * kPi * sphere->radius * sphere->radius);
    ls.emission = emit(Ray(p, ls.direction), nullptr);
    return ls;
  }
  LightSample sampleVisible(const Vec3& p, Vec2 s) const {
    Vec3 tc = sphere->center.sub(p);
    double dc = tc.length();
    Vec3 w = tc.normalize();
    Vec3 u = std::fabs(w.x) > 0.1 ? Vec3(0, 1, 0) : Vec3(1, 0, 0);
    u = u.cross(w).normalize();
    Vec3 v = w.cross(u);
    double sinMax = sphere->radius / dc;
    double cosMax = std::sqrt(std::max(0.0, 1.0 - sinMax * sinMax));
    double cosT = 1.0 - s.x * (1.0 - cosMax);
    double sinT = std::sqrt(std::max(0.0, 1.0 - cosT * cosT));
    double phi = 2.0 * kPi * s.y;
    Vec3 dir = u.mul(sinT * std::cos(phi)).add(v.mul(sinT * std::sin(phi))).add(w.mul(cosT));
    Ray r(p, dir);
    SurfaceInteraction h;
    if (!sphere->hit(r, 0.001, kInf, h)) return sampleUniform(p, s);
    LightSample ls;
    ls.point = h.point;
    ls.normal = h.normal;
    ls.direction = dir;
    ls.distance = h.t;
    ls.pdf = 1.0 / (2.0 * kPi * (1.0 - cosMax));
    ls.emission = emit(r, nullptr);
    return ls;
  }
  LightSample sample(const Vec3& p, const Vec3&, Vec2 s) const override {
    double dc = sphere->center.sub(p).length();
    if (dc <= sphere->radius) return sampleUniform(p, s);
    return sampleVisible(p, s);
  }
  double pdf(const Vec3& p, const Vec3&, const Vec3& dir) const override {
    SurfaceInteraction h;
    if (!sphere->hit(Ray(p, dir), 0.001, kInf, h)) return 0.0;
    double dc = sphere->center.sub(p).length();
    if (dc <= sphere->radius) return 1.0 / (4.0 * kPi * sphere->radius * sphere->radius);
    double sinMax = sphere->radius / dc;
    double cosMax = std::sqrt(std::max(0.0, 1.0 - sinMax * sinMax));
    return 1.0 / (2.0 * kPi * (1.0 - cosMax));
  }
  EmissionSample sampleEmission(Vec2 sp, Vec2 sd) const override {
    double z = 1.0 - 2.0 * sp.x;
    double r = std::sqrt(std::max(0.0, 1.0 - z * z));
    double phi = 2.0 * kPi * sp.y;
    Vec3 ld(r * std::cos(phi), r * std::sin(phi), z);
    Vec3 p = sphere->center.add(ld.mul(sphere->radius));
    double areaPdf = 1.0 / (4.0 * kPi * sphere->radius * sphere->radius);
    return sampleEmissionDirection(p, ld, areaPdf, sphere->material, sd);
  }
  void pdfLe(const Vec3& p, const Vec3& dir, double& pdfPos, double& pdfDir) const override {
    pdfPos = pdfDir = 0;
    double dc = p.sub(sphere->center).length();
    if (!(std::fabs(dc - sphere->radius) <= 0.001)) return;  // validatePointOnSphere
    Vec3 n = p.sub(sphere->center).normalize();
    if (dir.dot(n) <= 0) return;
    pdfPos = 1.0 / (4.0 * kPi * sphere->radius * sphere->radius);
    pdfDir = dir.dot(n) / kPi;
  }
};

// UniformInfiniteLight (uniform_infinite_light.go:40-132)
struct UniformInfiniteLight : Light {
  Vec3 emission, worldCenter;
  double worldRadius = 0;
  explicit UniformInfiniteLight(Vec3 e) : emission(e) {}
  LightType type() const override { return LightType::Infinite; }
  Vec3 emit(const Ray&, const SurfaceInteraction*) const override { return emission; }
  LightSample sample(const Vec3& p, const Vec3& n, Vec2 s) const override {
    LightSample ls;
    Vec3 dir = sampleCosineHemisphere(n, s);
    ls.point = p.add(dir.mul(1e10));
    ls.normal = dir.mul(-1);
    ls.direction = dir;
    ls.distance = kInf;
    ls.emission = emission;
    ls.pdf = dir.dot(n) / kPi;
    return ls;
  }
  double pdf(const Vec3&, const Vec3& n, const Vec3& dir) const override {
    double c = dir.dot(n);
    if (c <= 0) return 0.0;
    return c / kPi;
  }
  EmissionSample sampleEmission(Vec2 sp, Vec2 sd) const override {
    EmissionSample e;
    Ray r = sampleInfiniteLight(worldCenter, worldRadius, sp, sd, e.areaPdf, e.directionPdf);
    e.point = r.origin;
    e.normal = r.direction.mul(-1);
    e.direction = r.direction;
    e.emission = emission;
    return e;
  }
  void pdfLe(const Vec3&, const Vec3&, double& pdfPos, double& pdfDir) const override {
    pdfPos = pdfDir = 0;
    if (worldRadius <= 0) return;
    pdfPos = 1.0 / (kPi * worldRadius * worldRadius);
    pdfDir = 1.0 / (4.0 * kPi);
  }
  void preprocess(const Vec3& c, double r) override {
    worldCenter = c;
    worldRadius = r;
  }
};

// GradientInfiniteLight (gradient_infinite_light.go:43-147)
struct GradientInfiniteLight : Light {
  Vec3 top, bottom, worldCenter;
  double worldRadius = 0;
  GradientInfiniteLight(Vec3 t, Vec3 b) : top(t), bottom(b) {}
  LightType type() const override { return LightType::Infinite; }
  Vec3 forDirection(const Vec3& d) const {
    double t = 0.5 * (d.y + 1.0);
    return bottom.mul(1.0 - t).add(top.mul(t));
  }
  Vec3 emit(const Ray& r, const SurfaceInteraction*) const override {
    return forDirection(r.direction.normalize());
  }
  LightSample sample(const Vec3& p, const Vec3& n, Vec2 s) const override {
    LightSample ls;
    Vec3 dir = sampleCosineHemisphere(n, s);
    ls.point = p.add(dir.mul(1e10));
    ls.normal = dir.mul(-1);
    ls.direction = dir;
    ls.distance = kInf;
    ls.emission = forDirection(dir);
    ls.pdf = dir.dot(n) / kPi;
    return ls;
  }
  double pdf(const Vec3&, const Vec3& n, const Vec3& dir) const override {
    double c = dir.dot(n);
    if (c <= 0) return 0.0;
    return c / kPi;
  }
  EmissionSample sampleEmission(Vec2 sp, Vec2 sd) const override {
    EmissionSample e;
    Ray r = sampleInfiniteLight(worldCenter, worldRadius, sp, sd, e.areaPdf, e.directionPdf);
    e.point = r.origin;
    e.normal = r.direction.mul(-1);
    e.direction = r.direction;
    e.emission = forDirection(r.direction);
    return e;
  }
  void pdfLe(const Vec3&, const Vec3&, double& pdfPos, double& pdfDir) const override {
    pdfPos = pdfDir = 0;
    if (worldRadius <= 0) return;
    pdfPos = 1.0 / (kPi * worldRadius * worldRadius);
    pdfDir = 1.0 / (4.0 * kPi);
  }
  void preprocess(const Vec3& c, double r) override {
    worldCenter = c;
    worldRadius = r;
  }
};

// Spot falloff shared by the point and disc spot lights
// (point_spot_light.go:140-158, disc_spot_light.go:150-168): 0 outside the
// cone, 1 inside the inner cone, a quartic of the cosine ramp between
inline double spotFalloff(double cosAngle, double cosTotal, double cosStart) {
  if (cosAngle < cosTotal) return 0.0;
  if (cosAngle >= cosStart) return 1.0;
  double d = (cosAngle - cosTotal) / (cosStart - cosTotal);
  return d * d * d * d;
}

// DiscLight (disc_light.go:12-165)
struct DiscLight : Light {
  const Disc* disc;
  explicit DiscLight(const Disc* d) : disc(d) {}
  LightType type() const override { return LightType::Area; }
  double areaPdf() const { return 1.0 / (kPi * disc->radius * disc->radius); }
  // Disc.SampleUniform (disc.go:120-134)
  Vec3 samplePoint(Vec2 s) const {
    double r = std::sqrt(s.x) * disc->radius;
    double th = 2.0 * kPi * s.y;
    return disc->center.add(disc->right.mul(r * std::cos(th))).add(disc->up.mul(r * std::sin(th)));
  }
  Vec3 emit(const Ray& r, const SurfaceInteraction* hit) const override {
    if (disc->material && disc->material->isEmitter()) return disc->material->emit(r, hit);
    return {};
  }
  LightSample sample(const Vec3& p, const Vec3&, Vec2 s) const override {
    LightSample ls;
    Vec3 sp = samplePoint(s);
    Vec3 to = sp.sub(p);
    double dist = to.length();
    Vec3 dir = to.normalize();
    ls.point = sp;
    ls.normal = disc->normal;
    if (dist == 0) {
      ls.direction = Vec3(0, 1, 0);
      ls.distance = 0;
      ls.pdf = 1.0;
      return ls;
    }
    double pdf = areaPdf();
    double ct = std::fabs(disc->normal.dot(dir.mul(-1)));
    ls.pdf = ct < 1e-6 ? 0.0 : pdf * dist * dist / ct;
    ls.direction = dir;
    ls.distance = dist;
    ls.emission = emit(Ray(p, dir), nullptr);
    return ls;
  }
  double pdf(const Vec3& p, const Vec3&, const Vec3& dir) const override {
    SurfaceInteraction h;
    if (!disc->hit(Ray(p, dir), 0.001, kInf, h)) return 0.0;
    double ct = std::fabs(disc->normal.dot(dir.mul(-1)));
    if (ct < 1e-6) return 0.0;
    return areaPdf() * h.t * h.t / ct;
  }
  EmissionSample sampleEmission(Vec2 sp, Vec2 sd) const override {
    return sampleEmissionDirection(samplePoint(sp), disc->normal, areaPdf(), disc->material, sd);
  }
  void pdfLe(const Vec3& p, const Vec3& dir, double& pdfPos, double& pdfDir) const override {
    pdfPos = pdfDir = 0;
    // validatePointOnDisc (disc_light.go:153-165), tolerance 0.001
    Vec3 tp = p.sub(disc->center);
    double h = tp.dot(disc->normal);
    if (std::fabs(h) > 0.001) return;
    if (tp.sub(disc->normal.mul(h)).length() > disc->radius) return;
    if (dir.dot(disc->normal) <= 0) return;
    pdfPos = areaPdf();
    pdfDir = dir.dot(disc->normal) / kPi;
  }
};

// DiscSpotLight (disc_spot_light.go:64-283): a DiscLight whose disc carries
// the directional SpotEmissive material
struct DiscSpotLight : Light {
  Vec3 position, direction, emission;
  double cosTotal, cosStart;
  DiscLight base;
  DiscSpotLight(const Disc* d, Vec3 from, Vec3 to, Vec3 e, double coneDeg, double deltaDeg)
      : position(from), direction(to.sub(from).normalize()), emission(e), base(d) {
    cosTotal = std::cos(coneDeg * kPi / 180.0);
    cosStart = std::cos((coneDeg - deltaDeg) * kPi / 180.0);
  }
  LightType type() const override { return LightType::Area; }
  Vec3 emit(const Ray& r, const SurfaceInteraction* hit) const override { return base.emit(r, hit); }
  LightSample sample(const Vec3& p, const Vec3& n, Vec2 s) const override {
    LightSample ls = base.sample(p, n, s);
    Vec3 lightToPoint = p.sub(ls.point).normalize();
    ls.emission = ls.emission.mul(spotFalloff(direction.dot(lightToPoint), cosTotal, cosStart));
    return ls;
  }
  double pdf(const Vec3& p, const Vec3& n, const Vec3& dir) const override { return base.pdf(p, n, dir); }
  EmissionSample sampleEmission(Vec2 sp, Vec2 sd) const override {
    EmissionSample e;
    e.point = base.samplePoint(sp);
    e.normal = base.disc->normal;
    e.direction = sampleCone(direction, cosTotal, sd);
    e.emission = emission.mul(spotFalloff(e.direction.dot(direction), cosTotal, cosStart));
    e.areaPdf = base.areaPdf();
    e.directionPdf = 1.0 / (2.0 * kPi * (1.0 - cosTotal));  // UniformConePDF (light_sampling.go:83-85)
    return e;
  }
  void pdfLe(const Vec3& p, const Vec3& dir, double& pdfPos, double& pdfDir) const override {
    double bp, bd;
    base.pdfLe(p, dir, bp, bd);
    pdfPos = pdfDir = 0;
    if (bp == 0.0 || bd == 0.0) return;
    pdfPos = bp;
    if (dir.dot(direction) < cosTotal) return;
    pdfDir = bd;
  }
};

// PointSpotLight (point_spot_light.go:10-222): a delta light
struct PointSpotLight : Light {
  Vec3 position, direction, emission;
  double cosTotal, cosStart;
  PointSpotLight(Vec3 from, Vec3 to, Vec3 e, double coneDeg, double deltaDeg)
      : position(from), direction(to.sub(from).normalize()), emission(e) {
    cosTotal = std::cos(coneDeg * kPi / 180.0);
    cosStart = std::cos((coneDeg - deltaDeg) * kPi / 180.0);
  }
  LightType type() const override { return LightType::Point; }
  Vec3 emit(const Ray&, const SurfaceInteraction*) const override { return emission; }
  LightSample sample(const Vec3& p, const Vec3&, Vec2) const override {
    LightSample ls;
    ls.point = position;
    Vec3 to = position.sub(p);
    double dist = to.length();
    ls.pdf = 1.0;
    if (dist == 0) {
      ls.normal = Vec3(0, 1, 0);
      ls.direction = Vec3(0, 1, 0);
      ls.distance = 0;
      return ls;
    }
    Vec3 toLight = to.normalize();
    double att = spotFalloff(direction.dot(toLight.mul(-1)), cosTotal, cosStart);
    ls.emission = emission.mul(att / (dist * dist));
    ls.normal = toLight.mul(-1);
    ls.direction = toLight;
    ls.distance = dist;
    return ls;
  }
  double pdf(const Vec3& p, const Vec3&, const Vec3& dir) const override {
    Vec3 to = position.sub(p);
    if (to.length() == 0) return 0.0;
    return dir.dot(to.normalize()) > 0.999 ? 1.0 : 0.0;
  }
  EmissionSample sampleEmission(Vec2, Vec2 sd) const override {
    EmissionSample e;
    e.point = position;
    e.direction = sampleCone(direction, cosTotal, sd);
    e.normal = e.direction;
    e.emission = emission.mul(spotFalloff(e.direction.dot(direction), cosTotal, cosStart));
    e.areaPdf = 1.0;
    e.directionPdf = 1.0 / (2.0 * kPi * (1.0 - cosTotal));
    return e;
  }
  void pdfLe(const Vec3& p, const Vec3& dir, double& pdfPos, double& pdfDir) const override {
    pdfPos = pdfDir = 0;
    if (p.sub(position).length() > 0.001) return;
    if (dir.dot(direction) < cosTotal) return;
    pdfPos = 1.0;
    pdfDir = 1.0 / (2.0 * kPi * (1.0 - cosTotal));
  }
};

// WeightedLightSampler (weighted_light_sampler.go:11-128)
struct LightSampler {
  std::vector<const Light*> lights;
  std::vector<double> weights;
  // NewUniformLightSampler (weighted_light_sampler.go:57-78)
  static LightSampler uniform(const std::vector<const Light*>& ls) {
    LightSampler s;
    s.lights = ls;
    if (!ls.empty()) s.weights.assign(ls.size(), 1.0 / (double)ls.size());
    return s;
  }
  // NewWeightedLightSampler (weighted_light_sampler.go:22-54)
  static LightSampler weighted(const std::vector<const Light*>& ls, const std::vector<double>& w) {
    if (ls.size() != w.size()) throw std::runtime_error("lights length must match weights length");
    LightSampler s;
    s.lights = ls;
    double total = 0;
    for (double x : w) {
      if (x < 0) throw std::runtime_error("weights must be non-negative");
      total += x;
    }
    s.weights.resize(w.size());
    for (size_t i = 0; i < w.size(); i++)
      s.weights[i] = total == 0 ? 1.0 / (double)w.size() : w[i] / total;
    return s;
  }
  // SampleLight / SampleLightEmission (weighted_light_sampler.go:82-124)
  const Light* pick(double u, double& prob, int& index) const {
    if (lights.empty()) {
      prob = 0;
      index = -1;
      return nullptr;
    }
    double cum = 0;
    for (size_t i = 0; i < lights.size(); i++) {
      cum += weights[i];
      if (u <= cum) {
        prob = weights[i];
        index = (int)i;
        return lights[i];
      }
    }
    index = (int)lights.size() - 1;
    prob = weights[index];
    return lights[index];
  }
  // GetLightProbability (weighted_light_sampler.go:127-132)
  double probability(int i) const {
    if (i < 0 || i >= (int)weights.size()) return 0.0;
    return weights[i];
  }
};

// CalculateLightPDF (light_sampling.go:11-26)
inline double calculateLightPDF(const std::vector<const Light*>& lights, const LightSampler& ls,
                                const Vec3& p, const Vec3& n, const Vec3& dir) {
  if (lights.empty()) return 0.0;
  double total = 0;
  for (size_t i = 0; i < lights.size(); i++)
    total += lights[i]->pdf(p, n, dir) * ls.probability((int)i);
  return total;
}
// SampleLight (light_sampling.go:28-38)
inline bool sampleLight(const std::vector<const Light*>& lights, const LightSampler& ls,
                        const Vec3& p, const Vec3& n, Sampler& s, LightSample& out,
                        const Light*& light, int& index) {
  if (lights.empty()) return false;
  double prob;
  light = ls.pick(s.get1D(), prob, index);
  out = light->sample(p, n, s.get2D());
  out.pdf *= prob;
  return true;
}

// ---------------------------------------------------------------------------
// Scene (pkg/scene/scene.go)
// ---------------------------------------------------------------------------
struct SamplingConfig {
  int width = 0, height = 0, samplesPerPixel = 0, maxDepth = 5, rrMinBounces = 0;
  double adaptiveMinSamples = 0, adaptiveThreshold = 0;
};

struct Scene {
  std::unique_ptr<Camera> camera;
  std::vector<std::unique_ptr<ImageTexture>> textures;
  std::vector<std::unique_ptr<Material>> materials;
  std::vector<std::unique_ptr<Shape>> ownedShapes;
  std::vector<const Shape*> shapes;
  std::vector<std::unique_ptr<Light>> ownedLights;
  std::vector<const Light*> lights;
  std::unique_ptr<LightSampler> lightSampler;
  SamplingConfig sampling;
  std::unique_ptr<BVH> bvh;

  // Preprocess (scene.go:45-78)
  void preprocess() {
    bvh = std::make_unique<BVH>(shapes);
    for (auto& l : ownedLights) l->preprocess(bvh->center, bvh->radius);
    if (!lightSampler) lightSampler = std::make_unique<LightSampler>(LightSampler::uniform(lights));
  }
};

// ---------------------------------------------------------------------------
// Path tracing integrator (pkg/integrator/path_tracing.go)
// ---------------------------------------------------------------------------
// powerHeuristic (path_tracing.go:225-235)
inline double powerHeuristic(int nf, double fPdf, int ng, double gPdf) {
  if (fPdf == 0) return 0;
  double f = nf * fPdf, g = ng * gPdf;
  return (f * f) / (f * f + g * g);
}

inline Vec3 getEmittedLight(const Ray& ray, const SurfaceInteraction& hit) {  // :108-113
  if (hit.material && hit.material->isEmitter()) return hit.material->emit(ray, &hit);
  return {};
}

struct PathTracingIntegrator {
  SamplingConfig config;
  explicit PathTracingIntegrator(SamplingConfig c) : config(c) {}

  Vec3 rayColor(const Ray& ray, const Scene& scene, Sampler& s) const {  // :29-33
    return recurse(ray, scene, s, config.maxDepth, Vec3(1, 1, 1));
  }
  // rayColorRecursive (path_tracing.go:35-85)
  Vec3 recurse(const Ray& ray, const Scene& scene, Sampler& s, int depth, Vec3 thr) const {
    if (depth <= 0) return {};
    double comp;
    if (russianRoulette(depth, thr, s.get1D(), comp)) return {};
    SurfaceInteraction hit;
    if (!scene.bvh->hit(ray, 0.001, kInf, hit)) {
      Vec3 e;
      for (const Light* l : scene.lights)
        if (l->type() == LightType::Infinite) e = e.add(l->emit(ray, nullptr));
      return e.mul(comp);
    }
    Vec3 le = getEmittedLight(ray, hit);
    ScatterResult sc;
    if (!hit.material->scatter(ray, hit, s, sc)) return le.mul(comp);
    Vec3 col;
    if (sc.isSpecular()) {
      // calculateSpecularColor (:88-97)
      Vec3 nt = thr.mulVec(sc.attenuation);
      Vec3 inc = recurse(sc.scattered, scene, s, depth - 1, nt);
      col = sc.attenuation.mulVec(inc);
    } else {
      col = directLighting(scene, sc, hit, s).add(indirectLighting(scene, sc, hit, depth, thr, s));
    }
    return le.add(col).mul(comp);
  }
  // CalculateDirectLighting (path_tracing.go:116-157)
  Vec3 directLighting(const Scene& scene, const ScatterResult& sc, const SurfaceInteraction& hit,
                      Sampler& s) const {
    LightSample ls;
    const Light* l;
    int idx;
    if (!sampleLight(scene.lights, *scene.lightSampler, hit.point, hit.normal, s, ls, l, idx))
      return {};
    if (ls.emission.luminance() <= 0 || ls.pdf <= 0) return {};
    SurfaceInteraction tmp;
    if (scene.bvh->hit(Ray(hit.point, ls.direction), 0.001, ls.distance - 0.001, tmp)) return {};
    double cosine = ls.direction.dot(hit.normal);
    if (cosine <= 0) return {};
    bool isDelta;
    double mp = hit.material->pdf(sc.incoming.direction, ls.direction, hit.normal, isDelta);
    if (isDelta) return {};
    double w = powerHeuristic(1, ls.pdf, 1, mp);
    Vec3 brdf = hit.material->evaluateBRDF(sc.incoming.direction, ls.direction, &hit,
                                           TransportMode::Radiance);
    return brdf.mulVec(ls.emission).mul(cosine * w / ls.pdf);
  }
  // CalculateIndirectLighting (path_tracing.go:160-189)
  Vec3 indirectLighting(const Scene& scene, const ScatterResult& sc, const SurfaceInteraction& hit,
                        int depth, const Vec3& thr, Sampler& s) const {
    if (sc.pdf <= 0) return {};
    Vec3 sd = sc.scattered.direction.normalize();
    double cosine = sd.dot(hit.normal);
    if (cosine <= 0) return {};
    double lp = calculateLightPDF(scene.lights, *scene.lightSampler, hit.point, hit.normal, sd);
    double w = powerHeuristic(1, sc.pdf, 1, lp);
    Vec3 nt = thr.mulVec(sc.attenuation).mul(cosine / sc.pdf);
    Vec3 inc = recurse(sc.scattered, scene, s, depth - 1, nt);
    return sc.attenuation.mul(cosine * w / sc.pdf).mulVec(inc);
  }
  // ApplyRussianRoulette (path_tracing.go:193-220)
  bool russianRoulette(int depth, const Vec3& thr, double u, double& comp) const {
    int bounce = config.maxDepth - depth;
    if (!(bounce >= config.rrMinBounces)) {
      comp = 1.0;
      return false;
    }
    double surv = std::min(0.95, std::max(0.5, thr.luminance()));
    if (u > surv) {
      comp = 0.0;
      return true;
    }
    comp = 1.0 / surv;
    return false;
  }
};

// ---------------------------------------------------------------------------
// BDPT (pkg/integrator/bdpt.go, bdpt_mis.go)
// ---------------------------------------------------------------------------
struct Vertex {  // bdpt.go:14-36
  SurfaceInteraction si;
  const Light* light = nullptr;
  int lightIndex = -1;
  Vec3 incomingDirection;
  double areaPdfForward = 0, areaPdfReverse = 0;
  bool isLight = false, isCamera = false, isSpecular = false, isInfiniteLight = false;
  Vec3 beta, emittedLight;
  // IsOnSurface (bdpt.go:42-49)
  bool isOnSurface() const {
    if (isLight && light != nullptr) return light->type() == LightType::Area;
    return si.material != nullptr;
  }
  // convertSolidAngleToAreaPdf (bdpt_mis.go:341-363)
  double convertSolidAngleToAreaPdf(const Vertex& next, double pdf) const {
    if (next.isInfiniteLight) return pdf;
    Vec3 d = next.si.point.sub(si.point);
    double d2 = d.lengthSquared();
    if (d2 == 0) return 0.0;
    double inv = 1.0 / d2;
    if (next.isOnSurface()) pdf *= d.mul(std::sqrt(inv)).absDot(next.si.normal);
    return pdf * inv;
  }
};

struct Path {  // bdpt.go:52-55
  std::vector<Vertex> vertices;
  int length = 0;
};

struct SplatRay {  // integrator.go:9-12
  Ray ray;
  Vec3 color;
};

inline double remap0(double f) { return f != 0 ? f : 1.0; }  // bdpt_mis.go:367-372

struct BDPTIntegrator {
  SamplingConfig config;
  explicit BDPTIntegrator(SamplingConfig c) : config(c) {}

  // RayColor (bdpt.go:73-102)
  Vec3 rayColor(const Ray& ray, const Scene& scene, Sampler& s, std::vector<SplatRay>& splats) const {
    Path cp = generateCameraPath(ray, scene, s, config.maxDepth);
    Path lp = generateLightPath(scene, s, config.maxDepth);
    Vec3 total;
    for (int si = 0; si <= lp.length; si++) {
      for (int t = 1; t <= cp.length; t++) {
        Vertex sampled;
        bool hasSampled = false;
        std::vector<SplatRay> sp;
        Vec3 light = evaluateStrategy(cp, lp, si, t, scene, s, sp, sampled, hasSampled);
        if (!light.isZero() || !sp.empty()) {
          double w = misWeight(cp, lp, hasSampled ? &sampled : nullptr, si, t, scene);
          total = total.add(light.mul(w));
          for (auto& x : sp) {
            x.color = x.color.mul(w);
            splats.push_back(x);
          }
        }
      }
    }
    return total;
  }

  // generateCameraPath (bdpt.go:106-135)
  Path generateCameraPath(const Ray& ray, const Scene& scene, Sampler& s, int maxDepth) const {
    Path p;
    double areaPdf, dirPdf;
    scene.camera->calculateRayPDFs(ray, areaPdf, dirPdf);
    Vertex cv;
    cv.si.point = ray.origin;
    cv.si.normal = ray.direction.mul(-1);
    cv.isCamera = true;
    cv.beta = Vec3(1, 1, 1);
    p.vertices.push_back(cv);
    p.length++;
    extendPath(p, ray, Vec3(1, 1, 1), dirPdf, scene, s, maxDepth, true);
    return p;
  }

  // generateLightPath (bdpt.go:139-202)
  Path generateLightPath(const Scene& scene, Sampler& s, int maxDepth) const {
    Path p;
    if (scene.lights.empty()) return p;
    double selPdf;
    int idx;
    const Light* light = scene.lightSampler->pick(s.get1D(), selPdf, idx);
    Vec2 a = s.get2D();
    Vec2 b = s.get2D();
    EmissionSample es = light->sampleEmission(a, b);
    double cosTheta = es.direction.absDot(es.normal);
    Vertex lv;
    lv.si.point = es.point;
    lv.si.normal = es.normal;
    lv.light = light;
    lv.lightIndex = idx;
    lv.areaPdfForward = es.areaPdf * selPdf;
    lv.areaPdfReverse = 0;
    lv.isLight = true;
    lv.isInfiniteLight = light->type() == LightType::Infinite;
    lv.beta = es.emission;
    lv.emittedLight = es.emission;
    p.vertices.push_back(lv);
    p.length++;
    Ray ray(es.point, es.direction);
    Vec3 beta = es.emission.mul(cosTheta / (selPdf * es.areaPdf * es.directionPdf));
    extendPath(p, ray, beta, es.directionPdf, scene, s, maxDepth - 1, false);
    if (p.vertices[0].isInfiniteLight) {
      if (p.length > 1) {
        Vertex& fb = p.vertices[1];
        fb.areaPdfForward = es.areaPdf * selPdf;
        if (fb.si.material != nullptr) fb.areaPdfForward *= ray.direction.absDot(fb.si.normal);
      }
      p.vertices[0].areaPdfForward = infiniteLightDensity(es.point, es.normal, es.direction, scene);
    }
    return p;
  }

  // extendPath (bdpt.go:206-291)
  void extendPath(Path& path, Ray ray, Vec3 beta, double pdfFwd, const Scene& scene, Sampler& s,
                  int maxBounces, bool isCamera) const {
    for (int b = 0; b < maxBounces; b++) {
      int prevIdx = path.length - 1;
      SurfaceInteraction hit;
      if (!scene.bvh->hit(ray, 0.001, kInf, hit)) {
        if (isCamera) {
          Vec3 e;
          for (const Light* l : scene.lights)
            if (l->type() == LightType::Infinite) e = e.add(l->emit(ray, nullptr));
          path.vertices.push_back(backgroundVertex(ray, e, beta, pdfFwd));
          path.length++;
        }
        break;
      }
      Vertex v;
      v.si = hit;
      v.incomingDirection = ray.direction.mul(-1);
      v.beta = beta;
      v.emittedLight = getEmittedLight(ray, hit);
      v.isLight = !v.emittedLight.isZero();
      v.areaPdfForward = path.vertices[prevIdx].convertSolidAngleToAreaPdf(v, pdfFwd);
      ScatterResult sc;
      if (!hit.material->scatter(ray, hit, s, sc)) {
        path.vertices.push_back(v);
        path.length++;
        break;
      }
      pdfFwd = sc.pdf;
      v.isSpecular = sc.isSpecular();
      double cosTheta = sc.scattered.direction.absDot(hit.normal);
      if (sc.isSpecular()) beta = beta.mulVec(sc.attenuation);
      else beta = beta.mulVec(sc.attenuation).mul(cosTheta / sc.pdf);
      bool revDelta;
      double pdfRev = hit.material->pdf(sc.scattered.direction, ray.direction.mul(-1), hit.normal,
                                        revDelta);
      if (revDelta) {
        v.isSpecular = true;
        pdfRev = 0.0;
        pdfFwd = 0.0;
      }
      path.vertices[prevIdx].areaPdfReverse = v.convertSolidAngleToAreaPdf(path.vertices[prevIdx], pdfRev);
      path.vertices.push_back(v);
      path.length++;
      ray = sc.scattered;
    }
  }

  // evaluateBDPTStrategy (bdpt.go:294-313)
  Vec3 evaluateStrategy(const Path& cp, const Path& lp, int s, int t, const Scene& scene,
                        Sampler& smp, std::vector<SplatRay>& splats, Vertex& sampled,
                        bool& hasSampled) const {
    hasSampled = false;
    if (s == 1 && t == 1) return {};
    if (s == 0) return pathTracingStrategy(cp, t);
    if (t == 1) {
      lightTracingStrategy(lp, s, scene, smp, splats, sampled, hasSampled);
      return {};
    }
    if (s == 1) return directLightingStrategy(cp, t, scene, smp, sampled, hasSampled);
    return connectionStrategy(cp, lp, s, t, scene);
  }

  // evaluatePathTracingStrategy (bdpt.go:317-332)
  Vec3 pathTracingStrategy(const Path& cp, int t) const {
    if (t == 0 || t < cp.length) return {};
    const Vertex& last = cp.vertices[t - 1];
    return last.emittedLight.mulVec(last.beta);
  }

  // evaluateDirectLightingStrategy (bdpt.go:334-394)
  Vec3 directLightingStrategy(const Path& cp, int t, const Scene& scene, Sampler& smp,
                              Vertex& sampled, bool& hasSampled) const {
    const Vertex& cv = cp.vertices[t - 1];
    if (cv.isSpecular || cv.si.material == nullptr) return {};
    LightSample ls;
    const Light* light;
    int idx;
    if (!sampleLight(scene.lights, *scene.lightSampler, cv.si.point, cv.si.normal, smp, ls, light, idx) ||
        ls.emission.isZero() || ls.pdf <= 0)
      return {};
    double cosTheta = ls.direction.absDot(cv.si.normal);
    if (cosTheta <= 0) return {};
    Vec3 brdf = cv.si.material->evaluateBRDF(cv.incomingDirection, ls.direction, &cv.si,
                                             TransportMode::Radiance);
    Vec3 lb = ls.emission.mul(1 / ls.pdf);
    Vec3 contrib = brdf.mulVec(cv.beta).mulVec(lb).mul(cosTheta);
    if (contrib.isZero()) return {};
    SurfaceInteraction tmp;
    if (scene.bvh->hit(Ray(cv.si.point, ls.direction), 0.001, ls.distance - 0.001, tmp)) return {};
    sampled = Vertex();
    sampled.si.point = ls.point;
    sampled.si.normal = ls.normal;
    sampled.light = light;
    sampled.lightIndex = idx;
    sampled.areaPdfForward = ls.pdf;
    sampled.areaPdfReverse = 0;
    sampled.isLight = true;
    sampled.isInfiniteLight = light->type() == LightType::Infinite;
    sampled.beta = lb;
    sampled.emittedLight = ls.emission;
    hasSampled = true;
    return contrib;
  }

  // evaluateLightTracingStrategy (bdpt.go:398-486)
  void lightTracingStrategy(const Path& lp, int s, const Scene& scene, Sampler& smp,
                            std::vector<SplatRay>& splats, Vertex& sampled, bool& hasSampled) const {
    if (s <= 1 || s > lp.length) return;
    const Vertex& lv = lp.vertices[s - 1];
    if (lv.isSpecular) return;
    CameraSample cs;
    if (!scene.camera->sampleCameraFromPoint(lv.si.point, smp.get2D(), cs)) return;
    Vec3 toCam = cs.ray.direction.mul(-1);
    Vec3 brdf = evaluateBRDF(lv, toCam, TransportMode::Importance);
    Vec3 cb = cs.weight.mul(1 / cs.pdf);
    double cosine = toCam.dot(lv.si.normal);
    if (cosine <= 0) return;
    Vec3 contrib = brdf.mulVec(cb).mulVec(lv.beta);
    if (lv.isOnSurface()) contrib = contrib.mul(cosine);
    if (contrib.isZero()) return;
    double dist = lv.si.point.sub(cs.ray.origin).length();
    SurfaceInteraction tmp;
    if (scene.bvh->hit(Ray(lv.si.point, toCam), 0.001, dist - 0.001, tmp)) return;
    Vec3 dirToLight = lv.si.point.sub(cs.ray.origin).normalize();
    double lpdf = calculateLightPDF(scene.lights, *scene.lightSampler, cs.ray.origin, toCam, dirToLight);
    sampled = Vertex();
    sampled.si.point = cs.ray.origin;
    sampled.si.normal = toCam;
    sampled.isCamera = true;
    sampled.beta = cb;
    sampled.areaPdfForward = cs.pdf;
    sampled.areaPdfReverse = lpdf;
    hasSampled = true;
    splats.push_back({cs.ray, contrib});
  }

  // evaluateConnectionStrategy (bdpt.go:502-561)
  Vec3 connectionStrategy(const Path& cp, const Path& lp, int s, int t, const Scene& scene) const {
    if (s < 1 || t < 1 || s > lp.length || t > cp.length) return {};
    const Vertex& lv = lp.vertices[s - 1];
    const Vertex& cv = cp.vertices[t - 1];
    if (lv.isSpecular || cv.isSpecular) return {};
    Vec3 d = lv.si.point.sub(cv.si.point);
    double dist = d.length();
    if (dist < 0.001) return {};
    d = d.mul(1.0 / dist);
    double cc = d.dot(cv.si.normal);
    double cl = d.mul(-1).dot(lv.si.normal);
    if (cc <= 0 || cl <= 0) return {};
    double g = (cc * cl) / (dist * dist);
    Vec3 cb = evaluateBRDF(cv, d, TransportMode::Radiance);
    Vec3 lb = evaluateBRDF(lv, d.mul(-1), TransportMode::Importance);
    Vec3 contrib = lv.beta.mulVec(lb).mulVec(cb).mulVec(cv.beta).mul(g);
    if (contrib.isZero()) return {};
    SurfaceInteraction tmp;
    if (scene.bvh->hit(Ray(cv.si.point, d), 0.001, dist - 0.001, tmp)) return {};
    return contrib;
  }

  // evaluateBRDF (bdpt.go:564-583)
  Vec3 evaluateBRDF(const Vertex& v, const Vec3& out, TransportMode mode) const {
    if (v.isInfiniteLight) return {};
    if (v.isLight && v.si.material == nullptr) return {1, 1, 1};
    if (v.si.material == nullptr) return {};
    return v.si.material->evaluateBRDF(v.incomingDirection, out, &v.si, mode);
  }

  // createBackgroundVertex (bdpt.go:585-601)
  static Vertex backgroundVertex(const Ray& ray, const Vec3& bg, const Vec3& beta, double pdfFwd) {
    Vertex v;
    v.si.point = ray.origin.add(ray.direction.mul(1000.0));
    v.si.normal = ray.direction.mul(-1);
    v.incomingDirection = ray.direction.mul(-1);
    v.areaPdfForward = pdfFwd;
    v.areaPdfReverse = 0.0;
    v.isLight = !bg.isZero();
    v.isInfiniteLight = true;
    v.beta = beta;
    v.emittedLight = bg;
    return v;
  }

  // calculateMISWeight (bdpt_mis.go:13-57)
  double misWeight(const Path& cp, const Path& lp, const Vertex* sampled, int s, int t,
                   const Scene& scene) const {
    if (s + t == 2) return 1.0;
    double sum = 0, ri = 1.0;
    for (int i = t - 1; i > 0; i--) {
      double f, r;
      bool c;
      cameraVertexPdfs(i, cp, lp, sampled, s, t, scene, f, r, c);
      ri *= remap0(r) / remap0(f);
      if (c) sum += ri;
    }
    ri = 1.0;
    for (int i = s - 1; i >= 0; i--) {
      double f, r;
      bool c;
      lightVertexPdfs(i, cp, lp, sampled, s, t, scene, f, r, c);
      ri *= remap0(r) / remap0(f);
      if (c) sum += ri;
    }
    return 1.0 / (1.0 + sum);
  }

  // calculateMISCameraVertexPdfs (bdpt_mis.go:61-119)
  void cameraVertexPdfs(int i, const Path& cp, const Path& lp, const Vertex* sampled, int s, int t,
                        const Scene& scene, double& fwd, double& rev, bool& conn) const {
    const Vertex& v = cp.vertices[i];
    fwd = v.areaPdfForward;
    rev = v.areaPdfReverse;
    conn = !v.isSpecular;
    if (s == 0) {
      if (i == t - 1 && t > 1) {
        rev = lightOriginPdf(cp.vertices[t - 1], cp.vertices[t - 2], scene);
        conn = true;
      } else if (i == t - 2 && t > 2) {
        rev = vertexPdf(cp.vertices[t - 1], nullptr, cp.vertices[t - 2], scene);
      }
    } else if (t == 1) {
      if (i == 0) {
        fwd = sampled->areaPdfForward;
        rev = sampled->areaPdfReverse;
        conn = true;
      }
    } else if (s == 1) {
      if (i == t - 1 && t > 0) {
        rev = vertexPdf(*sampled, nullptr, cp.vertices[t - 1], scene);
        conn = true;
      } else if (i == t - 2 && t > 1) {
        rev = vertexPdf(cp.vertices[t - 1], sampled, cp.vertices[t - 2], scene);
      }
    } else {
      if (i == t - 1) {
        rev = vertexPdf(lp.vertices[s - 1], &lp.vertices[s - 2], cp.vertices[t - 1], scene);
        conn = true;
      } else if (i == t - 2 && t > 1) {
        rev = vertexPdf(cp.vertices[t - 1], &lp.vertices[s - 1], cp.vertices[t - 2], scene);
      }
    }
    if (i > 0) conn = conn && !cp.vertices[i - 1].isSpecular;
  }

  // calculateMISLightVertexPdfs (bdpt_mis.go:123-181)
  void lightVertexPdfs(int i, const Path& cp, const Path& lp, const Vertex* sampled, int s, int t,
                       const Scene& scene, double& fwd, double& rev, bool& conn) const {
    const Vertex& v = lp.vertices[i];
    fwd = v.areaPdfForward;
    rev = v.areaPdfReverse;
    bool deltaLight = v.isLight && v.light != nullptr && v.light->type() == LightType::Point;
    conn = !v.isSpecular && !deltaLight;
    if (i > 0) {
      const Vertex& p = lp.vertices[i - 1];
      bool pd = p.isLight && p.light != nullptr && p.light->type() == LightType::Point;
      conn = conn && (!p.isSpecular && !pd);
    }
    if (s == 0) {
    } else if (t == 1) {
      if (i == s - 1 && s > 1) {
        rev = vertexPdf(*sampled, nullptr, lp.vertices[s - 1], scene);
        conn = true;
      } else if (i == s - 2 && s > 1) {
        rev = vertexPdf(lp.vertices[s - 1], sampled, lp.vertices[s - 2], scene);
      }
    } else if (s == 1) {
      if (i == s - 1 && sampled != nullptr) {
        fwd = sampled->areaPdfForward;
        rev = vertexPdf(cp.vertices[t - 1], &cp.vertices[t - 2], *sampled, scene);
        conn = true;
      }
    } else {
      if (i == s - 1) {
        rev = vertexPdf(cp.vertices[t - 1], &cp.vertices[t - 2], lp.vertices[s - 1], scene);
        conn = true;
      } else if (i == s - 2 && s > 1) {
        rev = vertexPdf(lp.vertices[s - 1], &cp.vertices[t - 1], lp.vertices[s - 2], scene);
      }
    }
  }

  // calculateVertexPdf (bdpt_mis.go:186-236)
  double vertexPdf(const Vertex& curr, const Vertex* prev, const Vertex& next, const Scene& scene) const {
    if (curr.isLight) return lightPdf(curr, next, scene);
    Vec3 wn = next.si.point.sub(curr.si.point);
    if (wn.lengthSquared() == 0) return 0;
    wn = wn.normalize();
    Vec3 wp;
    if (prev != nullptr) {
      wp = prev->si.point.sub(curr.si.point);
      if (wp.lengthSquared() == 0) return 0;
      wp = wp.normalize();
    } else if (!curr.isCamera) {
      return 0;
    }
    double pdf;
    if (curr.isCamera) {
      double a;
      scene.camera->calculateRayPDFs(Ray(curr.si.point, wn), a, pdf);
      if (pdf == 0) return 0;
    } else if (curr.si.material != nullptr) {
      bool d;
      double mp = curr.si.material->pdf(wp, wn, curr.si.normal, d);
      if (d) return 0;
      pdf = mp;
    } else {
      return 0;
    }
    return curr.convertSolidAngleToAreaPdf(next, pdf);
  }

  // calculateLightPdf (bdpt_mis.go:239-272)
  double lightPdf(const Vertex& curr, const Vertex& to, const Scene& scene) const {
    Vec3 w = to.si.point.sub(curr.si.point);
    double inv = 1.0 / w.lengthSquared();
    w = w.mul(std::sqrt(inv));
    double pdf = 0;
    if (curr.isLight) {
      if (curr.isInfiniteLight) {
        double r = scene.bvh->radius;
        if (r == 0.0) r = 1.0;
        pdf = 1.0 / (kPi * r * r);
      } else if (curr.light != nullptr) {
        double pp, pd;
        curr.light->pdfLe(curr.si.point, w, pp, pd);
        pdf = pd * inv;
      }
    }
    if (to.isOnSurface()) pdf *= to.si.normal.absDot(w);
    return pdf;
  }

  // calculateLightOriginPdf (bdpt_mis.go:275-308)
  double lightOriginPdf(const Vertex& lv, const Vertex& to, const Scene& scene) const {
    Vec3 w = to.si.point.sub(lv.si.point);
    if (w.lengthSquared() == 0) return 0;
    w = w.normalize();
    if (lv.isInfiniteLight) return infiniteLightDensity(to.si.point, to.si.normal, w.mul(-1), scene);
    if (!lv.isLight || lv.light == nullptr) return 0;
    if (scene.lights.empty()) return 0;
    double choice = scene.lightSampler->probability(lv.lightIndex);
    double pp, pd;
    lv.light->pdfLe(lv.si.point, w, pp, pd);
    return pp * choice;
  }

  // calculateInfiniteLightDensity (bdpt_mis.go:313-335)
  double infiniteLightDensity(const Vec3& p, const Vec3& n, const Vec3& dir, const Scene& scene) const {
    if (scene.lights.empty()) return 0;
    double total = 0;
    for (size_t i = 0; i < scene.lights.size(); i++) {
      const Light* l = scene.lights[i];
      if (l->type() == LightType::Infinite)
        total += l->pdf(p, n, dir) * scene.lightSampler->probability((int)i);
    }
    return total;
  }
};

}  // namespace ref
