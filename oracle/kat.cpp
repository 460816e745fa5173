// kat.cpp - the reference's own known-answer tests, restated against the
// oracle.  TEST INFRASTRUCTURE ONLY.  Each case names the Go test
// (file:line, relative to the reference project root) whose inputs and
// expected values it uses; the fixtures mirror that test's helper functions.
// Output: one line per case, "PASS <name>" or "FAIL <name>: <detail>";
// exit status 0 when every case passes.
#include <cstdio>
#include <functional>
#include <sstream>

#include "oracle.hpp"

using namespace ref;

namespace {

int g_fail = 0, g_pass = 0;
std::string g_detail;

void check(bool ok, const std::string& name) {
  if (ok) {
    g_pass++;
    std::printf("PASS %s\n", name.c_str());
  } else {
    g_fail++;
    std::printf("FAIL %s: %s\n", name.c_str(), g_detail.c_str());
  }
  g_detail.clear();
}

bool near(double a, double b, double tol) {
  if (std::fabs(a - b) <= tol) return true;
  std::ostringstream o;
  o.precision(12);
  o << "got " << a << " want " << b << " tol " << tol;
  g_detail = o.str();
  return false;
}
bool nearV(const Vec3& a, const Vec3& b, double tol) {
  return near(a.x, b.x, tol) && near(a.y, b.y, tol) && near(a.z, b.z, tol);
}

// ---------------------------------------------------------------- fixtures
// Scene helpers of the Go tests, built with the oracle's types.
struct TestScene {
  std::unique_ptr<Scene> s = std::make_unique<Scene>();
  const Material* add(std::unique_ptr<Material> m) {
    s->materials.push_back(std::move(m));
    return s->materials.back().get();
  }
  template <class T>
  T* shape(std::unique_ptr<T> sh) {
    T* p = sh.get();
    p->id = (int)s->shapes.size();
    s->shapes.push_back(p);
    s->ownedShapes.push_back(std::move(sh));
    return p;
  }
  void light(std::unique_ptr<Light> l) {
    s->lights.push_back(l.get());
    s->ownedLights.push_back(std::move(l));
  }
};

CameraConfig cam(Vec3 c, Vec3 la, int w, double aspect, double vfov, double ap = 0, double fd = 0) {
  CameraConfig cc;
  cc.center = c;
  cc.lookAt = la;
  cc.up = Vec3(0, 1, 0);
  cc.width = w;
  cc.aspectRatio = aspect;
  cc.vfov = vfov;
  cc.aperture = ap;
  cc.focusDistance = fd;
  return cc;
}

// createSimpleTestScene (pkg/integrator/bdpt_test.go:280-320)
std::unique_ptr<TestScene> simpleTestScene() {
  auto t = std::make_unique<TestScene>();
  auto white = t->add(std::make_unique<Lambertian>(Vec3(0.7, 0.7, 0.7)));
  auto em = t->add(std::make_unique<Emissive>(Vec3(5, 5, 5)));
  t->shape(std::make_unique<Sphere>(Vec3(0, 0, -1), 0.5, white));
  auto q = t->shape(std::make_unique<Quad>(Vec3(-0.5, 2.0, -0.5), Vec3(1, 0, 0), Vec3(0, 0, 1), em));
  t->light(std::make_unique<QuadLight>(q));
  t->s->camera = std::make_unique<Camera>(cam(Vec3(0, 0, 0), Vec3(0, 0, -1), 100, 1.0, 45.0));
  t->s->sampling.maxDepth = 5;
  t->s->lightSampler = std::make_unique<LightSampler>(LightSampler::uniform(t->s->lights));
  t->s->preprocess();
  return t;
}

// createSceneWithLightsAndWeights (bdpt_test.go:323-361), quad lights only
std::unique_ptr<TestScene> sceneWithQuadLights(const std::vector<std::pair<Quad*, const Material*>>&,
                                               std::unique_ptr<TestScene> t, const std::vector<double>& w) {
  auto white = t->add(std::make_unique<Lambertian>(Vec3(0.7, 0.7, 0.7)));
  // the sphere is the first shape; lights' quads follow in light order
  auto sph = std::make_unique<Sphere>(Vec3(0, 0, -5), 0.5, white);
  std::vector<const Shape*> shapes;
  sph->id = 0;
  shapes.push_back(sph.get());
  t->s->ownedShapes.insert(t->s->ownedShapes.begin(), std::move(sph));
  for (auto* sh : t->s->shapes) shapes.push_back(sh);
  t->s->shapes = shapes;
  for (size_t i = 0; i < t->s->shapes.size(); i++) const_cast<Shape*>(t->s->shapes[i])->id = (int)i;
  t->s->camera = std::make_unique<Camera>(cam(Vec3(0, 0, 0), Vec3(0, 0, -1), 100, 1.0, 45.0));
  t->s->sampling.maxDepth = 5;
  if (!w.empty()) t->s->lightSampler = std::make_unique<LightSampler>(LightSampler::weighted(t->s->lights, w));
  else t->s->lightSampler = std::make_unique<LightSampler>(LightSampler::uniform(t->s->lights));
  t->s->preprocess();
  return t;
}

std::unique_ptr<TestScene> sceneWithQuadLight(Vec3 corner, Vec3 u, Vec3 v, Vec3 e) {
  auto t = std::make_unique<TestScene>();
  auto em = t->add(std::make_unique<Emissive>(e));
  auto q = t->shape(std::make_unique<Quad>(corner, u, v, em));
  t->light(std::make_unique<QuadLight>(q));
  return sceneWithQuadLights({}, std::move(t), {});
}

// createTestAreaLight (bdpt_test.go:369-377): 4x4 quad at y=2, normal down
struct AreaLightHolder {
  std::unique_ptr<Material> em = std::make_unique<Emissive>(Vec3(5, 5, 5));
  std::unique_ptr<Quad> q = std::make_unique<Quad>(Vec3(-2, 2, -3), Vec3(4, 0, 0), Vec3(0, 0, 4), em.get());
  std::unique_ptr<QuadLight> l = std::make_unique<QuadLight>(q.get());
};
AreaLightHolder& testAreaLight() {
  static AreaLightHolder h;
  return h;
}

// createGlancingTestSceneWithMaterial (bdpt_test.go:379-407).  The reference
// scene also holds a point spot light; camera subpaths only consult
// infinite lights, so it does not affect the cases that use this fixture.
std::unique_ptr<TestScene> glancingScene(std::unique_ptr<Material> m) {
  auto t = std::make_unique<TestScene>();
  auto mm = t->add(std::move(m));
  t->shape(std::make_unique<Sphere>(Vec3(0, 0, -2), 1.0, mm));
  t->s->camera = std::make_unique<Camera>(cam(Vec3(0, 0, 0), Vec3(0, 0, -1), 100, 1.0, 45.0));
  t->s->sampling.maxDepth = 5;
  t->s->lightSampler = std::make_unique<LightSampler>(LightSampler::uniform(t->s->lights));
  t->s->preprocess();
  return t;
}

// createLightSceneWithMaterial (bdpt_test.go:420-453)
std::unique_ptr<TestScene> lightScene(std::unique_ptr<Material> m) {
  auto t = std::make_unique<TestScene>();
  auto mm = t->add(std::move(m));
  auto black = t->add(std::make_unique<Lambertian>(Vec3(0, 0, 0)));
  auto em = t->add(std::make_unique<Emissive>(Vec3(5, 5, 5)));
  t->shape(std::make_unique<Sphere>(Vec3(0, -1.5, 0), 0.8, mm));
  t->shape(std::make_unique<Sphere>(Vec3(0, 0, 0), 10.0, black));
  // the quad light's geometry is not in Shapes in this fixture
  static std::vector<std::unique_ptr<Quad>> keep;
  keep.push_back(std::make_unique<Quad>(Vec3(-0.5, 1.0, -0.5), Vec3(1, 0, 0), Vec3(0, 0, 1), em));
  t->light(std::make_unique<QuadLight>(keep.back().get()));
  t->s->camera = std::make_unique<Camera>(cam(Vec3(3, 0, 0), Vec3(0, 0, 0), 100, 1.0, 45.0));
  t->s->sampling.maxDepth = 5;
  t->s->lightSampler = std::make_unique<LightSampler>(LightSampler::uniform(t->s->lights));
  t->s->preprocess();
  return t;
}

// createMinimalCornellScene(false) (bdpt_test.go:872-989)
std::unique_ptr<TestScene> minimalCornell() {
  auto t = std::make_unique<TestScene>();
  auto white = t->add(std::make_unique<Lambertian>(Vec3(0.73, 0.73, 0.73)));
  auto red = t->add(std::make_unique<Lambertian>(Vec3(0.65, 0.05, 0.05)));
  auto green = t->add(std::make_unique<Lambertian>(Vec3(0.12, 0.45, 0.15)));
  t->shape(std::make_unique<Quad>(Vec3(0, 0, 0), Vec3(556, 0, 0), Vec3(0, 0, 556), white));
  t->shape(std::make_unique<Quad>(Vec3(0, 556, 0), Vec3(556, 0, 0), Vec3(0, 0, 556), white));
  t->shape(std::make_unique<Quad>(Vec3(0, 0, 556), Vec3(556, 0, 0), Vec3(0, 556, 0), white));
  t->shape(std::make_unique<Quad>(Vec3(0, 0, 0), Vec3(0, 0, 556), Vec3(0, 556, 0), red));
  t->shape(std::make_unique<Quad>(Vec3(556, 0, 0), Vec3(0, 0, 556), Vec3(0, 556, 0), green));
  auto em = t->add(std::make_unique<Emissive>(Vec3(18, 15, 8).mul(2.5)));
  auto q = t->shape(std::make_unique<Quad>(Vec3(213, 556 - 0.001, 227), Vec3(130, 0, 0), Vec3(0, 0, 105), em));
  t->light(std::make_unique<QuadLight>(q));
  t->s->camera = std::make_unique<Camera>(cam(Vec3(278, 278, -800), Vec3(278, 278, 0), 400, 1.0, 40.0));
  t->s->lightSampler = std::make_unique<LightSampler>(LightSampler::uniform(t->s->lights));
  t->s->preprocess();
  return t;
}

// createTestVertex (bdpt_test.go:455-470)
Vertex testVertex(Vec3 p, Vec3 n, bool isLight, bool isCamera, const Material* m) {
  Vertex v;
  v.si.point = p;
  v.si.normal = n;
  v.si.material = m;
  v.isLight = isLight;
  v.isCamera = isCamera;
  v.isSpecular = false;
  v.beta = Vec3(1, 1, 1);
  v.areaPdfForward = 1.0;
  v.areaPdfReverse = 1.0;
  v.emittedLight = Vec3();
  v.incomingDirection = Vec3(0, 0, 1);
  return v;
}

bool isSpecularMat(const Material* m) {
  return dynamic_cast<const Metal*>(m) || dynamic_cast<const Dielectric*>(m);
}

// createTestCameraPathWithLight (bdpt_test.go:728-786)
Path testCameraPath(const std::vector<const Material*>& mats, const std::vector<Vec3>& pos,
                    const Light* hitLight = nullptr) {
  Path p;
  Vertex c;
  c.si.point = pos[0];
  c.si.normal = Vec3(0, 0, 1);
  c.isCamera = true;
  c.beta = Vec3(1, 1, 1);
  c.areaPdfForward = 1.0;
  p.vertices.push_back(c);
  for (size_t i = 1; i < pos.size(); i++) {
    const Material* m = mats[i - 1];
    Vertex v;
    v.si.point = pos[i];
    v.si.normal = Vec3(0, 1, 0);
    v.si.material = m;
    v.isSpecular = isSpecularMat(m);
    v.isLight = m->isEmitter();
    v.beta = Vec3(0.7, 0.7, 0.7);
    v.areaPdfForward = 1.0 / kPi;
    v.areaPdfReverse = 1.0 / kPi;
    if (i == pos.size() - 1 && v.isLight && hitLight) {
      v.light = hitLight;
      v.lightIndex = 0;
      Ray in = rayTo(pos[i - 1], pos[i]);
      v.emittedLight = m->emit(in, &v.si);
    }
    p.vertices.push_back(v);
  }
  p.length = (int)p.vertices.size();
  return p;
}

// createTestLightPath (bdpt_test.go:788-842)
Path testLightPath(const std::vector<const Material*>& mats, const std::vector<Vec3>& pos) {
  Path p;
  const QuadLight* l = testAreaLight().l.get();
  double pp, pd;
  l->pdfLe(pos[0], Vec3(0, -1, 0), pp, pd);
  Vertex v0;
  v0.si.point = pos[0];
  v0.si.normal = Vec3(0, -1, 0);
  v0.si.material = mats[0];
  v0.isLight = true;
  v0.light = l;
  v0.lightIndex = 0;
  v0.beta = Vec3(1, 1, 1);
  v0.areaPdfForward = pp;
  v0.emittedLight = Vec3(5, 5, 5);
  p.vertices.push_back(v0);
  for (size_t i = 1; i < pos.size(); i++) {
    Vertex v;
    v.si.point = pos[i];
    v.si.normal = Vec3(0, 1, 0);
    v.si.material = mats[i];
    v.isSpecular = isSpecularMat(mats[i]);
    v.beta = Vec3(0.7, 0.7, 0.7);
    v.areaPdfForward = 1.0 / kPi;
    v.areaPdfReverse = 1.0 / kPi;
    p.vertices.push_back(v);
  }
  p.length = (int)p.vertices.size();
  return p;
}

// createSampledLightVertex (bdpt_mis_test.go:965-985)
Vertex sampledLightVertex(const Material* em) {
  Vertex v;
  v.si.point = Vec3(0, 2, -1);
  v.si.normal = Vec3(0, -1, 0);
  v.si.material = em;
  v.light = testAreaLight().l.get();
  v.beta = Vec3(5, 5, 5);
  v.areaPdfForward = 1.0;
  v.areaPdfReverse = 0.0;
  v.isLight = true;
  v.emittedLight = Vec3(5, 5, 5);
  return v;
}

struct MockShape : Shape {  // bvh_test.go:12-23
  AABB b;
  explicit MockShape(AABB bb) : b(bb) {}
  bool hit(const Ray&, double, double, SurfaceInteraction&) const override { return false; }
  AABB boundingBox() const override { return b; }
};

// ---------------------------------------------------------------- geometry
void geometryTests() {
  Lambertian grey(Vec3(0.5, 0.5, 0.5));
  SurfaceInteraction h;
  {  // TestTriangle_Hit (pkg/geometry/triangle_test.go:11-108)
    Triangle tri(Vec3(0, 0, 0), Vec3(1, 0, 0), Vec3(0, 1, 0), &grey);
    struct C { const char* n; Ray r; bool hit; double t; };
    C cs[] = {{"center", Ray(Vec3(0.25, 0.25, -1), Vec3(0, 0, 1)), true, 1.0},
              {"edge", Ray(Vec3(0.5, 0, -1), Vec3(0, 0, 1)), true, 1.0},
              {"miss", Ray(Vec3(1, 1, -1), Vec3(0, 0, 1)), false, 0},
              {"parallel", Ray(Vec3(0.25, 0.25, 0), Vec3(1, 0, 0)), false, 0},
              {"behind", Ray(Vec3(0.25, 0.25, 1), Vec3(0, 0, -1)), true, 1.0}};
    for (auto& c : cs) {
      bool hit = tri.hit(c.r, 0.001, 10.0, h);
      bool ok = hit == c.hit;
      if (!ok) g_detail = "hit mismatch";
      if (ok && hit) ok = near(h.t, c.t, 1e-6) && near(c.r.at(h.t).sub(h.point).length(), 0, 1e-6);
      check(ok, std::string("triangle_test.go:11 TestTriangle_Hit/") + c.n);
    }
  }
  {  // TestQuad_Hit_* (pkg/geometry/quad_test.go:12-125)
    Quad q(Vec3(0, 0, 0), Vec3(1, 0, 0), Vec3(0, 0, 1), &grey);
    bool hit = q.hit(Ray(Vec3(0.5, 1, 0.5), Vec3(0, -1, 0)), 0.001, 1000.0, h);
    check(hit && near(h.t, 1.0, 1e-9) && nearV(h.point, Vec3(0.5, 0, 0.5), 1e-9),
          "quad_test.go:12 TestQuad_Hit_BasicIntersection");
    Vec3 outs[] = {{-0.5, 1, 0.5}, {1.5, 1, 0.5}, {0.5, 1, -0.5}, {0.5, 1, 1.5}};
    bool allMiss = true;
    for (auto& o : outs) allMiss &= !q.hit(Ray(o, Vec3(0, -1, 0)), 0.001, 1000.0, h);
    check(allMiss, "quad_test.go:41 TestQuad_Hit_OutsideBounds");
    Vec3 corners[] = {{0, 0, 0}, {1, 0, 0}, {0, 0, 1}, {1, 0, 1}};
    bool allHit = true;
    for (auto& c : corners) allHit &= q.hit(Ray(c.add(Vec3(0, 1, 0)), Vec3(0, -1, 0)), 0.001, 1000.0, h);
    check(allHit, "quad_test.go:86 TestQuad_Hit_CornerHits");
    check(!q.hit(Ray(Vec3(0.5, 1, 0.5), Vec3(1, 0, 0)), 0.001, 1000.0, h), "quad_test.go:111 TestQuad_Hit_ParallelRay");
    AABB b = q.boundingBox();  // TestAxisAlignedQuadBoundingBox (quad_test.go:175): thin Y slab
    check(near(b.min.y, -0.001, 1e-12) && near(b.max.y, 0.001, 1e-12) && near(b.max.x, 1, 1e-12),
          "quad_test.go:175 TestAxisAlignedQuadBoundingBox");
  }
  {  // TestSphere_Hit_* (pkg/geometry/sphere_test.go:11-130)
    Sphere s(Vec3(0, 0, 0), 1.0, &grey);
    check(!s.hit(Ray(Vec3(0, 2, 2), Vec3(0, 0, -1)), 0.001, 1000.0, h), "sphere_test.go:11 TestSphere_Hit_Miss");
    bool hit = s.hit(Ray(Vec3(0, 0, 2), Vec3(0, 0, -1)), 0.001, 1000.0, h);
    check(hit && near(h.t, 1.0, 1e-9) && h.frontFace && nearV(h.normal, Vec3(0, 0, 1), 1e-9),
          "sphere_test.go:22 TestSphere_Hit_FrontAndBackFace/front");
    hit = s.hit(Ray(Vec3(0, 0, 0), Vec3(0, 0, 1)), 0.001, 1000.0, h);
    check(hit && near(h.t, 1.0, 1e-9) && !h.frontFace && nearV(h.normal, Vec3(0, 0, -1), 1e-9),
          "sphere_test.go:22 TestSphere_Hit_FrontAndBackFace/back");
    hit = s.hit(Ray(Vec3(1, 0, 2), Vec3(0, 0, -1)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(1, 0, 0), 1e-9), "sphere_test.go:78 TestSphere_Hit_GlancingHit");
    Ray r(Vec3(0, 0, 2), Vec3(0, 0, -1));
    check(!s.hit(r, 0.001, 0.5, h) && !s.hit(r, 3.5, 1000.0, h), "sphere_test.go:96 TestSphere_Hit_Bounds");
    hit = s.hit(r, 0.001, 1000.0, h);
    check(hit && near(h.t, 1.0, 1e-9) && h.frontFace, "sphere_test.go:113 TestSphere_Hit_ClosestIntersection");
  }
  {  // TestBox_Hit_AxisAligned / Rotated (pkg/geometry/box_test.go:48-222)
    Box b(Vec3(0, 0, 0), Vec3(1, 1, 1), Vec3(0, 0, 0), &grey);
    struct C { const char* n; Ray r; bool hit; double t; };
    C cs[] = {{"front", Ray(Vec3(0, 0, -3), Vec3(0, 0, 1)), true, 2.0},
              {"right", Ray(Vec3(-3, 0, 0), Vec3(1, 0, 0)), true, 2.0},
              {"miss", Ray(Vec3(0, 3, -3), Vec3(0, 0, 1)), false, 0},
              {"inside", Ray(Vec3(0, 0, 0), Vec3(1, 0, 0)), true, 1.0}};
    for (auto& c : cs) {
      bool hit = b.hit(c.r, 0.001, 10.0, h);
      bool ok = hit == c.hit;
      if (!ok) g_detail = "hit mismatch";
      if (ok && hit) ok = near(h.t, c.t, 1e-6);
      check(ok, std::string("box_test.go:48 TestBox_Hit_AxisAligned/") + c.n);
    }
    Box rb(Vec3(0, 0, 0), Vec3(1, 1, 1), Vec3(0, kPi / 4, 0), &grey);
    Ray r(Vec3(0, 0, -3), Vec3(0, 0, 1));
    bool hit = rb.hit(r, 0.001, 10.0, h);
    // the 45-degree box presents its vertical edge at z = -sqrt(2)
    check(hit && h.t > 0 && h.t < 10 && near(r.at(h.t).sub(h.point).length(), 0, 1e-6) &&
              near(h.t, 3 - std::sqrt(2.0), 1e-9),
          "box_test.go:185 TestBox_Hit_Rotated");
  }
  {  // TestWorldRadius (pkg/geometry/bvh_test.go:251-331)
    struct C { const char* n; std::vector<AABB> boxes; Vec3 c; double r, tol; };
    C cs[] = {{"EmptyScene", {}, Vec3(), 0.0, 0.0},
              {"SingleSphere", {AABB(Vec3(-1, -1, -1), Vec3(1, 1, 1))}, Vec3(), std::sqrt(3.0), 1e-10},
              {"SceneWithInfinitePlane",
               {AABB(Vec3(-1, -1, -1), Vec3(1, 1, 1)), AABB(Vec3(-1e6, -0.1, -1e6), Vec3(1e6, 0.1, 1e6))},
               Vec3(),
               std::sqrt(2e12),
               1e-6},
              {"OnlyInfinitePlanes", {AABB(Vec3(-1e6, -0.1, -1e6), Vec3(1e6, 0.1, 1e6))}, Vec3(), std::sqrt(2e12), 1e-6}};
    for (auto& c : cs) {
      std::vector<std::unique_ptr<MockShape>> own;
      std::vector<const Shape*> shapes;
      for (auto& b : c.boxes) {
        own.push_back(std::make_unique<MockShape>(b));
        shapes.push_back(own.back().get());
      }
      BVH bvh(shapes);
      check(near(bvh.radius, c.r, c.tol) && nearV(bvh.center, c.c, c.tol), std::string("bvh_test.go:251 TestWorldRadius/") + c.n);
    }
  }
  {  // TestBVH_MultipleHitsInLeaf-style closest-hit through the binary BVH
    // (pkg/geometry/bvh_test.go:105-146): spheres along a line, the nearest wins
    std::vector<std::unique_ptr<Sphere>> own;
    std::vector<const Shape*> shapes;
    for (int i = 0; i < 20; i++) {
      own.push_back(std::make_unique<Sphere>(Vec3(0, 0, -2.0 * i - 3), 0.5, &grey));
      own.back()->id = i;
      shapes.push_back(own.back().get());
    }
    BVH bvh(shapes);
    bool hit = bvh.hit(Ray(Vec3(0, 0, 0), Vec3(0, 0, -1)), 0.001, kInf, h);
    check(hit && h.shape == 0 && near(h.t, 2.5, 1e-12), "bvh_test.go:105 TestBVH_MultipleHitsInLeaf (closest of 20)");
  }
  {  // TestWeFunction (pkg/geometry/camera_splat_test.go:179-263)
    Camera c(cam(Vec3(0, 0, 0), Vec3(0, 0, -1), 800, 16.0 / 9.0, 90, 0.1, 1.0));
    Ray center(Vec3(0, 0, 0), Vec3(0, 0, -1));
    Vec3 ed = Vec3(0.7, 0, -0.7).normalize();
    Vec3 cw = c.evaluateRayImportance(center), ew = c.evaluateRayImportance(Ray(Vec3(), ed));
    double cc = center.direction.dot(c.forward), ec = ed.dot(c.forward);
    double ratio = (cc * cc * cc * cc) / (ec * ec * ec * ec);
    bool ok = cw.luminance() > 0 && ew.luminance() > cw.luminance() && near(ew.luminance() / cw.luminance(), ratio, 0.01) &&
              c.evaluateRayImportance(Ray(Vec3(), Vec3(5, 0, -1).normalize())).luminance() == 0 &&
              c.evaluateRayImportance(Ray(Vec3(), Vec3(0, 0, 1))).luminance() == 0;
    check(ok, "camera_splat_test.go:179 TestWeFunction");
  }
  {  // TestMapRayToPixel (pkg/geometry/camera_splat_test.go:86-146)
    Camera c(cam(Vec3(0, 0, 0), Vec3(0, 0, -1), 800, 16.0 / 9.0, 90, 0.0, 1.0));
    PcgSampler s(42, 0);
    int px[5][2] = {{400, 225}, {0, 0}, {799, 0}, {0, 449}, {799, 449}};
    int tol[5] = {2, 5, 5, 5, 5};
    bool ok = true;
    for (int k = 0; k < 5; k++) {
      Vec2 a = s.get2D(), b = s.get2D();
      Ray r = c.getRay(px[k][0], px[k][1], a, b);
      int x, y;
      ok &= c.mapRayToPixel(r, x, y) && std::abs(x - px[k][0]) <= tol[k] && std::abs(y - px[k][1]) <= tol[k];
    }
    check(ok, "camera_splat_test.go:86 TestMapRayToPixel");
  }
  {  // TestCameraCalculateRayPDFs_InvalidRay (pkg/geometry/camera_test.go:98-113)
    Camera c(cam(Vec3(0, 0, 0), Vec3(0, 0, -1), 400, 1.0, 45.0));
    double a, d;
    c.calculateRayPDFs(Ray(Vec3(), Vec3(0, 0, 1)), a, d);
    double a2, d2, a3, d3;
    c.calculateRayPDFs(Ray(Vec3(), Vec3(0, 0, -1)), a2, d2);
    c.calculateRayPDFs(Ray(Vec3(), Vec3(0.5, 0, -1).normalize()), a3, d3);
    check(a == 0 && d == 0 && d2 > d3 && a2 > 0, "camera_test.go:67,98 TestCameraCalculateRayPDFs_{DirectionPDF,InvalidRay}");
  }
}

// ---------------------------------------------------------------- materials and lights
// Disc, cylinder and cone (pkg/geometry/disc_test.go, cylinder_test.go,
// cone_test.go): the hit / miss cases, distances, points and normals.
void quadricTests() {
  Lambertian grey(Vec3(0.5, 0.5, 0.5));
  SurfaceInteraction h;
  {  // TestDiscHit (disc_test.go:12-89), TestDiscBoundingBox (:91-117)
    Disc d(Vec3(0, 0, 0), Vec3(0, 1, 0), 1.0, &grey);
    struct C { const char* n; Ray r; bool hit; };
    C cs[] = {{"center", Ray(Vec3(0, 1, 0), Vec3(0, -1, 0)), true},
              {"edge", Ray(Vec3(1, 1, 0), Vec3(0, -1, 0)), true},
              {"outside radius", Ray(Vec3(1.1, 1, 0), Vec3(0, -1, 0)), false},
              {"parallel", Ray(Vec3(0, 0, 0), Vec3(1, 0, 0)), false},
              {"from below", Ray(Vec3(0, -1, 0), Vec3(0, 1, 0)), true}};
    for (auto& c : cs) {
      bool hit = d.hit(c.r, 0.001, 10.0, h);
      bool ok = hit == c.hit;
      if (!ok) g_detail = "hit mismatch";
      if (ok && hit) ok = near(h.t, 1.0, 1e-6);
      check(ok, std::string("disc_test.go:12 TestDiscHit/") + c.n);
    }
    AABB b = d.boundingBox();
    check(nearV(b.min, Vec3(-1, 0, -1), 1e-9) && nearV(b.max, Vec3(1, 0, 1), 1e-9),
          "disc_test.go:91 TestDiscBoundingBox");
  }
  {  // cylinder_test.go:98-560
    Cylinder c(Vec3(0, 0, 0), Vec3(0, 2, 0), 1.0, false, &grey);
    bool hit = c.hit(Ray(Vec3(2, 1, 0), Vec3(-1, 0, 0)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(1, 1, 0), 1e-6) && nearV(h.normal, Vec3(1, 0, 0), 1e-6) && h.frontFace,
          "cylinder_test.go:98 TestCylinder_Hit_SimpleHit");
    check(!c.hit(Ray(Vec3(2, 1, 0), Vec3(0, 1, 0)), 0.001, 1000.0, h), "cylinder_test.go:137 TestCylinder_Hit_Miss");
    check(c.hit(Ray(Vec3(2, 1, 0), Vec3(-1, 0, 0)), 0.001, 1000.0, h) &&
              !c.hit(Ray(Vec3(2, 3, 0), Vec3(-1, 0, 0)), 0.001, 1000.0, h) &&
              !c.hit(Ray(Vec3(2, -1, 0), Vec3(-1, 0, 0)), 0.001, 1000.0, h),
          "cylinder_test.go:156 TestCylinder_Hit_HeightBounds");
    hit = c.hit(Ray(Vec3(0, 1, 0), Vec3(1, 0, 0)), 0.001, 1000.0, h);
    check(hit && !h.frontFace && nearV(h.normal, Vec3(-1, 0, 0), 1e-6), "cylinder_test.go:205 TestCylinder_Hit_FromInside");
    Cylinder cx(Vec3(0, 0, 0), Vec3(3, 0, 0), 1.0, false, &grey);
    hit = cx.hit(Ray(Vec3(1.5, 2, 0), Vec3(0, -1, 0)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(1.5, 1, 0), 1e-6) && nearV(h.normal, Vec3(0, 1, 0), 1e-6),
          "cylinder_test.go:238 TestCylinder_Hit_ArbitraryOrientation");
    hit = c.hit(Ray(Vec3(-2, 1, 0), Vec3(1, 0, 0)), 0.001, 1000.0, h);
    check(hit && near(h.t, 1.0, 1e-6) && nearV(h.point, Vec3(-1, 1, 0), 1e-6),
          "cylinder_test.go:273 TestCylinder_Hit_TwoIntersections");
    Ray r(Vec3(2, 1, 0), Vec3(-1, 0, 0));
    check(!c.hit(r, 0.001, 0.5, h) && !c.hit(r, 3.5, 1000.0, h) && c.hit(r, 0.001, 1000.0, h) && near(h.t, 1.0, 1e-6),
          "cylinder_test.go:304 TestCylinder_Hit_TBounds");
    Cylinder cc(Vec3(0, 0, 0), Vec3(0, 2, 0), 1.0, true, &grey);
    hit = cc.hit(Ray(Vec3(0.5, 3, 0), Vec3(0, -1, 0)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(0.5, 2, 0), 1e-6) && nearV(h.normal, Vec3(0, 1, 0), 1e-6),
          "cylinder_test.go:339 TestCylinder_Capped_HitTopCap");
    hit = cc.hit(Ray(Vec3(0.5, -1, 0), Vec3(0, 1, 0)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(0.5, 0, 0), 1e-6) && nearV(h.normal, Vec3(0, -1, 0), 1e-6),
          "cylinder_test.go:377 TestCylinder_Capped_HitBottomCap");
    check(!cc.hit(Ray(Vec3(1.5, 3, 0), Vec3(0, -1, 0)), 0.001, 1000.0, h),
          "cylinder_test.go:415 TestCylinder_Capped_MissOutsideCapRadius");
    check(!c.hit(Ray(Vec3(0.5, 3, 0), Vec3(0, -1, 0)), 0.001, 1000.0, h),
          "cylinder_test.go:521 TestCylinder_Uncapped_NoCapHits");
  }
  {  // cone_test.go:227-660
    Cone c(Vec3(0, 0, 0), 1.0, Vec3(0, 2, 0), 0.0, false, &grey);
    bool hit = c.hit(Ray(Vec3(2, 1, 0), Vec3(-1, 0, 0)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(0.5, 1, 0), 1e-6), "cone_test.go:227 TestCone_Hit_SimpleHit");
    check(!c.hit(Ray(Vec3(2, 1, 0), Vec3(0, 1, 0)), 0.001, 1000.0, h), "cone_test.go:263 TestCone_Hit_Miss");
    check(c.hit(Ray(Vec3(2, 1, 0), Vec3(-1, 0, 0)), 0.001, 1000.0, h) &&
              !c.hit(Ray(Vec3(2, 3, 0), Vec3(-1, 0, 0)), 0.001, 1000.0, h) &&
              !c.hit(Ray(Vec3(2, -1, 0), Vec3(-1, 0, 0)), 0.001, 1000.0, h),
          "cone_test.go:286 TestCone_Hit_HeightBounds");
    Cone f(Vec3(0, 0, 0), 2.0, Vec3(0, 4, 0), 1.0, false, &grey);
    hit = f.hit(Ray(Vec3(3, 2, 0), Vec3(-1, 0, 0)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(1.5, 2, 0), 1e-6), "cone_test.go:339 TestCone_Hit_Frustum");
    check(c.hit(Ray(Vec3(0, 1, 0), Vec3(1, 0, 0)), 0.001, 1000.0, h) && !h.frontFace,
          "cone_test.go:371 TestCone_Hit_FromInside");
    Ray r(Vec3(2, 1, 0), Vec3(-1, 0, 0));
    check(!c.hit(r, 0.001, 1.0, h) && !c.hit(r, 10.0, 1000.0, h), "cone_test.go:399 TestCone_Hit_TBounds");
    Cone cp(Vec3(0, 0, 0), 1.0, Vec3(0, 2, 0), 0.0, true, &grey);
    hit = cp.hit(Ray(Vec3(0.5, -1, 0), Vec3(0, 1, 0)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(0.5, 0, 0), 1e-6) && nearV(h.normal, Vec3(0, -1, 0), 1e-6),
          "cone_test.go:428 TestCone_Capped_HitBaseCap_Pointed");
    Cone fc(Vec3(0, 0, 0), 1.0, Vec3(0, 2, 0), 0.5, true, &grey);
    hit = fc.hit(Ray(Vec3(0.3, -1, 0), Vec3(0, 1, 0)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(0.3, 0, 0), 1e-6), "cone_test.go:467 TestCone_Capped_HitBaseCap_Frustum");
    hit = fc.hit(Ray(Vec3(0.2, 3, 0), Vec3(0, -1, 0)), 0.001, 1000.0, h);
    check(hit && nearV(h.point, Vec3(0.2, 2, 0), 1e-6) && nearV(h.normal, Vec3(0, 1, 0), 1e-6),
          "cone_test.go:497 TestCone_Capped_HitTopCap_Frustum");
    Cone fu(Vec3(0, 0, 0), 1.0, Vec3(0, 2, 0), 0.3, false, &grey);
    check(!c.hit(Ray(Vec3(2, -1, 0), Vec3(0, 1, 0)), 0.001, 1000.0, h) &&
              !fu.hit(Ray(Vec3(2, -1, 0), Vec3(0, 1, 0)), 0.001, 1000.0, h) &&
              !fu.hit(Ray(Vec3(0.2, 3, 0), Vec3(0, -1, 0)), 0.001, 1000.0, h),
          "cone_test.go:609 TestCone_Uncapped_NoCapHits");
  }
}

void materialLightTests() {
  {  // TestReflectanceFunction (pkg/material/dielectric_test.go:129-154)
    double r0 = reflectance(1.0, 1.0 / 1.5), r90 = reflectance(0.0, 1.0 / 1.5), r45 = reflectance(0.707, 1.0 / 1.5);
    check(r0 >= 0.03 && r0 <= 0.06 && r90 >= 0.95 && r45 > r0 && r45 <= 0.2 && r90 > r45,
          "dielectric_test.go:129 TestReflectanceFunction");
  }
  {  // TestDielectricEvaluateBRDF_Refraction_TransportModes (dielectric_test.go:194-233)
    Dielectric g(1.5);
    SurfaceInteraction h;
    h.normal = Vec3(0, 1, 0);
    h.frontFace = true;
    Vec3 in = Vec3(1, -1, 0).normalize();
    Vec3 out = refractVec(in, h.normal, 1.0 / 1.5);
    Vec3 rad = g.evaluateBRDF(in, out, &h, TransportMode::Radiance), imp = g.evaluateBRDF(in, out, &h, TransportMode::Importance);
    check(!rad.isZero() && !imp.isZero() && near(rad.x / imp.x, (1 / 1.5) * (1 / 1.5), 1e-6),
          "dielectric_test.go:194 TestDielectricEvaluateBRDF_Refraction_TransportModes");
    Vec3 rin = Vec3(1, -1, 0).normalize(), rout = Vec3(1, 1, 0).normalize();
    Vec3 a = g.evaluateBRDF(rin, rout, &h, TransportMode::Radiance), b = g.evaluateBRDF(rin, rout, &h, TransportMode::Importance);
    check(nearV(a, b, 1e-9) && !a.isZero() && near(a.x, a.y, 1e-9), "dielectric_test.go:156 TestDielectricEvaluateBRDF_Reflection");
  }
  {  // TestNewMetal_FuzznessClamp (pkg/material/metal_test.go:10-34)
    Metal a(Vec3(1, 1, 1), 1.5), b(Vec3(1, 1, 1), -0.5), c(Vec3(1, 1, 1), 0.3);
    check(a.fuzz == 1.0 && b.fuzz == 0.0 && c.fuzz == 0.3, "metal_test.go:10 TestNewMetal_FuzznessClamp");
  }
  {  // TestLambertian_PDFCalculation (pkg/material/lambertian_test.go:11-40)
    Lambertian l(Vec3(0.5, 0.5, 0.5));
    bool d;
    double p = l.pdf(Vec3(), Vec3(0, 1, 0), Vec3(0, 1, 0), d);
    double p2 = l.pdf(Vec3(), Vec3(0, -1, 0), Vec3(0, 1, 0), d);
    check(near(p, 1 / kPi, 1e-12) && p2 == 0 && !d, "lambertian_test.go:11 TestLambertian_PDFCalculation");
  }
  {  // TestQuadLight_PDF_SolidAngleCalculation / HitAndMiss (pkg/lights/quad_light_test.go:89-175)
    Emissive em(Vec3(1, 1, 1));
    Quad q(Vec3(-0.5, -0.5, 0), Vec3(1, 0, 0), Vec3(0, 1, 0), &em);
    QuadLight l(&q);
    check(near(l.pdf(Vec3(0, 0, 1), Vec3(0, 0, 1), Vec3(0, 0, -1)), 1.0, 1e-6), "quad_light_test.go:150 TestQuadLight_PDF_SolidAngleCalculation");
    Quad q2(Vec3(-1, -1, 0), Vec3(2, 0, 0), Vec3(0, 2, 0), &em);
    QuadLight l2(&q2);
    bool ok = l2.pdf(Vec3(0, 0, 2), Vec3(0, 0, 1), Vec3(0, 0, -1)) > 0 && l2.pdf(Vec3(-1, -1, 2), Vec3(0, 0, 1), Vec3(0, 0, -1)) > 0 &&
              l2.pdf(Vec3(0, 0, 2), Vec3(0, 0, 1), Vec3(1, 1, -1).normalize()) == 0 && l2.pdf(Vec3(0, 0, 2), Vec3(0, 0, 1), Vec3(0, 0, 1)) == 0;
    check(ok, "quad_light_test.go:89 TestQuadLight_PDF_HitAndMiss");
    Emissive e5(Vec3(5, 5, 5));
    Quad q3(Vec3(-0.5, -0.5, 0), Vec3(1, 0, 0), Vec3(0, 1, 0), &e5);
    QuadLight l3(&q3);
    PcgSampler s(42, 0);
    LightSample ls = l3.sample(Vec3(0, 0, 2), Vec3(0, 0, 1), s.get2D());
    check(near(ls.point.z, 0, 1e-9) && ls.pdf > 0 && nearV(ls.emission, Vec3(5, 5, 5), 0) &&
              near(ls.direction.sub(ls.point.sub(Vec3(0, 0, 2)).normalize()).length(), 0, 1e-9),
          "quad_light_test.go:12 TestQuadLight_Sample_BasicSampling");
  }
  {  // TestNewWeightedLightSampler_Normalization / GetLightProbability (weighted_light_sampler_test.go:86,240)
    std::vector<const Light*> ls(3, nullptr);
    LightSampler w = LightSampler::weighted(ls, {1, 2, 1});
    LightSampler z = LightSampler::weighted(ls, {0, 0, 0});
    check(near(w.probability(1), 0.5, 1e-12) && near(w.probability(0), 0.25, 1e-12) && w.probability(3) == 0 &&
              near(z.probability(2), 1.0 / 3.0, 1e-12),
          "weighted_light_sampler_test.go:86,104,240 WeightedLightSampler probabilities");
  }
  {  // TestPowerHeuristic (pkg/integrator/path_tracing_test.go:264-315)
    check(near(powerHeuristic(1, 0.5, 1, 0.5), 0.5, 1e-5) && powerHeuristic(1, 0, 1, 0.5) == 0 &&
              near(powerHeuristic(1, 0.5, 1, 0), 1.0, 1e-5) && near(powerHeuristic(1, 0.8, 1, 0.2), 0.941176, 1e-5),
          "path_tracing_test.go:264 TestPowerHeuristic");
  }
}

// ---------------------------------------------------------------- BDPT
void bdptTests() {
  BDPTIntegrator bd8(SamplingConfig{});
  {  // TestVertexConvertSolidAngleToAreaPdf (pkg/integrator/bdpt_mis_test.go:19-141)
    Lambertian white(Vec3(0.7, 0.7, 0.7));
    struct C { const char* n; Vec3 fp, tp, tn; const Material* tm; bool inf; double sa, exp, tol; };
    C cs[] = {{"UnitDistance", {0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, &white, false, 1.0, 1.0, 1e-10},
              {"DistanceTwo", {0, 0, 0}, {2, 0, 0}, {-1, 0, 0}, &white, false, 1.0, 0.25, 1e-10},
              {"InfiniteLight", {0, 0, 0}, {1000, 1000, 1000}, {-1, -1, -1}, nullptr, true, 0.25, 0.25, 1e-10},
              {"ZeroDistance", {0, 0, 0}, {0, 0, 0}, {0, 1, 0}, &white, false, 1.0, 0.0, 1e-10},
              {"GrazingAngle", {0, 0, 0}, {1, 0.001, 0}, Vec3(-1, 0.001, 0).normalize(), &white, false, 1.0, 1.0, 0.1},
              {"VerySmallDistance", {0, 0, 0}, {1e-6, 0, 0}, {-1, 0, 0}, &white, false, 1.0, 1e12, 1e11},
              {"LargeDistance", {0, 0, 0}, {1e6, 0, 0}, {-1, 0, 0}, &white, false, 1.0, 1e-12, 1e-13},
              {"AlmostPerpendicular", {0, 0, 0}, {1, 0, 0}, {0, 0, 1}, &white, false, 1.0, 0.0, 1e-10}};
    for (auto& c : cs) {
      Vertex f = testVertex(c.fp, Vec3(0, 1, 0), false, false, nullptr);
      Vertex t = testVertex(c.tp, c.tn, false, false, c.tm);
      t.isInfiniteLight = c.inf;
      check(near(f.convertSolidAngleToAreaPdf(t, c.sa), c.exp, c.tol),
            std::string("bdpt_mis_test.go:19 TestVertexConvertSolidAngleToAreaPdf/") + c.n);
    }
  }
  {  // TestCalculateMISWeight (pkg/integrator/bdpt_mis_test.go:144-428)
    auto sc = simpleTestScene();
    BDPTIntegrator bd(SamplingConfig{0, 0, 0, 8, 0, 0, 0});
    Lambertian white(Vec3(0.7, 0.7, 0.7));
    Dielectric glass(1.5);
    Emissive em(Vec3(5, 5, 5));
    Metal mirror(Vec3(0.9, 0.9, 0.9), 0.0);
    Vertex slv = sampledLightVertex(&em);
    struct C { const char* n; Path cp, lp; const Vertex* sv; int s, t; double w; };
    Emissive em4(Vec3(4, 4, 4));
    Quad hq(Vec3(-0.5, 2.0, -1.5), Vec3(1, 0, 0), Vec3(0, 0, 1), &em4);
    QuadLight hitLight(&hq);
    std::vector<C> cs = {
        {"TrivialCase_s0t2", testCameraPath({&white}, {{0, 0, 0}, {0, 0, -1}}), Path(), nullptr, 0, 2, 1.0},
        {"DirectLighting_s1t2", testCameraPath({&white}, {{0, 0, 0}, {0, 0, -1}}), testLightPath({&em}, {{0, 2, -1}}), &slv, 1, 2, 0.752119},
        {"DirectLighting_s1t3_OneBounce", testCameraPath({&white, &white}, {{0, 0, 0}, {0, 0, -1}, {-1, 0, -1}}),
         testLightPath({&em}, {{-1, 2, -1}}), &slv, 1, 3, 0.583572},
        {"IndirectLighting_s2t2", testCameraPath({&white}, {{0, 0, 0}, {0, 0, -1}}), testLightPath({&em, &white}, {{0, 2, -1}, {0, 1, -1}}),
         nullptr, 2, 2, 0.097708},
        {"ComplexPath_s2t3", testCameraPath({&white, &white}, {{0, 0, 0}, {0, 0, -1}, {1, 0, -1}}),
         testLightPath({&em, &white}, {{1, 3, -1}, {1, 2, -1}}), nullptr, 2, 3, 0.069731},
        {"PathTracing_s0t4", testCameraPath({&white, &white, &white}, {{0, 0, 0}, {0, 0, -1}, {1, 0, -1}, {2, 0, -1}}), Path(),
         nullptr, 0, 4, 0.041875},
        {"PathTracing_s0t3_HitsLight", testCameraPath({&white, &em}, {{0, 0, 0}, {0, 0, -1}, {0, 2, -1}}, &hitLight), Path(), nullptr,
         0, 3, 0.202964},
        {"MultiBounceGlass_s1t3", testCameraPath({&glass, &white}, {{0, 0, 0}, {0, 0, -1}, {0, 0, -2}}), testLightPath({&em}, {{0, 2, -2}}),
         &slv, 1, 3, 0.951539},
        {"SpecularMirrorPath_s1t3", testCameraPath({&mirror, &white}, {{0, 0, 0}, {0, 0, -1}, {1, 0, -1}}),
         testLightPath({&em}, {{1, 2, -1}}), &slv, 1, 3, 0.951539},
        {"DirectSpecularLighting_s1t2", testCameraPath({&mirror}, {{0, 0, 0}, {0, 0, -1}}), testLightPath({&em}, {{0, 2, -1}}), &slv, 1,
         2, 0.444444},
        {"ComplexSpecularPath_s2t2", testCameraPath({&mirror}, {{0, 0, 0}, {0, 0, -1}}),
         testLightPath({&em, &mirror}, {{0, 3, -1}, {0, 2, -1}}), nullptr, 2, 2, 0.095925},
    };
    for (auto& c : cs) {
      double w = bd.misWeight(c.cp, c.lp, c.sv, c.s, c.t, *sc->s);
      check(w >= 0 && w <= 1 && near(w, c.w, 0.001), std::string("bdpt_mis_test.go:144 TestCalculateMISWeight/") + c.n);
    }
    // WeightedLightSampler_PathTracing_s0t3 (bdpt_mis_test.go:362-398)
    auto t = std::make_unique<TestScene>();
    auto e2 = t->add(std::make_unique<Emissive>(Vec3(2, 2, 2)));
    auto e5 = t->add(std::make_unique<Emissive>(Vec3(5, 5, 5)));
    auto q1 = t->shape(std::make_unique<Quad>(Vec3(-1.5, 2.0, -1.5), Vec3(1, 0, 0), Vec3(0, 0, 1), e2));
    auto q2 = t->shape(std::make_unique<Quad>(Vec3(-0.5, 2.0, -1.5), Vec3(1, 0, 0), Vec3(0, 0, 1), e5));
    t->light(std::make_unique<QuadLight>(q1));
    t->light(std::make_unique<QuadLight>(q2));
    auto ws = sceneWithQuadLights({}, std::move(t), {0.2, 0.8});
    Emissive em5(Vec3(5, 5, 5));
    Quad hq2(Vec3(-0.5, 2.0, -1.5), Vec3(1, 0, 0), Vec3(0, 0, 1), &em5);
    QuadLight hl2(&hq2);
    Path cp = testCameraPath({&white, &em}, {{0, 0, 0}, {0, 0, -1}, {0, 2, -1}}, &hl2);
    cp.vertices[2].lightIndex = 1;
    double w = bd.misWeight(cp, Path(), nullptr, 0, 3, *ws->s);
    check(near(w, 0.241453, 0.001), "bdpt_mis_test.go:362 TestCalculateMISWeight/WeightedLightSampler_PathTracing_s0t3");
  }
  {  // TestCalculateVertexPdf (pkg/integrator/bdpt_mis_test.go:682-749)
    auto sc = simpleTestScene();
    Lambertian white(Vec3(0.7, 0.7, 0.7));
    Vertex cam0;
    cam0.si.point = Vec3(0, 0, 0);
    cam0.si.normal = Vec3(0, 0, -1);
    cam0.isCamera = true;
    Vertex nx = testVertex(Vec3(0, 0, -1), Vec3(0, 0, 1), false, false, nullptr);
    check(near(bd8.vertexPdf(cam0, nullptr, nx, *sc->s), 1.46, 0.01), "bdpt_mis_test.go:682 TestCalculateVertexPdf/CameraVertex");
    Vertex cur = testVertex(Vec3(0, 0, -1), Vec3(0, 0, 1), false, false, &white);
    Vertex pv;
    pv.si.point = Vec3(0, 0, 0);
    pv.si.normal = Vec3(0, 0, -1);
    Vertex nx2 = testVertex(Vec3(1, 0, -1), Vec3(-1, 0, 1), false, false, nullptr);
    check(near(bd8.vertexPdf(cur, &pv, nx2, *sc->s), 0.0, 0.01), "bdpt_mis_test.go:682 TestCalculateVertexPdf/MaterialVertex");
    Vertex lv;
    lv.si.point = Vec3(0, 1, 0);
    lv.si.normal = Vec3(0, -1, 0);
    lv.isLight = true;
    lv.light = testAreaLight().l.get();
    Vertex nx3 = testVertex(Vec3(0, 0, 0), Vec3(0, 1, 0), false, false, nullptr);
    check(near(bd8.vertexPdf(lv, nullptr, nx3, *sc->s), 0.0, 0.01), "bdpt_mis_test.go:682 TestCalculateVertexPdf/LightVertex");
  }
  {  // TestEvaluateDirectLightingStrategy (pkg/integrator/bdpt_light_test.go:170-378)
    BDPTIntegrator bd(SamplingConfig{0, 0, 0, 3, 0, 0, 0});
    Lambertian diff(Vec3(0.7, 0.5, 0.3));
    Metal m8(Vec3(0.8, 0.8, 0.8), 0.0);
    struct C { const char* n; Vec3 lightCorner; const Material* mat; Vec3 beta; bool spec; Vec3 exp; double tol; };
    C cs[] = {{"DiffuseSurfaceWithQuadLight", {-0.5, 2.0, -0.5}, &diff, {0.8, 0.6, 0.4}, false, {0.223, 0.119, 0.0477}, 1e-3},
              {"SurfaceWithNegativeCosine", {-0.5, -2.0, -0.5}, &diff, {0.8, 0.6, 0.4}, false, {0, 0, 0}, 1e-6},
              {"SpecularSurface", {-0.5, 2.0, -0.5}, &m8, {1, 1, 1}, true, {0, 0, 0}, 1e-6},
              {"ZeroBetaThroughput", {-0.5, 2.0, -0.5}, &diff, {0, 0, 0}, false, {0, 0, 0}, 1e-6}};
    for (auto& c : cs) {
      auto sc = sceneWithQuadLight(c.lightCorner, Vec3(1, 0, 0), Vec3(0, 0, 1), Vec3(5, 5, 5));
      Vertex cv;
      cv.si.point = Vec3(0, 0, 0);
      cv.si.normal = Vec3(0, 1, 0);
      cv.si.material = c.mat;
      cv.beta = c.beta;
      cv.isSpecular = c.spec;
      cv.incomingDirection = c.spec ? Vec3() : Vec3(0, 0, 1);
      Path p;
      p.vertices.push_back(testVertex(Vec3(0, 0, 5), Vec3(0, 0, -1), false, true, nullptr));
      p.vertices.push_back(cv);
      p.length = 2;
      ListSampler ls({0.0}, {Vec2(0.5, 0.5)}, {});
      Vertex sampled;
      bool has;
      Vec3 r = bd.directLightingStrategy(p, 2, *sc->s, ls, sampled, has);
      bool ok = nearV(r, c.exp, c.tol);
      if (ok && c.exp.luminance() > 0) ok = has && sampled.isLight && nearV(sampled.si.point, Vec3(0, 2, 0), 1e-9);
      check(ok, std::string("bdpt_light_test.go:170 TestEvaluateDirectLightingStrategy/") + c.n);
    }
  }
  {  // TestCameraPathBetaPropagation (pkg/integrator/bdpt_light_test.go:825-933)
    BDPTIntegrator bd(SamplingConfig{0, 0, 0, 5, 0, 0, 0});
    Ray gr = rayTo(Vec3(0, 0, 0), Vec3(0.5, 0, -1.5));
    struct Exp { int idx; Vec3 beta; bool cam, spec; double tol; };
    struct C { const char* n; std::function<std::unique_ptr<Material>()> mk; ListSampler s; std::vector<Exp> e; };
    std::vector<C> cs = {
        {"Diffuse", [] { return std::make_unique<Lambertian>(Vec3(0.7, 0.7, 0.7)); },
         ListSampler({0.5, 0.5}, {Vec2(0.0, 0.5)}, {Vec3(0, 1, 0)}),
         {{0, {1, 1, 1}, true, false, 1e-9}, {1, {1, 1, 1}, false, false, 1e-9}, {2, {0.7, 0.7, 0.7}, false, false, 1e-2}}},
        {"Specular", [] { return std::make_unique<Metal>(Vec3(0.9, 0.85, 0.8), 0.0); },
         ListSampler({0.5}, {Vec2(0.5, 0.5)}, {Vec3(0, 0, 1)}),
         {{0, {1, 1, 1}, true, false, 1e-9}, {1, {1, 1, 1}, false, true, 1e-9}, {2, {0.9, 0.85, 0.8}, false, false, 1e-6}}},
        {"Dielectric", [] { return std::make_unique<Dielectric>(1.5); },
         ListSampler({0.2, 0.5, 0.5, 0.5}, {Vec2(0.5, 0.5), Vec2(0.3, 0.7)}, {Vec3(0, 0, 1), Vec3(0, 1, 0)}),
         {{0, {1, 1, 1}, true, false, 1e-9}, {1, {1, 1, 1}, false, true, 1e-9}, {2, {1, 1, 1}, false, true, 1e-6}}},
    };
    for (auto& c : cs) {
      auto sc = glancingScene(c.mk());
      Path p = bd.generateCameraPath(gr, *sc->s, c.s, 3);
      bool ok = p.length >= (int)c.e.size();
      if (!ok) g_detail = "path too short";
      for (auto& e : c.e) {
        if (!ok) break;
        const Vertex& v = p.vertices[e.idx];
        ok = nearV(v.beta, e.beta, e.tol) && v.isCamera == e.cam && v.isSpecular == e.spec;
        if (ok == false && g_detail.empty()) g_detail = "flags mismatch at vertex " + std::to_string(e.idx);
      }
      check(ok, std::string("bdpt_light_test.go:825 TestCameraPathBetaPropagation/") + c.n);
    }
  }
  {  // TestLightPathBetaPropagation (pkg/integrator/bdpt_light_test.go:935-1008)
    BDPTIntegrator bd(SamplingConfig{0, 0, 0, 5, 0, 0, 0});
    struct Exp { int idx; Vec3 beta; bool light, spec; };
    struct C { const char* n; std::function<std::unique_ptr<Material>()> mk; std::vector<Exp> e; };
    std::vector<C> cs = {
        {"Diffuse", [] { return std::make_unique<Lambertian>(Vec3(0.7, 0.7, 0.7)); },
         {{0, {5, 5, 5}, true, false}, {1, {15.7, 15.7, 15.7}, false, false}, {2, {11.7, 11.7, 11.7}, false, false}}},
        {"Specular", [] { return std::make_unique<Metal>(Vec3(0.9, 0.85, 0.8), 0.0); },
         {{0, {5, 5, 5}, true, false}, {1, {15.7, 15.7, 15.7}, false, true}, {2, {14.137, 13.351, 12.566}, false, false}}},
        {"Dielectric", [] { return std::make_unique<Dielectric>(1.5); },
         {{0, {5, 5, 5}, true, false}, {1, {15.7, 15.7, 15.7}, false, true}, {2, {15.7, 15.7, 15.7}, false, true}}},
    };
    for (auto& c : cs) {
      ListSampler s({0.0, 0.5, 0.5}, {Vec2(0.5, 0.5), Vec2(0.5, 0.0), Vec2(0.0, 0.5), Vec2(0.0, 0.5), Vec2(0.0, 0.5)},
                    {Vec3(0, -1, 0)});
      auto sc = lightScene(c.mk());
      Path p = bd.generateLightPath(*sc->s, s, 3);
      // compareToExpectedPath (bdpt_light_test.go:1010-1054): relative beta tolerance 1e-3
      bool ok = p.length <= (int)c.e.size();
      if (!ok) g_detail = "path too long";
      for (auto& e : c.e) {
        if (!ok) break;
        if (e.idx >= p.length) {
          ok = false;
          g_detail = "missing vertex";
          break;
        }
        const Vertex& v = p.vertices[e.idx];
        auto rel = [&](double a, double b) { return std::fabs(a / b) - 1 <= 1e-3; };
        ok = rel(v.beta.x, e.beta.x) && rel(v.beta.y, e.beta.y) && rel(v.beta.z, e.beta.z) && v.isLight == e.light &&
             v.isSpecular == e.spec && !v.isCamera;
        if (!ok) {
          std::ostringstream o;
          o << "vertex " << e.idx << " beta " << v.beta.x << "," << v.beta.y << "," << v.beta.z;
          g_detail = o.str();
        }
      }
      check(ok, std::string("bdpt_light_test.go:935 TestLightPathBetaPropagation/") + c.n);
    }
  }
  {  // TestPdfPropagation (pkg/integrator/bdpt_mis_test.go:751-960)
    BDPTIntegrator bd(SamplingConfig{0, 0, 0, 5, 0, 0, 0});
    struct Exp { int idx; double fwd, rev, tol; };
    struct C { const char* n; bool camera; bool cornell; std::function<std::unique_ptr<Material>()> mk; ListSampler s; std::vector<Exp> e; };
    std::vector<C> cs = {
        {"CameraPath_Diffuse_MultipleSurfaceBounces", true, true, [] { return std::make_unique<Lambertian>(Vec3(0.7, 0.7, 0.7)); },
         ListSampler({0.5, 0.5, 0.5, 0.5, 0.5}, {Vec2(0.8, 0.5), Vec2(0.3, 0.7), Vec2(0.1, 0.9)}, {Vec3(-0.5, 0.5, 0.3), Vec3(0.2, -0.8, 0.1)}),
         {{0, 0.0, 1.424e-6, 1e-6}, {1, 0.0, 0.886e-6, 1e-6}, {2, 1.000e-6, 1.263e-6, 1e-6}, {3, 1.263e-6, 0.0, 1e-6}}},
        {"CameraPath_Diffuse_BasicPropagation", true, false, [] { return std::make_unique<Lambertian>(Vec3(0.7, 0.7, 0.7)); },
         ListSampler({0.5, 0.5}, {Vec2(0.0, 0.5)}, {Vec3(0, 1, 0)}),
         {{0, 0.0, 0.195589, 1e-6}, {1, 1.048629, 0.0, 1e-6}, {2, 0.225079, 0.0, 1e-6}}},
        {"CameraPath_Specular_DeltaFunctions", true, false, [] { return std::make_unique<Metal>(Vec3(0.9, 0.85, 0.8), 0.0); },
         ListSampler({0.5}, {Vec2(0.5, 0.5)}, {Vec3(0, 0, 1)}), {{0, 0.0, 0.0, 1e-6}, {1, 1.048629, 0.0, 1e-6}, {2, 0.0, 0.0, 1e-6}}},
        {"CameraPath_Dielectric_EnergyConservation", true, false, [] { return std::make_unique<Dielectric>(1.5); },
         ListSampler({0.2, 0.5, 0.5, 0.5}, {Vec2(0.5, 0.5), Vec2(0.3, 0.7)}, {Vec3(0, 0, 1), Vec3(0, 1, 0)}),
         {{0, 0.0, 0.0, 1e-6}, {1, 1.048629, 0.0, 1e-6}, {2, 0.0, 0.0, 1e-6}}},
        {"LightPath_Diffuse_EmissionPropagation", false, false, [] { return std::make_unique<Lambertian>(Vec3(0.7, 0.7, 0.7)); },
         ListSampler({0.0, 0.5, 0.5, 0.5, 0.5, 0.5}, {Vec2(0.5, 0.5), Vec2(0.5, 0.0), Vec2(0.0, 0.5), Vec2(0.0, 0.5), Vec2(0.0, 0.5)},
                     {Vec3(0, -1, 0)}),
         {{0, 1.0, 0.110142, 1e-6}, {1, 0.110142, 0.002046, 1e-6}, {2, 0.002046, 0.0, 1e-6}}},
        {"LightPath_Specular_DeltaHandling", false, false, [] { return std::make_unique<Metal>(Vec3(0.9, 0.85, 0.8), 0.0); },
         ListSampler({0.0, 0.5, 0.5, 0.5, 0.5, 0.5}, {Vec2(0.5, 0.5), Vec2(0.5, 0.0), Vec2(0.0, 0.5), Vec2(0.0, 0.5), Vec2(0.0, 0.5)},
                     {Vec3(0, -1, 0)}),
         {{0, 1.0, 0.0, 1e-6}, {1, 0.110142, 0.002780, 1e-6}, {2, 0.0, 0.0, 1e-9}}},
    };
    for (auto& c : cs) {
      Path p;
      std::unique_ptr<TestScene> sc;
      if (c.camera) {
        Ray ray;
        if (c.cornell) {
          sc = minimalCornell();
          ray = Ray(Vec3(278, 400, -200), Vec3(0, -1, 0.5).normalize());
        } else {
          sc = glancingScene(c.mk());
          ray = rayTo(Vec3(0, 0, 0), Vec3(0.5, 0, -1.5));
        }
        p = bd.generateCameraPath(ray, *sc->s, c.s, 3);
      } else {
        sc = lightScene(c.mk());
        p = bd.generateLightPath(*sc->s, c.s, 3);
      }
      bool ok = p.length >= (int)c.e.size();
      if (!ok) g_detail = "path too short: " + std::to_string(p.length);
      for (auto& e : c.e) {
        if (!ok) break;
        const Vertex& v = p.vertices[e.idx];
        ok = near(v.areaPdfForward, e.fwd, e.tol) && near(v.areaPdfReverse, e.rev, e.tol);
        if (!ok) g_detail = "vertex " + std::to_string(e.idx) + ": " + g_detail;
      }
      check(ok, std::string("bdpt_mis_test.go:751 TestPdfPropagation/") + c.n);
    }
  }
}

// ---------------------------------------------------------------- renderer
void rendererTests() {
  // TestGetSamplesForPass-style schedule (pkg/renderer/progressive.go:98-123,
  // progressive_test.go): 1 pass -> all samples; 7 passes of 50 -> 1,9,17,...,50
  struct Sched {
    int init, maxS, passes;
    int forPass(int p) const {
      if (passes == 1) return maxS;
      if (p == 1) return init;
      int per = (maxS - init) / (passes - 1);
      int t = init + (p - 1) * per;
      if (p == passes) t = maxS;
      return t;
    }
  };
  Sched a{1, 50, 7}, b{1, 64, 1};
  check(a.forPass(1) == 1 && a.forPass(2) == 9 && a.forPass(6) == 41 && a.forPass(7) == 50 && b.forPass(1) == 64,
        "progressive.go:98 getSamplesForPass schedule");
}

}  // namespace

// Point spot, disc and disc spot lights (pkg/lights/point_spot_light_test.go,
// disc_light_test.go, disc_spot_light_test.go).  Where the reference draws
// its sample points from math/rand, a fixed grid of sample points stands in;
// the checked properties are the reference's.
void spotLightTests() {
  const double pi = kPi;
  std::vector<Vec2> grid;
  for (int i = 0; i < 10; i++)
    for (int j = 0; j < 10; j++) grid.push_back(Vec2((i + 0.37) / 10.0, (j + 0.61) / 10.0));
  {  // TestPointSpotLight_NewPointSpotLight (point_spot_light_test.go:11-48)
    PointSpotLight l(Vec3(0, 5, 0), Vec3(0, 0, 0), Vec3(1, 1, 1), 45.0, 5.0);
    check(l.direction.sub(Vec3(0, -1, 0)).length() < 1e-6 && std::fabs(l.cosTotal - std::cos(45.0 * pi / 180)) < 1e-6 &&
              std::fabs(l.cosStart - std::cos(40.0 * pi / 180)) < 1e-6,
          "point_spot_light_test.go:11 TestPointSpotLight_NewPointSpotLight");
  }
  {  // TestPointSpotLight_Sample_WithinCone (:50-94)
    PointSpotLight l(Vec3(0, 5, 0), Vec3(0, 0, 0), Vec3(100, 100, 100), 60.0, 5.0);
    Vec3 tp(0, 1, 0);
    LightSample s = l.sample(tp, Vec3(0, 1, 0), Vec2(0.3, 0.7));
    double d = 4.0;
    check(s.point.sub(Vec3(0, 5, 0)).length() < 1e-6 && s.direction.sub(Vec3(0, 1, 0)).length() < 1e-6 &&
              std::fabs(s.distance - d) < 1e-6 &&
              std::fabs(s.emission.length() - Vec3(100, 100, 100).length() / (d * d)) < 1e-6 && s.pdf == 1.0,
          "point_spot_light_test.go:50 TestPointSpotLight_Sample_WithinCone");
  }
  {  // TestPointSpotLight_Sample_OutsideCone (:96-118)
    PointSpotLight l(Vec3(0, 5, 0), Vec3(0, 0, 0), Vec3(100, 100, 100), 30.0, 5.0);
    LightSample s = l.sample(Vec3(10, 1, 0), Vec3(0, 1, 0), Vec2(0.3, 0.7));
    check(s.emission.length() <= 0.1, "point_spot_light_test.go:96 TestPointSpotLight_Sample_OutsideCone");
  }
  {  // TestPointSpotLight_PDF (:120-147)
    PointSpotLight l(Vec3(0, 5, 0), Vec3(0, 0, 0), Vec3(100, 100, 100), 60.0, 5.0);
    Vec3 tp(0, 1, 0), n(0, 1, 0), toL = Vec3(0, 5, 0).sub(tp).normalize();
    check(l.pdf(tp, n, toL) == 1.0 && l.pdf(tp, n, toL.mul(-1)) == 0.0 && l.pdf(tp, n, Vec3(1, 0, 0)) == 0.0,
          "point_spot_light_test.go:120 TestPointSpotLight_PDF");
  }
  Emissive e10(Vec3(10, 10, 10)), e5(Vec3(5, 5, 5)), e1(Vec3(1, 1, 1));
  {  // TestDiscLightSample (disc_light_test.go:12-54)
    Disc d(Vec3(0, 1, 0), Vec3(0, -1, 0), 1.0, &e10);
    DiscLight l(&d);
    bool ok = true;
    for (Vec2 u : grid) {
      LightSample s = l.sample(Vec3(0, 0, 0), Vec3(0, 1, 0), u);
      ok = ok && s.point.sub(d.center).length() <= 1.0 + 1e-6 &&
           s.direction.sub(s.point.normalize()).length() < 1e-12 && std::fabs(s.distance - s.point.length()) < 1e-6 &&
           s.pdf > 0 && s.emission.length() > 0;
    }
    check(ok, "disc_light_test.go:12 TestDiscLightSample");
  }
  {  // TestDiscLightPDF (:56-108)
    Disc d(Vec3(0, 1, 0), Vec3(0, -1, 0), 1.0, &e10);
    DiscLight l(&d);
    Vec3 o(0, 0, 0), n(0, 1, 0);
    check(l.pdf(o, n, Vec3(0, 1, 0)) > 0, "disc_light_test.go:56 TestDiscLightPDF/Direction hits center of disc");
    check(l.pdf(o, n, Vec3(1, 1, 0).normalize()) > 0, "disc_light_test.go:56 TestDiscLightPDF/Direction hits edge of disc");
    check(l.pdf(o, n, Vec3(2, 1, 0).normalize()) == 0, "disc_light_test.go:56 TestDiscLightPDF/Direction misses disc");
    check(l.pdf(o, n, Vec3(1, 0, 0)) == 0, "disc_light_test.go:56 TestDiscLightPDF/Direction parallel to disc");
  }
  {  // TestDiscLightSampleConsistency (:110-133)
    Disc d(Vec3(0, 2, 0), Vec3(0, -1, 0), 0.5, &e5);
    DiscLight l(&d);
    bool ok = true;
    for (Vec2 u : grid) {
      LightSample s = l.sample(Vec3(0, 0, 0), Vec3(0, 1, 0), u);
      ok = ok && std::fabs(s.pdf - l.pdf(Vec3(0, 0, 0), Vec3(0, 1, 0), s.direction)) <= 1e-10;
    }
    check(ok, "disc_light_test.go:110 TestDiscLightSampleConsistency");
  }
  {  // TestDiscLightEdgeCase (:175-204)
    Disc d(Vec3(0, 1, 0), Vec3(0, -1, 0), 1.0, &e1);
    DiscLight l(&d);
    LightSample s = l.sample(Vec3(0, 0.99, 0), Vec3(0, 1, 0), Vec2(0.42, 0.17));
    check(s.distance > 0 && s.pdf > 0 && s.point.sub(d.center).length() <= 1.0 + 1e-6,
          "disc_light_test.go:175 TestDiscLightEdgeCase");
  }
  {  // TestDiscLight_SampleEmission (:206-273), TestDiscLight_EmissionSampling_Coverage (:351-410)
    Disc d(Vec3(0, 0, 0), Vec3(0, 1, 0), 1.0, &e5);
    DiscLight l(&d);
    bool ok = true;
    int centre = 0;
    for (size_t k = 0; k < grid.size(); k++) {
      EmissionSample s = l.sampleEmission(grid[k], grid[(k * 37 + 11) % grid.size()]);
      double ct = s.direction.dot(s.normal);
      double pp, pd;
      l.pdfLe(s.point, s.direction, pp, pd);
      ok = ok && s.point.length() <= 1.0 + 1e-9 && std::fabs(s.point.y) <= 1e-9 &&
           s.normal.sub(Vec3(0, 1, 0)).length() <= 1e-9 && ct > 0 && std::fabs(s.direction.length() - 1) <= 1e-9 &&
           std::fabs(s.areaPdf - 1.0 / pi) <= 1e-9 && std::fabs(s.directionPdf - ct / pi) <= 1e-9 &&
           s.emission.x == 5.0 && s.emission.y == 5.0 && s.emission.z == 5.0 && std::fabs(s.areaPdf - pp) <= 1e-6;
      centre += s.point.length() <= 0.5;
    }
    check(ok, "disc_light_test.go:206 TestDiscLight_SampleEmission");
    check(std::fabs(centre / (double)grid.size() - 0.25) <= 0.1, "disc_light_test.go:351 TestDiscLight_EmissionSampling_Coverage");
  }
  {  // TestDiscLight_EmissionPDF (:275-349)
    Disc d(Vec3(0, 0, 0), Vec3(0, 1, 0), 1.0, &e1);
    DiscLight l(&d);
    struct Cs { const char* n; Vec3 p, dir; bool expect; };
    Cs cs[] = {{"Point on disc, direction in hemisphere", Vec3(0.5, 0, 0), Vec3(0, 1, 0), true},
               {"Point on disc, direction below surface", Vec3(0.5, 0, 0), Vec3(0, -1, 0), false},
               {"Point outside disc radius", Vec3(2, 0, 0), Vec3(0, 1, 0), false},
               {"Point above disc plane", Vec3(0.5, 1, 0), Vec3(0, 1, 0), false},
               {"Point at disc center", Vec3(0, 0, 0), Vec3(0, 1, 0), true}};
    for (const Cs& c : cs) {
      double pp, pd;
      l.pdfLe(c.p, c.dir, pp, pd);
      bool ok = c.expect ? std::fabs(pp - 1.0 / pi) <= 1e-9 : pp == 0;
      check(ok, std::string("disc_light_test.go:275 TestDiscLight_EmissionPDF/") + c.n);
    }
  }
  {  // TestDiscSpotLightFalloff (disc_spot_light_test.go:11-76)
    double ct = std::cos(30 * pi / 180), cs = std::cos(25 * pi / 180);
    double mid = std::cos(27.5 * pi / 180);
    double dm = (mid - ct) / (cs - ct);
    struct Fc { const char* n; double c, want; };
    Fc fc[] = {{"Inside inner cone", std::cos(20 * pi / 180), 1.0},
               {"At falloff start edge", std::cos(25 * pi / 180), 1.0},
               {"In falloff region", mid, dm * dm * dm * dm},
               {"At total width edge", std::cos(30 * pi / 180), 0.0},
               {"Outside cone", std::cos(35 * pi / 180), 0.0}};
    for (const Fc& f : fc)
      check(std::fabs(spotFalloff(f.c, ct, cs) - f.want) <= 1e-6,
            std::string("disc_spot_light_test.go:11 TestDiscSpotLightFalloff/") + f.n);
  }
  {  // TestDiscSpotLightSample (:78-144)
    Vec3 from(0, 2, 0), to(0, 0, 0);
    Vec3 dir = to.sub(from).normalize();
    SpotEmissive m(Vec3(5, 5, 5), dir);
    Disc d(from, dir, 0.2, &m);
    DiscSpotLight l(&d, from, to, Vec3(5, 5, 5), 45.0, 10.0);
    struct Sc { const char* n; Vec3 p; bool expect; };
    Sc cs[] = {{"Point directly below", Vec3(0, 0, 0), true},
               {"Point at edge of inner cone", Vec3(0.7, 0, 0), true},
               {"Point in falloff region", Vec3(1.0, 0, 0), true},
               {"Point outside cone", Vec3(3.0, 0, 0), false}};
    for (const Sc& c : cs) {
      bool ok = true;
      for (Vec2 u : grid) {
        LightSample s = l.sample(c.p, Vec3(0, 1, 0), u);
        bool lit = s.emission.length() > 0;
        ok = ok && s.point.sub(from).length() <= 0.2 + 1e-6 && (c.expect ? lit && s.pdf > 0 : !lit);
      }
      check(ok, std::string("disc_spot_light_test.go:78 TestDiscSpotLightSample/") + c.n);
    }
  }
  {  // TestDiscSpotLightConsistentFalloff (:256-317): the falloff follows the sampled point
    Vec3 from(0, 3, 0), to(0, 0, 0);
    Vec3 dir = to.sub(from).normalize();
    SpotEmissive m(Vec3(10, 10, 10), dir);
    Disc d(from, dir, 1.5, &m);
    DiscSpotLight l(&d, from, to, Vec3(10, 10, 10), 30.0, 5.0);
    Vec3 tp(1.5, 0, 0);
    Vec3 a = l.sample(tp, Vec3(0, 1, 0), Vec2(0.0, 0.0)).emission;
    // the disc's `up` axis is +x here: theta = pi/2 is the edge nearest the point, 3pi/2 the farthest
    Vec3 b = l.sample(tp, Vec3(0, 1, 0), Vec2(1.0, 0.25)).emission;
    Vec3 c = l.sample(tp, Vec3(0, 1, 0), Vec2(1.0, 0.75)).emission;
    check(!(a.sub(b).length() == 0 && a.sub(c).length() == 0) && c.length() < b.length(),
          "disc_spot_light_test.go:256 TestDiscSpotLightConsistentFalloff");
  }
  {  // TestDiscSpotLightCreation (:319-366)
    Vec3 from(1, 2, 3), to(4, 5, 6);
    SpotEmissive m(Vec3(2, 3, 4), to.sub(from).normalize());
    Disc d(from, to.sub(from), 0.3, &m);
    DiscSpotLight l(&d, from, to, Vec3(2, 3, 4), 25.0, 8.0);
    check(l.position.sub(from).length() == 0 && l.direction.sub(to.sub(from).normalize()).length() == 0 &&
              std::fabs(l.cosTotal - std::cos(25 * pi / 180)) <= 1e-6 &&
              std::fabs(l.cosStart - std::cos(17 * pi / 180)) <= 1e-6 && l.base.disc->radius == 0.3,
          "disc_spot_light_test.go:319 TestDiscSpotLightCreation");
  }
}

// ImageTexture.Evaluate (pkg/material/image_texture_test.go)
void textureTests() {
  auto eq = [](Vec3 a, Vec3 b) { return a.sub(b).length() == 0; };
  {  // TestImageTextureEvaluate (:10-53): 2x2 checker, row 0 at the top
    ImageTexture t;
    t.width = t.height = 2;
    t.pixels = {Vec3(1, 1, 1), Vec3(0, 0, 0), Vec3(0, 0, 0), Vec3(1, 1, 1)};
    Vec3 w(1, 1, 1), b(0, 0, 0);
    check(eq(t.evaluate(Vec2(0.1, 0.1)), b) && eq(t.evaluate(Vec2(0.9, 0.1)), w) && eq(t.evaluate(Vec2(0.1, 0.9)), w) &&
              eq(t.evaluate(Vec2(0.9, 0.9)), b),
          "image_texture_test.go:10 TestImageTextureEvaluate");
  }
  {  // TestImageTextureWrapping (:55-78)
    ImageTexture t;
    t.width = t.height = 1;
    t.pixels = {Vec3(1, 0, 0)};
    bool ok = true;
    for (Vec2 uv : {Vec2(0.5, 0.5), Vec2(1.5, 0.5), Vec2(0.5, 1.5), Vec2(-0.5, -0.5), Vec2(2.3, 3.7)})
      ok = ok && eq(t.evaluate(uv), Vec3(1, 0, 0));
    check(ok, "image_texture_test.go:55 TestImageTextureWrapping");
  }
  {  // TestImageTextureSampling (:80-112): 4x4 ramp
    ImageTexture t;
    t.width = t.height = 4;
    for (int y = 0; y < 4; y++)
      for (int x = 0; x < 4; x++) t.pixels.push_back(Vec3(1, 1, 1).mul((y * 4 + x) / 15.0));
    check(eq(t.evaluate(Vec2(0.125, 0.875)), Vec3(0, 0, 0)) && eq(t.evaluate(Vec2(0.875, 0.125)), Vec3(1, 1, 1)),
          "image_texture_test.go:80 TestImageTextureSampling");
  }
}

int main() {
  try {
    textureTests();
    geometryTests();
    quadricTests();
    spotLightTests();
    materialLightTests();
    bdptTests();
    rendererTests();
  } catch (const std::exception& e) {
    std::printf("FAIL exception: %s\n", e.what());
    return 2;
  }
  std::printf("SUMMARY pass=%d fail=%d\n", g_pass, g_fail);
  return g_fail == 0 ? 0 : 1;
}
