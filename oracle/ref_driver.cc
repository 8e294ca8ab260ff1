// Test-oracle driver over the reference renderer's own objects (built by
// oracle/Makefile into oracle/_ref/; test infrastructure only, never shipped).
//
//   ref_driver hits  scene.muon out.bin [linear|bvh]
//     Parses with the reference Parser (muon/parser.cc:230), casts the sample-0
//     ray through every pixel centre with Camera::CastRay (muon/camera.cc:37;
//     pixel centre per muon/sampling.cc:89-91) and intersects it with the
//     reference acceleration structure (muon/acceleration.cc:65 / :168).
//     Per pixel (row-major, y outer), little endian:
//       float ray[6]; int32 hit; int32 prim_id; float distance; float pos[3];
//       float normal[3]; float albedo[3]
//     prim_id is the index in scene-file order, known only for the linear
//     structure (which keeps AddPrimitive order); -2 with the BVH. The fields
//     are the inputs of NormalsTracer/AlbedoTracer/DepthTracer
//     (muon/integration.cc:47-72).
//
//   ref_driver render scene.muon out.bin [spp] [seed]
//     Renderer::Render's sample loop (muon/renderer.cc:34-66) on one thread:
//     TileImage + TileQueue order, Sampler::NextSample, CastRay, the scene's
//     integrator Trace. Accumulates an FP64 film instead of the FP32 one.
//     spp overrides pixel_samples; seed (if given) replaces the scene's seed
//     generator before tiles and the path tracer are seeded.
//     Output: int32 w, h, spp, then w*h*3 doubles of sums and of sums of
//     squares, then uint64 primary, secondary, object tests, bounds tests.
//
//   ref_driver hitkeys scene.muon pixels.bin out.bin
//     As `hits`, through the reference BVH (muon/acceleration.cc:65-142), for
//     the listed pixels only (int32 x, y pairs), with a key of the primitive
//     hit in place of an id (the BVH reorders its primitives): per pixel
//       float ray[6]; int32 hit; int32 kind (0 triangle, 1 sphere);
//       float distance; float pos[3]; float normal[3]; float albedo[3];
//       float object_bounds[6] (min, max); float face_normal[3] (Tri::Normal,
//       the unnormalised (v1-v0)x(v2-v0), muon/objects.cc:48-56; 0 for a
//       sphere); float transform[16] (the primitive's object-to-world matrix,
//       column-major)
//     from which the fixture script recovers the parse-order id.
//
//   ref_driver pixels scene.muon pixels.bin out.bin spp seed
//     The scene's integrator (reseeded as by `render`) traced spp times
//     through each listed pixel (int32 x, y pairs): sample 0 at the pixel
//     centre, later ones jittered in the pixel (muon/sampling.cc:89-107) with
//     an mt19937 of `seed` (the jitter sequence is the driver's own: only the
//     distribution of sample positions matters). For converged values of a
//     pixel subset of a large frame. Output: int32 n, spp, then n*3 doubles of
//     sums and n*3 of sums of squares.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <random>
#include <string>
#include <vector>

#include "muon/acceleration.h"
#include "muon/integration.h"
#include "muon/options.h"
#include "muon/parser.h"
#include "muon/sampling.h"

namespace {

// Reads Structure::primitives_ (protected) through a derived-class member
// pointer, to map primitives back to their AddPrimitive order.
struct PrimitiveAccess : muon::acceleration::Structure {
  static std::vector<std::unique_ptr<muon::Primitive>> &Of(muon::acceleration::Structure &s) {
    return s.*(&PrimitiveAccess::primitives_);
  }
};

muon::Options MakeOptions(bool linear) {
  muon::Options o;
  o.output = "";
  o.acceleration = linear ? muon::AccelerationType::kLinear : muon::AccelerationType::kBVH;
  o.partition_strategy = muon::PartitionStrategy::kSAH;
  o.parallelism = 1;
  o.show_stats = false;
  return o;
}

int Hits(const char *scene, const char *out_path, bool linear) {
  muon::Options options = MakeOptions(linear);
  muon::Parser parser(scene, options);
  muon::SceneConfig sc = parser.Parse();
  std::map<const muon::Primitive *, int32_t> ids;
  if (linear) {
    auto &prims = PrimitiveAccess::Of(*sc.scene->root);
    for (size_t i = 0; i < prims.size(); ++i) ids[prims[i].get()] = static_cast<int32_t>(i);
  }
  auto ws = sc.scene->root->CreateWorkspace();
  int w = sc.scene->width, h = sc.scene->height;
  std::ofstream out(out_path, std::ios::binary);
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      muon::Ray r = sc.scene->camera->CastRay(x + 0.5f, y + 0.5f);
      auto hit = sc.scene->root->Intersect(ws.get(), r);
      float ray[6];
      for (int k = 0; k < 3; ++k) ray[k] = r.origin()[k], ray[3 + k] = r.direction()[k];
      int32_t head[2] = {hit ? 1 : 0, -1};
      float rec[10] = {0};
      if (hit) {
        head[1] = linear ? ids[hit->obj] : -2;
        rec[0] = hit->distance;
        for (int k = 0; k < 3; ++k) {
          rec[1 + k] = hit->pos[k];
          rec[4 + k] = hit->normal[k];
          rec[7 + k] = hit->obj->material->diffuse[k] + hit->obj->material->specular[k];
        }
      }
      out.write(reinterpret_cast<const char *>(ray), sizeof(ray));
      out.write(reinterpret_cast<const char *>(head), sizeof(head));
      out.write(reinterpret_cast<const char *>(rec), sizeof(rec));
    }
  }
  return 0;
}

std::vector<int32_t> ReadPixels(const char *pix_path) {
  std::ifstream pin(pix_path, std::ios::binary);
  std::vector<int32_t> pix;
  int32_t v;
  while (pin.read(reinterpret_cast<char *>(&v), sizeof(v))) pix.push_back(v);
  return pix;
}

int HitKeys(const char *scene, const char *pix_path, const char *out_path) {
  const std::vector<int32_t> pix = ReadPixels(pix_path);
  muon::Options options = MakeOptions(false);
  muon::Parser parser(scene, options);
  muon::SceneConfig sc = parser.Parse();
  auto ws = sc.scene->root->CreateWorkspace();
  std::ofstream out(out_path, std::ios::binary);
  for (size_t i = 0; i + 1 < pix.size(); i += 2) {
    muon::Ray r = sc.scene->camera->CastRay(pix[i] + 0.5f, pix[i + 1] + 0.5f);
    auto hit = sc.scene->root->Intersect(ws.get(), r);
    float ray[6];
    for (int k = 0; k < 3; ++k) ray[k] = r.origin()[k], ray[3 + k] = r.direction()[k];
    int32_t head[2] = {hit ? 1 : 0, 0};
    float rec[10] = {0};
    float key[25] = {0};
    if (hit) {
      rec[0] = hit->distance;
      for (int k = 0; k < 3; ++k) {
        rec[1 + k] = hit->pos[k];
        rec[4 + k] = hit->normal[k];
        rec[7 + k] = hit->obj->material->diffuse[k] + hit->obj->material->specular[k];
      }
      const auto *prim = dynamic_cast<const muon::Primitive *>(hit->obj);
      const auto *tri = dynamic_cast<const muon::Tri *>(hit->obj);
      head[1] = tri ? 0 : 1;
      const muon::Bounds b = prim->ObjectBounds();
      for (int k = 0; k < 3; ++k) key[k] = b.min_pos[k], key[3 + k] = b.max_pos[k];
      if (tri) {
        const glm::vec3 n = tri->Normal();
        for (int k = 0; k < 3; ++k) key[6 + k] = n[k];
      }
      const glm::mat4 &m = *prim->transform;
      for (int c = 0; c < 4; ++c)
        for (int k = 0; k < 4; ++k) key[9 + 4 * c + k] = m[c][k];
    }
    out.write(reinterpret_cast<const char *>(ray), sizeof(ray));
    out.write(reinterpret_cast<const char *>(head), sizeof(head));
    out.write(reinterpret_cast<const char *>(rec), sizeof(rec));
    out.write(reinterpret_cast<const char *>(key), sizeof(key));
  }
  return 0;
}

// Re-seeds as if the file had said `random_seed <seed>` before the
// integrator line: a fresh path-tracer RNG and tile seeds.
void Reseed(muon::SceneConfig &sc, long long seed) {
  if (seed < 0) return;
  sc.scene->seedgen = std::make_unique<muon::SeedGenerator>(static_cast<unsigned int>(seed));
  if (dynamic_cast<muon::PathTracer *>(sc.integrator_prototype.get())) {
    sc.integrator_prototype = std::make_unique<muon::PathTracer>(*sc.scene, sc.scene->seedgen->Next());
  }
}

int Pixels(const char *scene, const char *pix_path, const char *out_path, int spp, long long seed) {
  std::ifstream pin(pix_path, std::ios::binary);
  std::vector<int32_t> pix;
  int32_t v;
  while (pin.read(reinterpret_cast<char *>(&v), sizeof(v))) pix.push_back(v);
  const size_t n = pix.size() / 2;
  muon::Options options = MakeOptions(false);
  muon::Parser parser(scene, options);
  muon::SceneConfig sc = parser.Parse();
  Reseed(sc, seed);
  std::unique_ptr<muon::Integrator> integrator = sc.integrator_prototype->Clone();
  integrator->Init();
  std::mt19937 jitter(static_cast<unsigned int>(seed < 0 ? 0 : seed) ^ 0x9e3779b9u);
  std::uniform_real_distribution<float> u01(0.0f, 1.0f);
  std::vector<double> sum(3 * n, 0.0), sq(3 * n, 0.0);
  for (size_t i = 0; i < n; ++i) {
    const float px = static_cast<float>(pix[2 * i]), py = static_cast<float>(pix[2 * i + 1]);
    for (int k = 0; k < spp; ++k) {
      float x = px + 0.5f, y = py + 0.5f;
      if (k > 0) {
        x = px + u01(jitter);
        y = py + u01(jitter);
        if (x == px + 1.0f) x = std::nextafter(x, -std::numeric_limits<float>::infinity());
        if (y == py + 1.0f) y = std::nextafter(y, -std::numeric_limits<float>::infinity());
      }
      glm::vec3 c = integrator->Trace(sc.scene->camera->CastRay(x, y));
      for (int q = 0; q < 3; ++q) {
        sum[3 * i + q] += c[q];
        sq[3 * i + q] += static_cast<double>(c[q]) * c[q];
      }
    }
  }
  std::ofstream out(out_path, std::ios::binary);
  int32_t head[2] = {static_cast<int32_t>(n), spp};
  out.write(reinterpret_cast<const char *>(head), sizeof(head));
  out.write(reinterpret_cast<const char *>(sum.data()), sum.size() * sizeof(double));
  out.write(reinterpret_cast<const char *>(sq.data()), sq.size() * sizeof(double));
  return 0;
}

int Render(const char *scene, const char *out_path, int spp_override, long long seed) {
  muon::Options options = MakeOptions(false);
  muon::Parser parser(scene, options);
  muon::SceneConfig sc = parser.Parse();
  Reseed(sc, seed);
  if (spp_override > 0) sc.scene->pixel_samples = spp_override;
  const int w = sc.scene->width, h = sc.scene->height, spp = sc.scene->pixel_samples;
  std::vector<double> sum(3 * static_cast<size_t>(w) * h, 0.0), sq(sum.size(), 0.0);
  int num_tiles = muon::NumTiles(w, h, spp, 1);
  muon::TileQueue tiles(muon::TileImage(w, h, num_tiles, *sc.scene->seedgen));
  std::unique_ptr<muon::Integrator> integrator = sc.integrator_prototype->Clone();
  integrator->Init();
  absl::optional<muon::Tile> tile;
  while ((tile = tiles.TryDequeue())) {
    muon::Sampler sampler(tile.value(), spp);
    float x, y;
    while (sampler.NextSample(x, y)) {
      muon::Ray r = sc.scene->camera->CastRay(x, y);
      glm::vec3 c = integrator->Trace(r);
      size_t p = static_cast<size_t>(static_cast<int>(y)) * w + static_cast<int>(x);
      for (int k = 0; k < 3; ++k) {
        sum[3 * p + k] += c[k];
        sq[3 * p + k] += static_cast<double>(c[k]) * c[k];
      }
    }
  }
  muon::TraceStats ts = integrator->trace_stats();
  std::ofstream out(out_path, std::ios::binary);
  int32_t head[3] = {w, h, spp};
  out.write(reinterpret_cast<const char *>(head), sizeof(head));
  out.write(reinterpret_cast<const char *>(sum.data()), sum.size() * sizeof(double));
  out.write(reinterpret_cast<const char *>(sq.data()), sq.size() * sizeof(double));
  uint64_t counters[4] = {ts.primary_rays(), ts.secondary_rays(), ts.object_tests(), ts.bounds_tests()};
  out.write(reinterpret_cast<const char *>(counters), sizeof(counters));
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc >= 4 && std::string(argv[1]) == "hits") {
    return Hits(argv[2], argv[3], argc > 4 && std::string(argv[4]) == "linear");
  }
  if (argc >= 4 && std::string(argv[1]) == "render") {
    int spp = argc > 4 ? std::atoi(argv[4]) : 0;
    long long seed = argc > 5 ? std::atoll(argv[5]) : -1;
    return Render(argv[2], argv[3], spp, seed);
  }
  if (argc >= 5 && std::string(argv[1]) == "hitkeys") {
    return HitKeys(argv[2], argv[3], argv[4]);
  }
  if (argc >= 7 && std::string(argv[1]) == "pixels") {
    return Pixels(argv[2], argv[3], argv[4], std::atoi(argv[5]), std::atoll(argv[6]));
  }
  std::fprintf(stderr, "usage: ref_driver hits|hitkeys|render|pixels scene.muon ...\n");
  return 2;
}
