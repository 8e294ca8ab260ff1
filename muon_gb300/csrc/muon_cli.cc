// `muon` command-line renderer on the GPU path. Accepts the reference CLI's
// flags (muon/muon.cc:12-21): --scene, --output, --acceleration,
// --partition_strategy, --parallelism (host threads; unused, the GPU renders),
// --stats; plus --samples / --seed overrides and --intersect_mode.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/muon_gpu.h"

namespace {

const char kUsage[] =
    "usage: muon --scene=FILE [--output=FILE] [--acceleration=bvh|linear]\n"
    "            [--partition_strategy=sah|midpoint|uniform] [--parallelism=N] [--stats[=true|false]]\n"
    "            [--samples=N] [--seed=N] [--intersect_mode=exact|fast|watertight]\n"
    "Renders a .muon scene on the GPU and writes its film (PNG or PPM).\n";

bool Flag(const char *arg, const char *name, std::string *value) {
  size_t n = std::strlen(name);
  if (std::strncmp(arg, name, n) != 0) return false;
  if (arg[n] == '=') {
    *value = arg + n + 1;
    return true;
  }
  if (arg[n] == '\0') {
    *value = "";
    return true;
  }
  return false;
}

}  // namespace

int main(int argc, char **argv) {
  std::string scene, output, accel = "bvh", partition = "sah", stats = "true", samples, seed, tri = "exact";
  for (int i = 1; i < argc; ++i) {
    std::string v;
    if (Flag(argv[i], "--scene", &v)) scene = v;
    else if (Flag(argv[i], "--output", &v)) output = v;
    else if (Flag(argv[i], "--acceleration", &v)) accel = v;
    else if (Flag(argv[i], "--partition_strategy", &v)) partition = v;
    else if (Flag(argv[i], "--parallelism", &v)) continue;
    else if (Flag(argv[i], "--stats", &v)) stats = v.empty() ? "true" : v;
    else if (Flag(argv[i], "--samples", &v)) samples = v;
    else if (Flag(argv[i], "--seed", &v)) seed = v;
    else if (Flag(argv[i], "--intersect_mode", &v)) tri = v;
    else if (Flag(argv[i], "--help", &v) || Flag(argv[i], "-h", &v)) {
      std::fputs(kUsage, stdout);
      return 0;
    } else {
      std::fprintf(stderr, "unknown flag %s\n%s", argv[i], kUsage);
      return 1;
    }
  }
  if (scene.empty()) {
    std::fprintf(stderr, "A scene file is required\n%s", kUsage);
    return 1;
  }
  if (tri != "exact" && tri != "fast" && tri != "watertight") {
    std::fprintf(stderr, "unknown value for intersect_mode\n");
    return 1;
  }
  auto t_start = std::chrono::steady_clock::now();
  MuonParsedScene *ps = nullptr;
  if (muon_parse_scene_file(scene.c_str(), &ps) != MUON_OK) {
    std::fprintf(stderr, "parse failed: %s\n", muon_gpu_last_error());
    return 1;
  }
  MuonSceneDesc desc;
  MuonRenderParams params;
  muon_parsed_scene_desc(ps, &desc, &params);
  if (accel == "linear") desc.acceleration = MUON_ACCEL_LINEAR;
  else if (accel == "bvh") desc.acceleration = MUON_ACCEL_BVH;
  else {
    std::fprintf(stderr, "unknown value for acceleration\n");
    return 1;
  }
  if (partition == "uniform") desc.partition_strategy = MUON_PARTITION_UNIFORM;
  else if (partition == "midpoint") desc.partition_strategy = MUON_PARTITION_MIDPOINT;
  else if (partition == "sah") desc.partition_strategy = MUON_PARTITION_SAH;
  else {
    std::fprintf(stderr, "unknown value for partition_strategy\n");
    return 1;
  }
  // the SAH tree is built on the device (the same tree as the host builder's)
  // unless the scene is so small that the host is faster
  desc.builder = desc.partition_strategy == MUON_PARTITION_SAH && desc.num_triangles + desc.num_spheres >= 256
                     ? MUON_BUILDER_GPU_SAH
                     : MUON_BUILDER_HOST_SAH;
  if (!samples.empty()) params.pixel_samples = std::atoi(samples.c_str());
  if (!seed.empty()) params.seed = std::strtoull(seed.c_str(), nullptr, 10);
  params.intersect_mode = tri == "watertight" ? MUON_ISECT_WATERTIGHT : (tri == "fast" ? MUON_ISECT_FAST : MUON_ISECT_EXACT);
  MuonScene *gs = nullptr;
  if (muon_gpu_scene_create(&desc, &gs) != MUON_OK) {
    std::fprintf(stderr, "scene upload failed: %s\n", muon_gpu_last_error());
    return 1;
  }
  auto t_built = std::chrono::steady_clock::now();
  size_t np = static_cast<size_t>(desc.width) * desc.height;
  std::vector<double> sum(3 * np), sq(3 * np);
  std::vector<uint32_t> cnt(np);
  MuonFilm film{desc.width, desc.height, sum.data(), sq.data(), cnt.data()};
  if (muon_gpu_render(gs, &params, &film) != MUON_OK) {
    std::fprintf(stderr, "render failed: %s\n", muon_gpu_last_error());
    return 1;
  }
  auto t_end = std::chrono::steady_clock::now();
  const char *out = !output.empty() ? output.c_str() : muon_parsed_scene_output(ps);
  if (!out) out = "raytrace.png";
  if (muon_film_write(&film, muon_parsed_scene_gamma(ps), out) != MUON_OK) {
    std::fprintf(stderr, "write failed: %s\n", muon_gpu_last_error());
    return 1;
  }
  if (stats == "true" || stats == "1") {
    MuonStats st;
    muon_gpu_stats(gs, &st);
    double total = std::chrono::duration<double>(t_end - t_start).count();
    double build = std::chrono::duration<double>(t_built - t_start).count();
    std::fprintf(stderr, "---------------------------------------->>\n");
    std::fprintf(stderr, "%-18s : %12.2f (sec)\n", "Total time", total);
    std::fprintf(stderr, "%-18s : %12.2f (sec)\n", "Build time", build);
    std::fprintf(stderr, "%-18s : %12.2f (sec)\n", "Render time", total - build);
    std::fprintf(stderr, "%-18s : %12.3f (ms)\n", "GPU render time", st.render_ms);
    std::fprintf(stderr, "%-18s : %12llu\n", "Primary rays", (unsigned long long)st.primary_rays);
    std::fprintf(stderr, "%-18s : %12llu\n", "Secondary rays", (unsigned long long)st.secondary_rays);
    std::fprintf(stderr, "%-18s : %12llu\n", "Shadow rays", (unsigned long long)st.shadow_rays);
    std::fprintf(stderr, "---------------------------------------->>\n");
  }
  muon_gpu_scene_destroy(gs);
  muon_parsed_scene_free(ps);
  return 0;
}
