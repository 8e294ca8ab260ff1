// Host-side entry points of the C ABI: scene parsing and film output.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "host_scene.h"

using namespace muon_gpu;

struct MuonParsedScene {
  ParsedScene scene;
};

namespace {

int Fail(int code, const std::string &msg) {
  SetLastError(msg);
  return code;
}

// CRC-32 (ISO-HDLC polynomial 0xEDB88320) and Adler-32 for the PNG container.
uint32_t Crc32(const uint8_t *p, size_t n, uint32_t crc = 0) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    init = true;
  }
  crc = ~crc;
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
  return ~crc;
}

void Put32(std::vector<uint8_t> &v, uint32_t x) {
  v.push_back(x >> 24), v.push_back(x >> 16), v.push_back(x >> 8), v.push_back(x);
}

void Chunk(std::vector<uint8_t> &png, const char *kind, const std::vector<uint8_t> &body) {
  Put32(png, static_cast<uint32_t>(body.size()));
  size_t start = png.size();
  png.insert(png.end(), kind, kind + 4);
  png.insert(png.end(), body.begin(), body.end());
  Put32(png, Crc32(png.data() + start, png.size() - start));
}

// 8-bit RGB PNG with the image data in stored (uncompressed) deflate blocks,
// which needs no compression library.
bool WritePng(const std::string &path, const uint8_t *rgb, int w, int h) {
  std::vector<uint8_t> raw;
  raw.reserve(static_cast<size_t>(h) * (3 * w + 1));
  for (int y = 0; y < h; ++y) {
    raw.push_back(0);
    raw.insert(raw.end(), rgb + static_cast<size_t>(y) * 3 * w, rgb + static_cast<size_t>(y + 1) * 3 * w);
  }
  std::vector<uint8_t> z = {0x78, 0x01};
  uint32_t a = 1, b = 0;
  for (uint8_t c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  size_t pos = 0;
  do {
    size_t len = std::min<size_t>(65535, raw.size() - pos);
    bool final = pos + len == raw.size();
    z.push_back(final ? 1 : 0);
    z.push_back(len & 0xff), z.push_back(len >> 8);
    z.push_back(~len & 0xff), z.push_back((~len >> 8) & 0xff);
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
    pos += len;
  } while (pos < raw.size());
  Put32(z, (b << 16) | a);
  std::vector<uint8_t> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  std::vector<uint8_t> ihdr;
  Put32(ihdr, w), Put32(ihdr, h);
  ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});
  Chunk(png, "IHDR", ihdr);
  Chunk(png, "IDAT", z);
  Chunk(png, "IEND", {});
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char *>(png.data()), png.size());
  return static_cast<bool>(f);
}

bool WritePpm(const std::string &path, const uint8_t *rgb, int w, int h) {
  std::ofstream f(path, std::ios::binary);
  f << "P6\n" << w << " " << h << "\n255\n";
  f.write(reinterpret_cast<const char *>(rgb), static_cast<std::streamsize>(3) * w * h);
  return static_cast<bool>(f);
}

int ParseInto(const std::string &text, const std::string &base, MuonParsedScene **out) {
  if (!out) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  try {
    std::unique_ptr<MuonParsedScene> s(new MuonParsedScene());
    std::string err;
    if (!ParseScene(text, base, &s->scene, &err)) return Fail(MUON_ERR_PARSE, err);
    *out = s.release();
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed while parsing");
  }
  return MUON_OK;
}

}  // namespace

extern "C" {

int muon_parse_scene_file(const char *path, MuonParsedScene **out) {
  if (!path) return Fail(MUON_ERR_INVALID_ARG, "null path");
  std::ifstream f(path);
  if (!f) return Fail(MUON_ERR_PARSE, std::string("cannot open scene file ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  std::string p(path);
  size_t slash = p.find_last_of('/');
  return ParseInto(ss.str(), slash == std::string::npos ? "." : p.substr(0, slash), out);
}

int muon_parse_scene_string(const char *text, const char *base_dir, MuonParsedScene **out) {
  if (!text) return Fail(MUON_ERR_INVALID_ARG, "null text");
  return ParseInto(text, base_dir ? base_dir : ".", out);
}

int muon_parsed_scene_desc(const MuonParsedScene *s, MuonSceneDesc *desc, MuonRenderParams *params) {
  if (!s || !desc) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  const ParsedScene &p = s->scene;
  MuonSceneDesc d{};
  d.width = p.width;
  d.height = p.height;
  d.camera = p.camera;
  d.transforms = p.transforms.data();
  d.num_transforms = static_cast<int32_t>(p.transforms.size());
  d.materials = p.materials.data();
  d.num_materials = static_cast<int32_t>(p.materials.size());
  d.lights = p.lights.data();
  d.num_lights = static_cast<int32_t>(p.lights.size());
  d.triangles = p.triangles.data();
  d.num_triangles = static_cast<int64_t>(p.triangles.size());
  d.spheres = p.spheres.data();
  d.num_spheres = static_cast<int64_t>(p.spheres.size());
  d.acceleration = MUON_ACCEL_BVH;
  d.partition_strategy = MUON_PARTITION_SAH;
  d.max_leaf_size = 0;
  *desc = d;
  if (params) *params = p.params;
  return MUON_OK;
}

float muon_parsed_scene_gamma(const MuonParsedScene *s) { return s ? s->scene.gamma : 1.0f; }
const char *muon_parsed_scene_output(const MuonParsedScene *s) {
  return s && s->scene.has_output ? s->scene.output.c_str() : nullptr;
}
int32_t muon_parsed_scene_warnings(const MuonParsedScene *s) { return s ? s->scene.warnings : 0; }
void muon_parsed_scene_free(MuonParsedScene *s) { delete s; }

int muon_film_tonemap(const MuonFilm *film, float gamma, uint8_t *rgb) {
  if (!film || !film->sum || !film->count || !rgb || film->width <= 0 || film->height <= 0)
    return Fail(MUON_ERR_INVALID_ARG, "bad film");
  // Film::WriteOutput (muon/film.cc:21-43): the FP32 mean over the samples,
  // gamma via powf, clamp to [0, 1], times 255 truncated to a byte.
  const float inv_gamma = 1.0f / gamma;
  const size_t np = static_cast<size_t>(film->width) * film->height;
  for (size_t i = 0; i < np; ++i) {
    float n = static_cast<float>(film->count[i]);
    for (int c = 0; c < 3; ++c) {
      float v = n > 0.0f ? static_cast<float>(film->sum[3 * i + c]) / n : 0.0f;
      v = powf(v, inv_gamma);
      v = mm::clamp_ref(v, 0.0f, 1.0f);
      rgb[3 * i + c] = static_cast<uint8_t>(v * 255);
    }
  }
  return MUON_OK;
}

int muon_film_write(const MuonFilm *film, float gamma, const char *path) {
  if (!path) return Fail(MUON_ERR_INVALID_ARG, "null path");
  std::vector<uint8_t> rgb;
  try {
    rgb.resize(3 * static_cast<size_t>(film ? film->width : 0) * (film ? film->height : 0));
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  int rc = muon_film_tonemap(film, gamma, rgb.data());
  if (rc != MUON_OK) return rc;
  std::string p(path);
  bool png = p.size() >= 4 && (p.compare(p.size() - 4, 4, ".png") == 0 || p.compare(p.size() - 4, 4, ".PNG") == 0);
  bool ok = png ? WritePng(p, rgb.data(), film->width, film->height) : WritePpm(p, rgb.data(), film->width, film->height);
  return ok ? MUON_OK : Fail(MUON_ERR_IO, "cannot write " + p);
}

}  // extern "C"
