// C++ host layer over the C ABI (narval_gb300.h), shaped like the reference's render
// interface so reference code can switch to the GPU integrator with few changes:
//
//   narvalgb::SceneReader           io/SceneReader.h:51-54 (loadScene, getSettings, getMainCamera)
//   narvalgb::VolumetricPathIntegrator  integrators/Integrator.h:13-25 (Li, clone), batched
//   narvalgb::OfflineEngine         core/OfflineEngine.h:23-47 (coreLoop, postProcessing,
//                                   16-bit PPM written last pixel first as OfflineEngine.cpp:119-138)
//
// Header-only; link with libnarval_gb300.so. Errors throw narvalgb::Error carrying the
// ne_status and the library's message (the reference aborts with LOG(FATAL) instead).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "narval_gb300.h"

namespace narvalgb {

struct Error : std::runtime_error {
  ne_status status;
  Error(ne_status s, const std::string& m) : std::runtime_error(m + " (status " + std::to_string(s) + ")"), status(s) {}
};

struct Vec3 {
  float x, y, z;
};

// SceneReader: the parsed scene descriptor (host memory).
class SceneReader {
 public:
  SceneReader() = default;
  explicit SceneReader(const std::string& path, const std::string& resources = "") { loadScene(path, resources); }
  void loadScene(const std::string& path, const std::string& resources = "") {
    ne_scene_host* h = nullptr;
    char err[1024] = {0};
    std::string dir = resources;
    if (dir.empty()) {
      size_t p = path.find_last_of('/');
      dir = p == std::string::npos ? std::string(".") : path.substr(0, p);
    }
    ne_status st = ne_scene_host_load_json(path.c_str(), dir.c_str(), &h, err, sizeof err);
    if (st != NE_OK) throw Error(st, err);
    host_.reset(h);
  }
  const ne_scene_desc& getScene() const { return *ne_scene_host_desc(host_.get()); }
  const ne_settings& getSettings() const { return getScene().settings; }
  const ne_camera& getMainCamera() const { return getScene().camera; }

 private:
  struct Del {
    void operator()(ne_scene_host* h) const { ne_scene_host_destroy(h); }
  };
  std::unique_ptr<ne_scene_host, Del> host_;
};

// A CUDA device with one stream, and a scene uploaded to it.
class GpuScene {
 public:
  GpuScene(const SceneReader& reader, int device = 0) : settings_(reader.getSettings()) {
    ne_context* c = nullptr;
    ne_status st = ne_context_create(device, &c);
    if (st != NE_OK) throw Error(st, "no CUDA device");
    ctx_.reset(c);
    ne_scene* s = nullptr;
    st = ne_scene_upload(c, &reader.getScene(), &s);
    if (st != NE_OK) throw Error(st, ne_last_error(c));
    scene_ = s;
  }
  ~GpuScene() {
    if (scene_) ne_scene_destroy(scene_);
  }
  GpuScene(const GpuScene&) = delete;
  GpuScene& operator=(const GpuScene&) = delete;
  ne_scene* handle() const { return scene_; }
  ne_context* context() const { return ctx_.get(); }
  const ne_settings& settings() const { return settings_; }
  void check(ne_status st) const {
    if (st != NE_OK) throw Error(st, ne_last_error(ctx_.get()));
  }

 private:
  struct Del {
    void operator()(ne_context* c) const { ne_context_destroy(c); }
  };
  ne_settings settings_;
  std::unique_ptr<ne_context, Del> ctx_;
  ne_scene* scene_ = nullptr;
};

// Integrator::Li on the GPU. One ray per call works (the reference's interface) but a
// batch is what fills the device.
class VolumetricPathIntegrator {
 public:
  explicit VolumetricPathIntegrator(const GpuScene& scene, uint64_t seed = 0) : scene_(&scene), seed_(seed) {}
  Vec3 Li(const ne_ray& ray, ne_path_key key, uint32_t firstDim = 0) const {
    std::vector<Vec3> out = LiBatch(&ray, &key, 1, firstDim);
    return out[0];
  }
  std::vector<Vec3> LiBatch(const ne_ray* rays, const ne_path_key* keys, size_t n, uint32_t firstDim = 0) const {
    ne_render_params p = params();
    std::vector<Vec3> out(n);
    scene_->check(ne_li_batch(scene_->handle(), &p, rays, keys, n, firstDim, reinterpret_cast<float*>(out.data())));
    return out;
  }
  VolumetricPathIntegrator* clone() const { return new VolumetricPathIntegrator(*scene_, seed_); }

 private:
  ne_render_params params() const {
    ne_render_params p = {seed_, 0, -1, -1, 3, 0, 0};
    return p;
  }
  const GpuScene* scene_;
  uint64_t seed_;
};

// OfflineEngine: renders the scene's settings, tone maps like postProcessing and writes
// the reference's 16-bit binary PPM.
class OfflineEngine {
 public:
  explicit OfflineEngine(const GpuScene& scene, uint64_t seed = 0, bool refTiles = true)
      : scene_(&scene), seed_(seed), refTiles_(refTiles) {}

  // core/OfflineEngine.cpp:27-52: exposure 0.5, gamma 2.2, clamp to [0, 1].
  static Vec3 postProcessing(Vec3 hdr) {
    auto f = [](float c) {
      float m = 1.0f - std::exp(-c * 0.5f);
      m = std::pow(m, 1.0f / 2.2f);
      return m < 0.0f ? 0.0f : (m > 1.0f ? 1.0f : m);
    };
    return Vec3{f(hdr.x), f(hdr.y), f(hdr.z)};
  }

  ne_render_stats render(std::vector<Vec3>& hdr) const {
    const ne_settings& s = scene_->settings();
    hdr.assign((size_t)s.width * s.height, Vec3{0, 0, 0});
    ne_render_params p = {seed_, 0, -1, -1, 3, 0, refTiles_ ? NE_RENDER_REF_TILES : 0u};
    ne_render_stats st;
    scene_->check(ne_render(scene_->handle(), &p, reinterpret_cast<float*>(hdr.data()), &st));
    return st;
  }

  // core/OfflineEngine.cpp:78-146.
  ne_render_stats coreLoop(const std::string& path = "output.ppm") {
    std::vector<Vec3> hdr;
    ne_render_stats st = render(hdr);
    pixels.resize(hdr.size());
    for (size_t i = 0; i < hdr.size(); i++) pixels[i] = postProcessing(hdr[i]);
    const ne_settings& s = scene_->settings();
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw Error(NE_ERR_INVALID_ARG, "cannot open " + path);
    const int maxValue = 65535;
    std::fprintf(f, "P6\n%d %d\n%d\n", s.width, s.height, maxValue);
    for (long i = (long)pixels.size() - 1; i >= 0; i--) {
      const float c[3] = {pixels[i].x, pixels[i].y, pixels[i].z};
      for (float v : c) {
        // v is in [0, 1] after postProcessing, or NaN (a NaN path): written as 0, the value the
        // reference's undefined NaN-to-integer conversion gives on x86-64 and AArch64
        uint16_t q = (v >= 0.0f) ? (uint16_t)(v * maxValue) : (uint16_t)0;
        unsigned char out[2] = {(unsigned char)((q >> 8) & 0xFF), (unsigned char)(q & 0xFF)};
        std::fwrite(out, 1, 2, f);
      }
    }
    std::fclose(f);
    return st;
  }

  std::vector<Vec3> pixels;

 private:
  const GpuScene* scene_;
  uint64_t seed_;
  bool refTiles_;
};

}  // namespace narvalgb
