// SSFRenderer.hpp — header-only C++ facade with the reference's class shape
// (fluids/SSFRenderer.h:4-74) over the C ABI of include/pbf_ssf.h, for C++
// callers that replace `#include "SSFRenderer.h"`.
//
// Differences from the reference class, all forced by the headless boundary:
//  - the constructor takes the renderer parameters (camera matrices included)
//    instead of a Camera* and a GL sky texture; the sky is a host cube map
//    (setSky) or a uniform colour;
//  - render() takes device positions (float4) and a device colour image
//    instead of a vertex array object, plus an optional stream;
//  - loadParams() takes the parameter struct instead of reading the
//    GUIParams singleton;
//  - errors throw pbf::Error instead of exit()ing.
#pragma once

#include "../../include/pbf_ssf.h"
#include "Simulator.hpp"

namespace pbf {

class SSFRenderer {
 public:
  // fluids/SSFRenderer.h:14 — SSFRenderer(Camera*, width, height, sky_texture).
  explicit SSFRenderer(const pbf_ssf_params& params) { check(pbf_ssf_create(&params, &r_), "pbf_ssf_create"); }
  ~SSFRenderer() { pbf_ssf_destroy(r_); }
  SSFRenderer(const SSFRenderer&) = delete;
  SSFRenderer& operator=(const SSFRenderer&) = delete;

  // The reference's settings and camera at width x height.
  static pbf_ssf_params defaults(int width = 1600, int height = 1200) {
    pbf_ssf_params p;
    pbf_ssf_params_default(&p);
    p.width = width;
    p.height = height;
    const float pos[3] = {1.f, -5.f, 2.f}, focus[3] = {0.f, 0.f, 1.5f};
    check(pbf_ssf_look_at(&p, pos, focus, 60.f), "pbf_ssf_look_at");
    return p;
  }

  // fluids/SSFRenderer.h:18 — render(p_vao, nparticle): device positions in,
  // device colour image (width x height float4) out.
  void render(const void* d_pos, int nparticle, void* d_color, void* stream = nullptr) {
    check(pbf_ssf_render(r_, d_pos, nparticle, d_color, stream), "pbf_ssf_render");
  }

  // fluids/SSFRenderer.h:28 — loadParams().
  void loadParams(const pbf_ssf_params& p) { check(pbf_ssf_set_params(r_, &p), "pbf_ssf_set_params"); }
  pbf_ssf_params params() const {
    pbf_ssf_params p;
    check(pbf_ssf_get_params(r_, &p), "pbf_ssf_get_params");
    return p;
  }

  // The sky cube map: host RGB floats [6][size][size][3] in GL face order, or nullptr.
  void setSky(const float* faces, int size) { check(pbf_ssf_set_sky(r_, faces, size), "pbf_ssf_set_sky"); }

  // The last render's smoothed depth, thickness and normal_D images (device copies).
  void images(void* d_depth, void* d_thick, void* d_normal_D, void* stream = nullptr) {
    check(pbf_ssf_images(r_, d_depth, d_thick, d_normal_D, stream), "pbf_ssf_images");
  }

  pbf_ssf* handle() const { return r_; }

 private:
  pbf_ssf* r_ = nullptr;
};

}  // namespace pbf
