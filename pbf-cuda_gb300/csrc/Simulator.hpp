// Simulator.hpp — header-only C++ facade with the reference's class shape
// (fluids/Simulator.h:7-61) over the C ABI of include/pbf.h, for C++ callers
// that replace `#include "Simulator.h"`.
//
// Differences from the reference class, all forced by the headless boundary:
//  - step() takes device pointers to float4 (x, y, z, w) instead of OpenGL
//    buffer names, plus an optional stream;
//  - loadParams()/saveParams() take/return the parameter struct instead of
//    touching a GUIParams singleton;
//  - errors throw pbf::Error instead of exit()ing.
#pragma once

#include <stdexcept>
#include <string>

#include "../../include/pbf.h"

namespace pbf {

class Error : public std::runtime_error {
 public:
  Error(pbf_status s, const std::string& what) : std::runtime_error(what), status(s) {}
  pbf_status status;
};

inline void check(pbf_status s, const char* what) {
  if (s != PBF_OK)
    throw Error(s, std::string(what) + ": " + pbf_status_string(s) + ": " + pbf_last_error());
}

struct Float3 {
  float x, y, z;
};

class Simulator {
 public:
  // fluids/Simulator.h:10 — Simulator(const GUIParams&, float3 ulim, float3 llim).
  Simulator(const pbf_params& params, Float3 ulim, Float3 llim, int max_particles) {
    const float u[3] = {ulim.x, ulim.y, ulim.z}, l[3] = {llim.x, llim.y, llim.z};
    check(pbf_create(&params, u, l, max_particles, &s_), "pbf_create");
  }
  ~Simulator() { pbf_destroy(s_); }
  Simulator(const Simulator&) = delete;
  Simulator& operator=(const Simulator&) = delete;

  // fluids/Simulator.h:37 — step(d_pos, d_npos, d_vel, d_nvel, d_iid, nparticle).
  void step(void* d_pos, void* d_npos, void* d_vel, void* d_nvel, uint32_t* d_iid, int nparticle,
            void* stream = nullptr) {
    check(pbf_step(s_, d_pos, d_npos, d_vel, d_nvel, d_iid, nparticle, stream), "pbf_step");
  }

  // fluids/Simulator.h:39-40.
  void loadParams(const pbf_params& p) { check(pbf_set_params(s_, &p), "pbf_set_params"); }
  pbf_params saveParams() const {
    pbf_params p;
    check(pbf_get_params(s_, &p), "pbf_get_params");
    return p;
  }

  // fluids/Simulator.h:42.
  void setLim(const Float3& ulim, const Float3& llim) {
    const float u[3] = {ulim.x, ulim.y, ulim.z}, l[3] = {llim.x, llim.y, llim.z};
    check(pbf_set_limits(s_, u, l), "pbf_set_limits");
  }

  pbf_solver* handle() const { return s_; }

 private:
  pbf_solver* s_ = nullptr;
};

}  // namespace pbf
