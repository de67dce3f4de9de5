// ref_launch.cu — host side of the reference harness (test infrastructure,
// part of the oracle; never linked into libpbf).
//
// Runs the reference's own kernels — compiled unmodified from
// fluids/Simulator.cu + fluids/Simulator_kernel.cuh into a device-only cubin
// by build_ref.py — on a GPU.  This file restates only the host sequencing of
// Simulator::step (fluids/Simulator.cpp:10-99, fluids/Simulator.cu:165-273)
// and the host-side constructors of the functors the kernels take by value,
// with device pointers in place of the OpenGL interop mapping.  The sort and
// the copy are the same thrust calls the reference makes.
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/copy.h>
#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/sort.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/pbf.h"

namespace {

// Host mirrors of the functor types the reference kernels take by value
// (declaration order = layout).
struct GridXyz {  // getGridxyz / getGridId, fluids/Simulator.cu:22-27, :56-62
  float3 llim;
  float h;
  int3 gridDim;
};
struct XyzToId {  // fluids/Simulator.cu:39-42
  int3 gridDim;
};
struct DensityBoundaryArgs {  // fluids/Simulator.cu:139-142
  float3 ulim, llim;
  float h;
};
struct Poly6 {  // fluids/Simulator.cu:75-83
  float coef, h2;
};
struct SpikyGrad {  // fluids/Simulator.cu:92-98
  float h, coef;
};
struct UpdateVelocity {  // fluids/Simulator.cu:127-129
  float inv_dt;
};
static_assert(sizeof(GridXyz) == 28 && sizeof(XyzToId) == 12 && sizeof(DensityBoundaryArgs) == 28 &&
                  sizeof(Poly6) == 8 && sizeof(SpikyGrad) == 8 && sizeof(UpdateVelocity) == 4,
              "functor layouts");

constexpr double kRefPi = 3.14159265359;  // fluids/helper.h:4

// getPoly6(float h) (fluids/Simulator.cu:77-83).
Poly6 make_poly6(float h) {
  Poly6 p;
  p.h2 = h * h;
  const float ih = 1.f / h;
  const float ih3 = ih * ih * ih;
  const float ih9 = ih3 * ih3 * ih3;
  p.coef = (float)((double)(315.f * ih9) / (64.0 * kRefPi));
  return p;
}

// getPoly6::operator() on the host (fluids/Simulator.cu:84-89).
float poly6_host(const Poly6& p, float r2) {
  if (r2 >= p.h2) return 0;
  const float d = p.h2 - r2;
  return p.coef * d * d * d;
}

// getSpikyGrad(float h) (fluids/Simulator.cu:94-98).
SpikyGrad make_spiky(float h) {
  SpikyGrad s;
  s.h = h;
  float h6 = h * h;
  h6 = h6 * h6 * h6;
  s.coef = (float)(-45.0 / (kRefPi * (double)h6));
  return s;
}

char g_err[512] = "";
CUmodule g_mod = nullptr;
CUfunction f_advect, f_range, f_lambda, f_tpos, f_xsph, f_gridid, f_updvel;

int fail(const char* what, int code) {
  snprintf(g_err, sizeof(g_err), "%s", what);
  return code;
}

#define RT(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      snprintf(g_err, sizeof(g_err), "%s: %s", #call, cudaGetErrorString(e_)); \
      return 3;                                                               \
    }                                                                         \
  } while (0)

#define DRV(call)                                                   \
  do {                                                              \
    CUresult r_ = (call);                                           \
    if (r_ != CUDA_SUCCESS) {                                       \
      const char* s_ = nullptr;                                     \
      cuGetErrorString(r_, &s_);                                    \
      snprintf(g_err, sizeof(g_err), "%s: %s", #call, s_ ? s_ : "?"); \
      return 4;                                                     \
    }                                                               \
  } while (0)

int launch(CUfunction f, int n, int block, unsigned smem, void** args) {
  const int grid = (n + block - 1) / block;  // ceilDiv (fluids/helper.h:13)
  DRV(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, 0, args, nullptr));
  return 0;
}

struct DeviceState {
  float3 *pos = nullptr, *npos = nullptr, *vel = nullptr, *nvel = nullptr, *tpos = nullptr;
  unsigned *iid = nullptr, *gridId = nullptr, *gridStart = nullptr, *gridEnd = nullptr;
  float *lambda = nullptr, *pho = nullptr;
  int cap = 0, cells_cap = 0;
};

int alloc_state(DeviceState& d, int n, int cells) {
  RT(cudaMalloc(&d.pos, sizeof(float3) * n));
  RT(cudaMalloc(&d.npos, sizeof(float3) * n));
  RT(cudaMalloc(&d.vel, sizeof(float3) * n));
  RT(cudaMalloc(&d.nvel, sizeof(float3) * n));
  RT(cudaMalloc(&d.tpos, sizeof(float3) * n));
  RT(cudaMalloc(&d.iid, sizeof(unsigned) * n));
  RT(cudaMalloc(&d.gridId, sizeof(unsigned) * n));
  RT(cudaMalloc(&d.gridStart, sizeof(unsigned) * cells));
  RT(cudaMalloc(&d.gridEnd, sizeof(unsigned) * cells));
  RT(cudaMalloc(&d.lambda, sizeof(float) * n));
  RT(cudaMalloc(&d.pho, sizeof(float) * n));
  d.cap = n;
  d.cells_cap = cells;
  return 0;
}

void free_state(DeviceState& d) {
  void* p[] = {d.pos, d.npos, d.vel, d.nvel, d.tpos, d.iid, d.gridId, d.gridStart, d.gridEnd, d.lambda, d.pho};
  for (void* q : p)
    if (q) cudaFree(q);
  d = DeviceState();
}

int3 grid_dims(const float ulim[3], const float llim[3], float h) {
  // fluids/Simulator.cu:187-188
  const float dx = ulim[0] - llim[0], dy = ulim[1] - llim[1], dz = ulim[2] - llim[2];
  return make_int3((int)ceilf(dx / h), (int)ceilf(dy / h), (int)ceilf(dz / h));
}

// One Simulator::step on device state d (roles pos/npos/vel/nvel as given).
// sync: keep the reference's cudaDeviceSynchronize between phases
// (fluids/Simulator.cpp:44-79).
int ref_step_device(const pbf_params& P, const float ulim_[3], const float llim_[3], DeviceState& d,
                    float3* pos, float3* npos, float3* vel, float3* nvel, int n, bool sync) {
  const float3 ulim = make_float3(ulim_[0], ulim_[1], ulim_[2]);
  const float3 llim = make_float3(llim_[0], llim_[1], llim_[2]);
  const float h = P.h;
  const int3 dims = grid_dims(ulim_, llim_, h);
  const long long cells = (long long)dims.x * dims.y * dims.z;
  if (cells > d.cells_cap) return fail("grid larger than allocated", 2);
  float dt = P.dt;
  // advect (fluids/Simulator.cu:165-176); gravity along -up (the reference: (0, 0, -g))
  float3 g = make_float3(P.up[0] == 0.f ? 0.f : -P.g * P.up[0], P.up[1] == 0.f ? 0.f : -P.g * P.up[1],
                         P.up[2] == 0.f ? 0.f : -P.g * P.up[2]);
  {
    void* args[] = {&d.iid, &pos, &npos, &vel, &n, &dt, &g, (void*)&ulim, (void*)&llim};
    if (int r = launch(f_advect, n, 128, 0, args)) return r;
  }
  if (sync) RT(cudaDeviceSynchronize());
  // buildGridHash (fluids/Simulator.cu:178-211)
  GridXyz gx{llim, h, dims};
  {
    void* args[] = {&npos, &d.gridId, &n, &gx};
    if (int r = launch(f_gridid, n, 128, 0, args)) return r;
  }
  {
    thrust::device_ptr<float3> t_pos(pos), t_vel(vel), t_npos(npos), t_nvel(nvel);
    thrust::device_ptr<unsigned> t_id(d.gridId), t_iid(d.iid);
    thrust::sort_by_key(t_id, t_id + n,
                        thrust::make_zip_iterator(thrust::make_tuple(t_pos, t_vel, t_npos, t_nvel, t_iid)));
  }
  RT(cudaMemset(d.gridStart, 0, sizeof(unsigned) * cells));
  RT(cudaMemset(d.gridEnd, 0, sizeof(unsigned) * cells));
  {
    void* args[] = {&d.gridId, &d.gridStart, &d.gridEnd, &n};
    if (int r = launch(f_range, n, 128, sizeof(unsigned) * (128 + 2), args)) return r;
  }
  if (sync) RT(cudaDeviceSynchronize());
  // correctDensity x niter (fluids/Simulator.cu:213-249)
  XyzToId xi{dims};
  DensityBoundaryArgs db{ulim, llim, h};
  Poly6 p6 = make_poly6(h);
  SpikyGrad sp = make_spiky(h);
  float pho0 = P.pho0, eps = P.lambda_eps, kb = P.k_boundaryDensity, n_corr = P.n_corr;
  const float coef_corr = -P.k_corr / powf(poly6_host(p6, P.delta_q * P.delta_q), P.n_corr);
  for (int it = 0; it < P.niter; ++it) {
    {
      void* args[] = {&d.iid, &d.lambda, &d.pho, &d.gridId, &d.gridStart, &d.gridEnd, (void*)&dims, &npos,
                      &n, &pho0, &eps, &kb, (void*)&h, &gx, &xi, &db, &p6, &sp};
      if (int r = launch(f_lambda, n, 128, 0, args)) return r;
    }
    {
      float cc = coef_corr;
      void* args[] = {&d.lambda, &d.iid, &d.gridId, &d.gridStart, &d.gridEnd, (void*)&dims, &npos, &d.tpos,
                      &n, &pho0, (void*)&h, &cc, &n_corr, &gx, &xi, (void*)&ulim, (void*)&llim, &p6, &sp};
      if (int r = launch(f_tpos, n, 128, 0, args)) return r;
    }
    thrust::copy_n(thrust::device_ptr<float3>(d.tpos), n, thrust::device_ptr<float3>(npos));
  }
  if (sync) RT(cudaDeviceSynchronize());
  // updateVelocity (fluids/Simulator.cu:267-273)
  {
    UpdateVelocity uv{1.f / dt};
    void* args[] = {&pos, &npos, &vel, &n, &uv};
    if (int r = launch(f_updvel, n, 128, 0, args)) return r;
  }
  if (sync) RT(cudaDeviceSynchronize());
  // correctVelocity (fluids/Simulator.cu:251-265)
  {
    float c = P.c_XSPH;
    void* args[] = {&d.pho, &d.iid, &d.gridStart, &d.gridEnd, (void*)&dims, &npos, &vel, &nvel, &n, &c,
                    (void*)&h, &gx, &xi, &p6};
    if (int r = launch(f_xsph, n, 128, 0, args)) return r;
  }
  if (sync) RT(cudaDeviceSynchronize());
  RT(cudaGetLastError());
  return 0;
}

}  // namespace

extern "C" {

const char* pbfref_last_error(void) { return g_err; }

// Loads the cubin and finds the kernels by name.
int pbfref_init(const char* cubin_path) {
  if (g_mod) return 0;
  RT(cudaFree(nullptr));  // create the primary context
  DRV(cuModuleLoad(&g_mod, cubin_path));
  unsigned count = 0;
  DRV(cuModuleGetFunctionCount(&count, g_mod));
  CUfunction* fs = new CUfunction[count];
  if (cuModuleEnumerateFunctions(fs, count, g_mod) != CUDA_SUCCESS) {
    delete[] fs;
    return fail("cuModuleEnumerateFunctions failed", 4);
  }
  struct Want {
    const char* needle;
    CUfunction* out;
    bool exact;
  } want[] = {{"13advect_kernel", &f_advect, false},
              {"16computeGridRange", &f_range, false},
              {"13computeLambda", &f_lambda, false},
              {"11computetpos", &f_tpos, false},
              {"11computeXSPH", &f_xsph, false},
              {"pbfref_grid_id", &f_gridid, true},
              {"pbfref_update_velocity", &f_updvel, true}};
  for (auto& w : want) *w.out = nullptr;
  for (unsigned k = 0; k < count; ++k) {
    const char* name = nullptr;
    if (cuFuncGetName(&name, fs[k]) != CUDA_SUCCESS || !name) continue;
    for (auto& w : want) {
      const bool hit = w.exact ? std::strcmp(name, w.needle) == 0 : std::strstr(name, w.needle) != nullptr;
      if (hit) {
        if (*w.out) {
          delete[] fs;
          return fail("kernel name matched twice", 5);
        }
        *w.out = fs[k];
      }
    }
  }
  delete[] fs;
  for (auto& w : want)
    if (!*w.out) {
      snprintf(g_err, sizeof(g_err), "kernel %s not found in the cubin", w.needle);
      return 5;
    }
  return 0;
}

// One reference step on host float3 arrays.  pos/vel/iid are permuted in place
// and vel is overwritten as in the reference; npos/nvel receive the new state.
// Optional outputs (may be NULL): rho/lambda of the last lambda pass, the
// sorted cell ids, start/end per cell (cells = dims product), dims.
int pbfref_step(const pbf_params* P, const float ulim[3], const float llim[3], float* h_pos, float* h_vel,
                float* h_npos, float* h_nvel, unsigned* h_iid, int n, float* h_rho, float* h_lambda,
                unsigned* h_ids, unsigned* h_start, unsigned* h_end, int dims_out[3]) {
  if (!g_mod) return fail("pbfref_init not called", 1);
  if (n <= 0) return fail("n must be positive", 1);
  const int3 dims = grid_dims(ulim, llim, P->h);
  const long long cells = (long long)dims.x * dims.y * dims.z;
  if (dims_out) {
    dims_out[0] = dims.x;
    dims_out[1] = dims.y;
    dims_out[2] = dims.z;
  }
  DeviceState d;
  int r = alloc_state(d, n, (int)cells);
  if (r) {
    free_state(d);
    return r;
  }
  const size_t b3 = sizeof(float3) * n;
  r = [&]() -> int {
    RT(cudaMemcpy(d.pos, h_pos, b3, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d.vel, h_vel, b3, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d.iid, h_iid, sizeof(unsigned) * n, cudaMemcpyHostToDevice));
    RT(cudaMemset(d.npos, 0, b3));
    RT(cudaMemset(d.nvel, 0, b3));
    if (int q = ref_step_device(*P, ulim, llim, d, d.pos, d.npos, d.vel, d.nvel, n, true)) return q;
    RT(cudaMemcpy(h_pos, d.pos, b3, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(h_vel, d.vel, b3, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(h_npos, d.npos, b3, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(h_nvel, d.nvel, b3, cudaMemcpyDeviceToHost));
    RT(cudaMemcpy(h_iid, d.iid, sizeof(unsigned) * n, cudaMemcpyDeviceToHost));
    if (h_rho) RT(cudaMemcpy(h_rho, d.pho, sizeof(float) * n, cudaMemcpyDeviceToHost));
    if (h_lambda) RT(cudaMemcpy(h_lambda, d.lambda, sizeof(float) * n, cudaMemcpyDeviceToHost));
    if (h_ids) RT(cudaMemcpy(h_ids, d.gridId, sizeof(unsigned) * n, cudaMemcpyDeviceToHost));
    if (h_start) RT(cudaMemcpy(h_start, d.gridStart, sizeof(unsigned) * cells, cudaMemcpyDeviceToHost));
    if (h_end) RT(cudaMemcpy(h_end, d.gridEnd, sizeof(unsigned) * cells, cudaMemcpyDeviceToHost));
    return 0;
  }();
  free_state(d);
  return r;
}

// Times `steps` reference steps after `warmup` untimed ones on device-resident
// state (tic-toc roles as fluids/FluidSystem.cpp:112-117), with the
// reference's per-phase device synchronisation (sync != 0) or without it (the
// same launches, stream-ordered).  ulim_x[k] is the x-max wall of step k
// (warm-up steps first); ms_out receives the total time of the timed steps
// (CUDA events around them, in ms).
int pbfref_bench(const pbf_params* P, const float ulim[3], const float llim[3], const float* h_pos,
                 const float* h_vel, int n, int warmup, int steps, const float* ulim_x, int sync,
                 double* ms_out) {
  if (!g_mod) return fail("pbfref_init not called", 1);
  const int3 dims = grid_dims(ulim, llim, P->h);
  const long long cells = (long long)dims.x * dims.y * dims.z;
  DeviceState d;
  int r = alloc_state(d, n, (int)cells);
  if (r) {
    free_state(d);
    return r;
  }
  r = [&]() -> int {
    const size_t b3 = sizeof(float3) * n;
    RT(cudaMemcpy(d.pos, h_pos, b3, cudaMemcpyHostToDevice));
    RT(cudaMemcpy(d.vel, h_vel, b3, cudaMemcpyHostToDevice));
    unsigned* iid = new unsigned[n];
    for (int k = 0; k < n; ++k) iid[k] = (unsigned)k;
    cudaError_t e = cudaMemcpy(d.iid, iid, sizeof(unsigned) * n, cudaMemcpyHostToDevice);
    delete[] iid;
    RT(e);
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    bool tic = false;
    for (int k = 0; k < warmup + steps; ++k) {
      if (k == warmup) {
        RT(cudaDeviceSynchronize());
        RT(cudaEventRecord(e0));
      }
      float u[3] = {ulim_x ? ulim_x[k] : ulim[0], ulim[1], ulim[2]};
      int q = tic ? ref_step_device(*P, u, llim, d, d.npos, d.pos, d.nvel, d.vel, n, sync != 0)
                  : ref_step_device(*P, u, llim, d, d.pos, d.npos, d.vel, d.nvel, n, sync != 0);
      if (q) return q;
      tic = !tic;
    }
    RT(cudaEventRecord(e1));
    RT(cudaEventSynchronize(e1));
    float ms = 0.f;
    RT(cudaEventElapsedTime(&ms, e0, e1));
    *ms_out = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return 0;
  }();
  free_state(d);
  return r;
}

}  // extern "C"
