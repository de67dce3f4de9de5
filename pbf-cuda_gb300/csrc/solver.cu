// solver.cu — the per-particle passes of one step, in cell order:
//   reorder   gather pos/vel/iid by the sorted permutation, recompute x*
//   lambda    density rho_i and lambda_i        computeLambda  (fluids/Simulator_kernel.cuh:52-129)
//   delta_p   s_corr, clamp, wall clamp         computetpos    (fluids/Simulator_kernel.cuh:131-194)
//             the last iteration also writes v = (x_final - x) / dt and the
//             caller's permuted pos / iid       h_updateVelocity (fluids/Simulator.cu:127-137)
//   xsph      XSPH viscosity                    computeXSPH    (fluids/Simulator_kernel.cuh:196-239)
//
// Every pass is gather-only (no atomics, no cross-thread writes), so results
// are deterministic.  Neighbour semantics follow the reference exactly: the
// grid is built once per step from x*, every pass looks up the 3x3x3 cells
// around cell(current x_i) in that (stale) grid, and candidates are visited in
// the reference's order (dx, dy outer; the three z-consecutive cells of a
// column form one contiguous run of sorted slots, visited in slot order).
// Jacobi iterations ping-pong between two position buffers instead of the
// reference's tpos -> npos copy (fluids/Simulator.cu:247-248).
//
// IEEE semantics follow the reference's: its kernels evaluate every candidate
// of the window, so a NaN distance (from a NaN position) poisons the sums, a
// non-finite lambda_j poisons delta_p through a zero gradient, and
// 0 * v / (rho_i + rho_j) is NaN when both densities are zero.  Here the
// candidate test is written NaN-inclusively (!(r2 >= h2), as the reference's
// `if (r2 >= h2) return 0`), and the two poisoning rules that need every
// candidate's lambda / density / velocity run only when a per-step flag says
// such a value exists (StepFlag); otherwise candidates outside the cutoff
// contribute exactly zero and are skipped.
#include "pbf_internal.cuh"

namespace pbf {

namespace {

constexpr int kThreads = 256;

// Sorted-slot range [s, e) of cells (x, y, z-1 .. z+1) clipped to the grid.
// cs[cells] == n, so e <= n; the clamp keeps even an inconsistent table in range.
__device__ __forceinline__ void column_run(const StepConsts& c, const uint32_t* __restrict__ cs,
                                           int n, int x, int y, int z, int& s, int& e) {
  const int zlo = max(z - 1, 0), zhi = min(z + 1, c.dims[2] - 1);
  const int base = (x * c.dims[1] + y) * c.dims[2];
  s = (int)__ldg(cs + base + zlo);
  e = min((int)__ldg(cs + base + zhi + 1), n);
}

__global__ void __launch_bounds__(kThreads)
k_reorder(const uint32_t* __restrict__ perm, const float4* __restrict__ pos,
          const float4* __restrict__ vel, const uint32_t* __restrict__ iid, int n, StepConsts c,
          float4* __restrict__ xs, float4* __restrict__ xa, uint32_t* __restrict__ iid_s,
          uint32_t* __restrict__ flags) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < kNumFlags) flags[k] = 0u;  // the step's flags start clear
  if (k >= n) return;
  const uint32_t p = min(perm[k], (uint32_t)(n - 1));  // a permutation of [0, n): the min never binds
  const float4 x = pos[p];
  const float4 v = vel[p];
  const float vx = fmaf(c.dt, c.g[0], v.x), vy = fmaf(c.dt, c.g[1], v.y),
              vz = fmaf(c.dt, c.g[2], v.z);
  xs[k] = x;
  xa[k] = make_float4(fmaf(c.dt, vx, x.x), fmaf(c.dt, vy, x.y), fmaf(c.dt, vz, x.z), x.w);
  iid_s[k] = iid[p];
}

__global__ void __launch_bounds__(kThreads)
k_lambda(const float4* __restrict__ X, const uint32_t* __restrict__ cs, int n, StepConsts c,
         float* __restrict__ lambda, float* __restrict__ rho, uint32_t* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = X[i];
  const int3 q = cell_of(c, xi);
  float pho = 0.f, gl2 = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= c.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= c.dims[1]) continue;
      int s, e;
      column_run(c, cs, n, x, y, q.z, s, e);
      for (int j = s; j < e; ++j) {
        const float4 xj = __ldg(X + j);
        const float ex = xi.x - xj.x, ey = xi.y - xj.y, ez = xi.z - xj.z;
        const float r2 = dist2(ex, ey, ez);
        if (!(r2 >= c.h2)) {  // NaN-inclusive, as getPoly6
          pho += poly6_inside(c, r2);
          if (!(r2 < c.keps2)) {  // as getSpikyGrad's |r| < KERNAL_EPS test
            const float ir = rsqrtf(r2);
            const float t = c.h - r2 * ir;
            const float sc = c.spiky_coef_rho0 * t * t * ir;
            const float ax = sc * ex, ay = sc * ey, az = sc * ez;
            gx += ax;
            gy += ay;
            gz += az;
            if (j != i) gl2 += dist2(ax, ay, az);
          }
        }
      }
    }
  }
  if (c.k_b != 0.f) pho += c.k_b * boundary_density(c, xi);
  const float grad_l2 = gl2 + dist2(gx, gy, gz);
  const float lam = -(pho / c.pho0 - 1.f) / (grad_l2 + c.lambda_eps);
  lambda[i] = lam;
  rho[i] = pho;
  if (!isfinite(lam)) atomicOr(&flags[kFlagLambdaNonFinite], 1u);
  if (!(pho > 0.f) || !isfinite(pho)) atomicOr(&flags[kFlagXsphExact], 1u);
}

// delta_p for slot i: sum over neighbours j != i of (lambda_i + lambda_j + s_corr) grad W,
// then / pho0, per-component clamp to +-max_dp, wall clamp.
// exact: also apply the reference's poisoning of the sum by a non-finite
// lambda through a zero gradient (candidates j != i outside the cutoff).
template <bool kExact>
__device__ __forceinline__ float4 delta_p(const StepConsts& c, const float4* __restrict__ X,
                                          const float* __restrict__ lambda,
                                          const uint32_t* __restrict__ cs, int n, int i,
                                          float4 xi) {
  const int3 q = cell_of(c, xi);
  const float li = lambda[i];
  float ax = 0.f, ay = 0.f, az = 0.f;
  bool poison = false;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= c.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= c.dims[1]) continue;
      int s, e;
      column_run(c, cs, n, x, y, q.z, s, e);
      for (int j = s; j < e; ++j) {
        const float4 xj = __ldg(X + j);
        const float ex = xi.x - xj.x, ey = xi.y - xj.y, ez = xi.z - xj.z;
        const float r2 = dist2(ex, ey, ez);
        if (!(r2 >= c.h2) && !(r2 < c.keps2) && j != i) {  // NaN-inclusive, as the reference
          const float w = poly6_inside(c, r2);
          const float corr = c.coef_corr * pow_corr(c, w);
          const float ir = rsqrtf(r2);
          const float t = c.h - r2 * ir;
          const float f = (li + __ldg(lambda + j) + corr) * (c.spiky_coef * t * t * ir);
          ax = fmaf(f, ex, ax);
          ay = fmaf(f, ey, ay);
          az = fmaf(f, ez, az);
        } else if (kExact && j != i) {
          // zero gradient: (lambda_i + lambda_j + s_corr) * 0 is NaN iff a lambda is not finite
          poison |= !isfinite(li) || !isfinite(__ldg(lambda + j));
        }
      }
    }
  }
  if (kExact && poison) ax = ay = az = __int_as_float(0x7fffffff);
  const float dx = fmaxf(fminf(ax / c.pho0, c.max_dp), -c.max_dp);
  const float dy = fmaxf(fminf(ay / c.pho0, c.max_dp), -c.max_dp);
  const float dz = fmaxf(fminf(az / c.pho0, c.max_dp), -c.max_dp);
  return make_float4(fmaxf(fminf(xi.x + dx, c.hi[0]), c.lo[0]),
                     fmaxf(fminf(xi.y + dy, c.hi[1]), c.lo[1]),
                     fmaxf(fminf(xi.z + dz, c.hi[2]), c.lo[2]), xi.w);
}

__global__ void __launch_bounds__(kThreads)
k_delta_p(const float4* __restrict__ X, const float* __restrict__ lambda,
          const uint32_t* __restrict__ cs, int n, StepConsts c, const uint32_t* __restrict__ flags,
          float4* __restrict__ T) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T[i] = flags[kFlagLambdaNonFinite] ? delta_p<true>(c, X, lambda, cs, n, i, X[i])
                                     : delta_p<false>(c, X, lambda, cs, n, i, X[i]);
}

// Last iteration: x_final -> npos, v = (x_final - x) * (1/dt) -> vel, and the
// caller's pos / iid receive the permuted inputs (the reference's in-place sort).
__global__ void __launch_bounds__(kThreads)
k_delta_p_final(const float4* __restrict__ X, const float* __restrict__ lambda,
                const uint32_t* __restrict__ cs, int n, StepConsts c,
                const float4* __restrict__ xs, const uint32_t* __restrict__ iid_s,
                float4* __restrict__ npos, float4* __restrict__ vel, float4* __restrict__ pos,
                uint32_t* __restrict__ iid, uint32_t* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xf = flags[kFlagLambdaNonFinite] ? delta_p<true>(c, X, lambda, cs, n, i, X[i])
                                                : delta_p<false>(c, X, lambda, cs, n, i, X[i]);
  const float4 x0 = xs[i];
  npos[i] = make_float4(xf.x, xf.y, xf.z, x0.w);
  const float4 v = make_float4((xf.x - x0.x) * c.inv_dt, (xf.y - x0.y) * c.inv_dt,
                               (xf.z - x0.z) * c.inv_dt, 0.f);
  vel[i] = v;
  if (!isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z)) atomicOr(&flags[kFlagXsphExact], 1u);
  pos[i] = x0;
  iid[i] = iid_s[i];
}

__global__ void __launch_bounds__(kThreads)
k_xsph(const float4* __restrict__ X, const float4* __restrict__ V, const float* __restrict__ rho,
       const uint32_t* __restrict__ cs, int n, StepConsts c, const uint32_t* __restrict__ flags,
       float4* __restrict__ NV) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool exact = flags[kFlagXsphExact] != 0u;
  bool px = false, py = false, pz = false;  // exact path: NaN from 0 * v / (rho_i + rho_j)
  const float4 xi = X[i];
  const float4 vi = V[i];
  const float ri = rho[i];
  const int3 q = cell_of(c, xi);
  float ax = 0.f, ay = 0.f, az = 0.f;
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= c.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= c.dims[1]) continue;
      int s, e;
      column_run(c, cs, n, x, y, q.z, s, e);
      for (int j = s; j < e; ++j) {
        const float4 xj = __ldg(X + j);
        const float r2 = dist2(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        if (!(r2 >= c.h2)) {  // NaN-inclusive, as getPoly6
          const float4 vj = __ldg(V + j);
          const float w2 = 2.f * poly6_inside(c, r2) / (ri + __ldg(rho + j));
          ax = fmaf(vj.x - vi.x, w2, ax);
          ay = fmaf(vj.y - vi.y, w2, ay);
          az = fmaf(vj.z - vi.z, w2, az);
        } else if (exact) {
          // W = 0: 2 (v_j - v_i) * 0 / (rho_i + rho_j) is NaN iff the velocity
          // difference is not finite or the denominator is 0 or NaN
          const float4 vj = __ldg(V + j);
          const float den = ri + __ldg(rho + j);
          const bool bad_den = !(den != 0.f) || isnan(den);
          px |= bad_den || !isfinite(vj.x - vi.x);
          py |= bad_den || !isfinite(vj.y - vi.y);
          pz |= bad_den || !isfinite(vj.z - vi.z);
        }
      }
    }
  }
  const float qnan = __int_as_float(0x7fffffff);
  if (px) ax = qnan;
  if (py) ay = qnan;
  if (pz) az = qnan;
  NV[i] = make_float4(fmaf(c.c_xsph, ax, vi.x), fmaf(c.c_xsph, ay, vi.y),
                      fmaf(c.c_xsph, az, vi.z), 0.f);
}

}  // namespace

cudaError_t reorder(const StepConsts& c, const uint32_t* perm, const float4* pos, const float4* vel,
                    const uint32_t* iid, int n, SolverScratch& s, cudaStream_t stream) {
  k_reorder<<<(n + kThreads - 1) / kThreads, kThreads, 0, stream>>>(perm, pos, vel, iid, n, c,
                                                                     s.xs, s.xa, s.iid_s, s.flags);
  return cudaGetLastError();
}

cudaError_t launch_lambda(const StepConsts& c, const float4* X, const uint32_t* cs, int n,
                          float* lambda, float* rho, uint32_t* flags, cudaStream_t stream) {
  k_lambda<<<(n + kThreads - 1) / kThreads, kThreads, 0, stream>>>(X, cs, n, c, lambda, rho, flags);
  return cudaGetLastError();
}

cudaError_t launch_delta_p(const StepConsts& c, const float4* X, const float* lambda,
                           const uint32_t* cs, int n, const uint32_t* flags, float4* T,
                           cudaStream_t stream) {
  k_delta_p<<<(n + kThreads - 1) / kThreads, kThreads, 0, stream>>>(X, lambda, cs, n, c, flags, T);
  return cudaGetLastError();
}

cudaError_t launch_delta_p_final(const StepConsts& c, const float4* X, const float* lambda,
                                 const uint32_t* cs, int n, const SolverScratch& s, float4* pos,
                                 float4* npos, float4* vel, uint32_t* iid, cudaStream_t stream) {
  k_delta_p_final<<<(n + kThreads - 1) / kThreads, kThreads, 0, stream>>>(
      X, lambda, cs, n, c, s.xs, s.iid_s, npos, vel, pos, iid, s.flags);
  return cudaGetLastError();
}

cudaError_t launch_xsph(const StepConsts& c, const float4* X, const float4* V, const float* rho,
                        const uint32_t* cs, int n, const uint32_t* flags, float4* NV,
                        cudaStream_t stream) {
  k_xsph<<<(n + kThreads - 1) / kThreads, kThreads, 0, stream>>>(X, V, rho, cs, n, c, flags, NV);
  return cudaGetLastError();
}

}  // namespace pbf
