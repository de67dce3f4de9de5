// adjoint.cu — reverse pass of one step (pbf_backward): the vector-Jacobian
// product of the step with the neighbour sets and the clamp states of the
// forward held fixed.  The reference has no adjoint.
//
// Every pass is a gather over the same 27-cell windows as the forward (no
// atomics on per-particle results in the common case): a pair term that the
// forward adds to particle i's output also depends on particle j's inputs,
// and j gathers that transposed term from i when i lies in j's window too.
// Windows are centred on a particle's current cell but index the grid of the
// predicted positions, so a pair can be one-sided when a particle crossed a
// cell boundary during the step's iterations; each pair checks this
// (near_cell on the packed cells), and i scatters the terms that j cannot
// gather; they are summed exactly in any order (scatter_term, k_bwd_acc) and
// small kernels then fold them in, so the reverse pass is bitwise
// reproducible.
// Kernels:
//   W(q) = a (h^2 - q)^3,  W'(q) = -3a (h^2 - q)^2,  q = |r|^2
//   F(r) = phi(s) r,  phi = b (h - s)^2 / s,  s = |r|        (spiky gradient)
//   J(r) = dF/dr = phi I + (phi'(s) / s) r r^T,  phi' = -b (h - s)(h + s) / s^2
// Per iteration k (last to first), with X = X_k, lambda = lambda_k and the
// adjoint of X_{k+1}:
//   delta_p 1: u = X + clamp(P / pho0), X_{k+1} = box(u): the clamps pass the
//              adjoint through where inactive, the wall takes it where active;
//              Pbar = ubar masked by the MAX_DP clamp / pho0
//   delta_p 2: lambdabar_i = sum_j F.(Pbar_i - Pbar_j)
//              xbar_i += sum_j (lambda_i + lambda_j + s_ij) J (Pbar_i - Pbar_j)
//                              + ds/dr (F.(Pbar_i - Pbar_j))
//   lambda 1:  Cbar = -lambdabar / D, Sbar = -lambdabar lambda / D (D = S + eps),
//              rhobar_tot = rhobar (last iteration, from XSPH) + Cbar / pho0
//   lambda 2:  xbar_i += sum_j 2 W'(q) r (rhobar_i + rhobar_j)
//                              + J (a_ij - a_ji) / pho0,  a_ij = 2 Sbar_i (g_ij + G_i)
// XSPH (nv_i = v_i + c sum_j (v_j - v_i) w_ij, w = 2 W / (rho_i + rho_j)):
//   vbar_i = nvbar_i + c sum_j w_ij (nvbar_j - nvbar_i)
//   xbar_i += sum_j c (nvbar_i - nvbar_j).(v_j - v_i) 2 W' / (rho_i + rho_j) 2 r
//   rhobar_i = sum_j c (nvbar_i - nvbar_j).(v_j - v_i) (-2 W / (rho_i + rho_j)^2)
#include "pbf_internal.cuh"

namespace pbf {

namespace {

constexpr int kThreads = 128;
// Below this many particles a warp shares each particle (see lane_sum).
constexpr int kWarpPerParticleBelow = 131072;
// Lanes that split one particle's window in the reverse kernels of steps
// under kWarpPerParticleBelow particles: BackwardArgs::lanes (8, 16 or 32;
// pbf_tuning's bwd_lanes), 32 by default.  Few lanes suit windows of a few
// hundred candidates (less reduction per particle); many lanes suit piled-up
// states, where a handful of particles hold windows of thousands.

__device__ __forceinline__ void column_run(const SceneGeom& g, const uint32_t* __restrict__ cs,
                                           int n, int x, int y, int z, int& s, int& e) {
  const int zlo = max(z - 1, 0), zhi = min(z + 1, g.dims[2] - 1);
  const int base = g.cell_base + (x * g.dims[1] + y) * g.dims[2];
  s = (int)__ldg(cs + base + zlo);
  e = max(min((int)__ldg(cs + base + zhi + 1), n), s);
}

// f(j) for every candidate of the window of cell q, in order; with stride L,
// lane `lane` takes every L-th candidate of each run.
template <class F>
__device__ __forceinline__ void for_window(const SceneGeom& g, const uint32_t* __restrict__ cs,
                                           int n, int3 q, F&& f, int lane = 0, int stride = 1) {
  for (int dx = -1; dx <= 1; ++dx) {
    const int x = q.x + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = q.y + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      int s, e;
      column_run(g, cs, n, x, y, q.z, s, e);
      for (int j = s + lane; j < e; j += stride) f(j);
    }
  }
}

struct Vec {
  float x, y, z;
};
__device__ __forceinline__ Vec vsub(float4 a, float4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ float vdot(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ float dpoly6(const StepConsts& c, float q) {
  const float d = c.h2 - q;
  return -3.f * c.poly6_coef * d * d;
}

__device__ __forceinline__ float4 ld4(const float4* p, int i) { return __ldg(p + i); }

// Cells packed 21 bits per axis (grid dimensions are far below 2^21).
__device__ __forceinline__ unsigned long long pack_cell(int3 q) {
  return ((unsigned long long)q.x << 42) | ((unsigned long long)q.y << 21) | (unsigned long long)q.z;
}

// True when the cells differ by at most one along every axis, i.e. when a
// window centred on one contains the other.
__device__ __forceinline__ bool near_cell(unsigned long long a, unsigned long long b) {
  const int ax = (int)(a >> 42), ay = (int)((a >> 21) & 0x1FFFFF), az = (int)(a & 0x1FFFFF);
  const int bx = (int)(b >> 42), by = (int)((b >> 21) & 0x1FFFFF), bz = (int)(b & 0x1FFFFF);
  return abs(ax - bx) <= 1 && abs(ay - by) <= 1 && abs(az - bz) <= 1;
}

__device__ __forceinline__ void atomic_add3(float4* p, float x, float y, float z) {
  atomicAdd(&p->x, x);
  atomicAdd(&p->y, y);
  atomicAdd(&p->z, z);
}

// ---- exact scattered sums ------------------------------------------------------------
//
// A term that particle i cannot leave for j to gather is scattered to j.  Float
// atomics would add the terms in arrival order, so the result would change
// from run to run in its last bits; instead every term is listed (any order),
// each target keeps its term count and its largest finite |term| per component
// (integer atomics), k_bwd_acc then adds every listed term as a 64-bit integer
// scaled by 2^sh, sh = 62 - e - bits(count) with the largest |term| < 2^e (so
// no sum can overflow; integer sums do not depend on the order), and the fold
// converts back.  Each term is rounded to 2^-sh, at most 2^-62 of the target's
// largest term times its count: far below float rounding.  Non-finite terms
// are tracked per component (NaN, +inf, -inf) and give the IEEE sum's NaN or
// infinity.  Terms beyond the list's capacity go to fix / fixv with float
// atomics (results then correct but not bitwise reproducible; sc_ctr[1]
// counts them).

__device__ __forceinline__ int scale_shift(unsigned maxbits, unsigned cnt) {
  int e = 0;
  const float mx = __uint_as_float(maxbits);
  if (mx > 0.f) frexpf(mx, &e);  // mx < 2^e
  return 62 - e - (32 - __clz(cnt));
}

__device__ __forceinline__ void note_term(const BackwardArgs& a, int comp, int j, float v) {
  if (isfinite(v)) {
    if (v != 0.f) atomicMax(&a.sc_max[comp * a.sc_stride + j], __float_as_uint(fabsf(v)));
  } else {
    const unsigned bit = isnan(v) ? 1u : (v > 0.f ? 2u : 4u);
    atomicOr(&a.sc_nonfin[j], bit << (3 * comp));
  }
}

// Scatters (x, y, z, w) to target j: kind 0 (fix: position adjoints xyz and
// lambda / rho adjoint w) or kind 1 (fixv: velocity adjoints xyz).
__device__ __forceinline__ void scatter_term(const BackwardArgs& a, int kind, int j, float x, float y, float z,
                                             float w) {
  const unsigned slot = atomicAdd(&a.sc_ctr[0], 1u);
  if (slot >= (unsigned)a.sc_cap) {
    atomicAdd(&a.sc_ctr[1], 1u);
    float4* f = kind == 0 ? a.fix : a.fixv;
    atomic_add3(f + j, x, y, z);
    if (kind == 0) atomicAdd(&f[j].w, w);
    return;
  }
  a.sc_key[slot] = make_int2(j, kind);
  a.sc_val[slot] = make_float4(x, y, z, w);
  atomicAdd(&a.sc_cnt[kind * a.sc_stride + j], 1u);
  const int base = kind == 0 ? 0 : 4;
  note_term(a, base, j, x);
  note_term(a, base + 1, j, y);
  note_term(a, base + 2, j, z);
  if (kind == 0) note_term(a, 3, j, w);
}

// Adds every listed term into its target's fixed-point sums (grid-stride).
__global__ void __launch_bounds__(256) k_bwd_acc(BackwardArgs a) {
  const unsigned listed = min(a.sc_ctr[0], (unsigned)a.sc_cap);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < listed; e += gridDim.x * blockDim.x) {
    const int2 key = a.sc_key[e];
    const float4 v = a.sc_val[e];
    const int j = key.x, kind = key.y, base = kind == 0 ? 0 : 4, comps = kind == 0 ? 4 : 3;
    const unsigned cnt = a.sc_cnt[kind * a.sc_stride + j];
    const float vs[4] = {v.x, v.y, v.z, v.w};
    for (int c = 0; c < comps; ++c) {
      if (!isfinite(vs[c]) || vs[c] == 0.f) continue;
      const int comp = base + c;
      const int sh = scale_shift(a.sc_max[comp * a.sc_stride + j], cnt);
      const long long q = __double2ll_rn(ldexp((double)vs[c], sh));  // |q| < 2^62 / cnt
      atomicAdd(&a.sc_acc[comp * a.sc_stride + j], (unsigned long long)q);
    }
  }
}

// The exact sum of component `comp` of target j's listed terms, with its
// scratch set back to zero.
__device__ __forceinline__ float take_sum(const BackwardArgs& a, int comp, int j, unsigned cnt, unsigned nonfin) {
  const size_t k = (size_t)comp * a.sc_stride + j;
  const unsigned bits = (nonfin >> (3 * comp)) & 7u;
  const unsigned long long acc = a.sc_acc[k];
  const unsigned mx = a.sc_max[k];
  a.sc_acc[k] = 0ull;
  a.sc_max[k] = 0u;
  if (bits) {
    if ((bits & 1u) || (bits & 6u) == 6u) return __int_as_float(0x7fffffff);
    return (bits & 2u) ? __int_as_float(0x7f800000) : __int_as_float((int)0xff800000);
  }
  if (cnt == 0u || acc == 0ull) return 0.f;
  return (float)ldexp((double)(long long)acc, -scale_shift(mx, cnt));
}

// Target i's scattered sums of `kind` (xyz, and w for fix), its scratch
// cleared, plus what overflowed into fix / fixv (also cleared).
__device__ __forceinline__ float4 take_scattered(const BackwardArgs& a, int kind, int i) {
  const unsigned cnt = a.sc_cnt[kind * a.sc_stride + i];
  a.sc_cnt[kind * a.sc_stride + i] = 0u;
  const unsigned nonfin = a.sc_nonfin[i];
  float4* f = kind == 0 ? a.fix : a.fixv;
  const float4 o = f[i];
  f[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  const int base = kind == 0 ? 0 : 4;
  float4 s;
  s.x = take_sum(a, base, i, cnt, nonfin) + o.x;
  s.y = take_sum(a, base + 1, i, cnt, nonfin) + o.y;
  s.z = take_sum(a, base + 2, i, cnt, nonfin) + o.z;
  s.w = kind == 0 ? take_sum(a, 3, i, cnt, nonfin) + o.w : 0.f;
  return s;
}

// After a fold: the list is empty again, and each target's non-finite bits
// of the folded kind are clear.
__device__ __forceinline__ void clear_nonfin(const BackwardArgs& a, int i, unsigned mask) {
  const unsigned nf = a.sc_nonfin[i];
  if (nf & mask) a.sc_nonfin[i] = nf & ~mask;
}

// L lanes share one particle (L = 1, or BackwardArgs::lanes for small steps,
// where one thread per particle would leave most SMs idle): its lanes split
// the window and add their sums in a fixed tree, so lane 0 holds the result.
template <int L>
__device__ __forceinline__ float lane_sum(float v) {
  if constexpr (L > 1) {
    // the L lanes of one particle are an aligned group of the warp (L divides
    // 32 and the blocks hold whole warps); they return together, so only the
    // group takes part: other groups of a warp may have returned already
    const unsigned lane = threadIdx.x & 31u;
    const unsigned mask = L == 32 ? 0xffffffffu : ((1u << L) - 1u) << (lane & ~(unsigned)(L - 1));
    for (int o = L / 2; o > 0; o >>= 1) v += __shfl_down_sync(mask, v, o, L);
  }
  return v;
}

template <int L>
__device__ __forceinline__ Vec lane_sum(Vec v) {
  return {lane_sum<L>(v.x), lane_sum<L>(v.y), lane_sum<L>(v.z)};
}

// phi(s) and phi'(s) / s of the spiky gradient F = phi r (|r| = s).
__device__ __forceinline__ void spiky_parts(const StepConsts& c, float s, float& phi, float& k) {
  const float d = c.h - s;
  phi = c.spiky_coef * d * d / s;
  k = -c.spiky_coef * d * (c.h + s) / (s * s * s);
}

// J v = phi v + k r (r . v)
__device__ __forceinline__ Vec jac(float phi, float k, Vec r, Vec v) {
  const float rv = vdot(r, v);
  return {phi * v.x + k * r.x * rv, phi * v.y + k * r.y * rv, phi * v.z + k * r.z * rv};
}

// Packed cells of positions X (the grid's, or the current ones).
__global__ void __launch_bounds__(256)
k_bwd_cells(BackwardArgs a, const float4* __restrict__ X, unsigned long long* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  out[i] = pack_cell(cell_of(a.c, geom_of(a.c, a.G, i), ld4(X, i)));
}

// ---- XSPH and the velocity update --------------------------------------------------

template <int L>
__global__ void __launch_bounds__(kThreads)
k_bwd_xsph(BackwardArgs a) {
  const StepConsts& c = a.c;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / L, lane = t % L;
  if (i >= a.n) return;
  const float4 xi = ld4(a.XK, i), x0i = ld4(a.xs, i), gi = ld4(a.g_nvel, i);
  const float4 vi = make_float4((xi.x - x0i.x) * c.inv_dt, (xi.y - x0i.y) * c.inv_dt,
                                (xi.z - x0i.z) * c.inv_dt, 0.f);
  const float ri = a.rho[i];
  const unsigned long long gci = a.gcell[i];
  const SceneGeom g = geom_of(c, a.G, i);
  Vec vb = {0.f, 0.f, 0.f}, xb = {0.f, 0.f, 0.f};
  float rb = 0.f;
  for_window(g, a.cs, a.n, cell_of(c, g, xi), [&](int j) {
    if (j == i) return;
    const float4 xj = ld4(a.XK, j);
    const Vec r = vsub(xi, xj);
    const float q = vdot(r, r);
    if (!(q < c.h2)) return;
    const float4 x0j = ld4(a.xs, j);
    const Vec dv = {(xj.x - x0j.x) * c.inv_dt - vi.x, (xj.y - x0j.y) * c.inv_dt - vi.y,
                    (xj.z - x0j.z) * c.inv_dt - vi.z};
    const float den = ri + a.rho[j];
    const float W = poly6_inside(c, q);
    const float w = 2.f * W / den;
    const float dq = 2.f * dpoly6(c, q) / den * 2.f;  // d w / d x_i per unit of r
    const float dr = -2.f * W / (den * den);           // d w / d rho
    // nv_i's term c w (v_j - v_i): its adjoint on i's inputs
    const float own = c.c_xsph * (gi.x * dv.x + gi.y * dv.y + gi.z * dv.z);
    vb.x -= c.c_xsph * w * gi.x;
    vb.y -= c.c_xsph * w * gi.y;
    vb.z -= c.c_xsph * w * gi.z;
    xb.x += own * dq * r.x;
    xb.y += own * dq * r.y;
    xb.z += own * dq * r.z;
    rb += own * dr;
    if (near_cell(gci, a.kcell[j])) {
      // i is in j's window: nv_j's term c w (v_i - v_j) on i's inputs
      const float4 gj = ld4(a.g_nvel, j);
      const float tr = -c.c_xsph * (gj.x * dv.x + gj.y * dv.y + gj.z * dv.z);
      vb.x += c.c_xsph * w * gj.x;
      vb.y += c.c_xsph * w * gj.y;
      vb.z += c.c_xsph * w * gj.z;
      xb.x += tr * dq * r.x;
      xb.y += tr * dq * r.y;
      xb.z += tr * dq * r.z;
      rb += tr * dr;
    } else {
      // j cannot gather nv_i's term: scatter its adjoint on j's inputs
      scatter_term(a, 1, j, c.c_xsph * w * gi.x, c.c_xsph * w * gi.y, c.c_xsph * w * gi.z, 0.f);
      scatter_term(a, 0, j, -own * dq * r.x, -own * dq * r.y, -own * dq * r.z, own * dr);
    }
  }, lane, L);
  vb = lane_sum<L>(vb);
  xb = lane_sum<L>(xb);
  rb = lane_sum<L>(rb);
  if (lane != 0) return;
  vb = {gi.x + vb.x, gi.y + vb.y, gi.z + vb.z};  // nv_i = v_i + ...: the identity part
  // v = (X_K - X0) / dt: the position adjoint of the step's output plus XSPH's
  const float4 gp = ld4(a.g_npos, i);
  a.gx[i] = make_float4(gp.x + xb.x + vb.x * c.inv_dt, gp.y + xb.y + vb.y * c.inv_dt,
                        gp.z + xb.z + vb.z * c.inv_dt, 0.f);
  a.gx0[i] = make_float4(-vb.x * c.inv_dt, -vb.y * c.inv_dt, -vb.z * c.inv_dt, 0.f);
  a.grho[i] = rb;
}

// Folds the scattered XSPH adjoints in and clears their scratch.
__global__ void __launch_bounds__(256)
k_bwd_fix_xsph(BackwardArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) a.sc_ctr[0] = 0u;  // every listed term has been added (k_bwd_acc)
  if (i >= a.n) return;
  const float4 f = take_scattered(a, 0, i), v = take_scattered(a, 1, i);
  clear_nonfin(a, i, 0x1fffffu);
  const float4 g = a.gx[i], g0 = a.gx0[i];
  const float t = a.c.inv_dt;
  a.gx[i] = make_float4(g.x + f.x + v.x * t, g.y + f.y + v.y * t, g.z + f.z + v.z * t, 0.f);
  a.gx0[i] = make_float4(g0.x - v.x * t, g0.y - v.y * t, g0.z - v.z * t, 0.f);
  a.grho[i] += f.w;
}

// Folds scattered position adjoints into gx_next (and, with kLambda, the w
// part into lambdabar) and clears their scratch.
template <bool kLambda>
__global__ void __launch_bounds__(256)
k_bwd_fix(BackwardArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) a.sc_ctr[0] = 0u;
  if (i >= a.n) return;
  const float4 f = take_scattered(a, 0, i);
  clear_nonfin(a, i, 0xfffu);
  const float4 g = a.gx_next[i];
  a.gx_next[i] = make_float4(g.x + f.x, g.y + f.y, g.z + f.z, 0.f);
  if (kLambda) a.lbar[i] += f.w;
}

// ---- delta_p -----------------------------------------------------------------------

// Recomputes P_i (the forward's sum), applies the clamps' transposes.  Writes
// Pbar, starts the X_k adjoint with ubar, and adds this block's wall
// adjoints to wall_part[block][6] (ulim xyz, llim xyz).
template <int L>
__global__ void __launch_bounds__(kThreads)
k_bwd_dp1(BackwardArgs a, const float4* __restrict__ X, const float* __restrict__ lam) {
  const StepConsts& c = a.c;
  __shared__ float wall[6][kThreads];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / L, lane = tid % L;
  float w6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float Px = 0.f, Py = 0.f, Pz = 0.f;
  if (i < a.n) {
    const float4 xi = ld4(X, i);
    const float li = lam[i];
    const SceneGeom g = geom_of(c, a.G, i);
    for_window(g, a.cs, a.n, cell_of(c, g, xi), [&](int j) {
      const float4 xj = ld4(X, j);
      const float ex = xi.x - xj.x, ey = xi.y - xj.y, ez = xi.z - xj.z;
      const float r2 = dist2(ex, ey, ez);
      if (!(r2 >= c.h2) && !(r2 < c.keps2) && j != i) {
        const float corr = c.coef_corr * pow_corr(c, poly6_inside(c, r2));
        const float ir = rsqrtf(r2);
        const float t = c.h - r2 * ir;
        const float f = (li + __ldg(lam + j) + corr) * (c.spiky_coef * t * t * ir);
        Px = fmaf(f, ex, Px);
        Py = fmaf(f, ey, Py);
        Pz = fmaf(f, ez, Pz);
      }
    }, lane, L);
    Px = lane_sum<L>(Px);
    Py = lane_sum<L>(Py);
    Pz = lane_sum<L>(Pz);
  }
  if (i < a.n && lane == 0) {
    const float4 xi = ld4(X, i);
    const SceneGeom g = geom_of(c, a.G, i);
    const float4 gn = ld4(a.gx, i);  // adjoint of X_{k+1}
    const float P[3] = {Px, Py, Pz}, x[3] = {xi.x, xi.y, xi.z}, gin[3] = {gn.x, gn.y, gn.z};
    float ub[3], pb[3];
    for (int ax = 0; ax < 3; ++ax) {
      const float dpa = P[ax] / c.pho0;
      const float u = x[ax] + fmaxf(fminf(dpa, c.max_dp), -c.max_dp);
      ub[ax] = gin[ax];
      if (u > g.hi[ax]) {
        w6[ax] = gin[ax];
        ub[ax] = 0.f;
      } else if (u < g.lo[ax]) {
        w6[3 + ax] = gin[ax];
        ub[ax] = 0.f;
      }
      pb[ax] = (dpa < c.max_dp && dpa > -c.max_dp) ? ub[ax] / c.pho0 : 0.f;
    }
    a.pbar[i] = make_float4(pb[0], pb[1], pb[2], 0.f);
    a.gx_next[i] = make_float4(ub[0], ub[1], ub[2], 0.f);
    a.kcell[i] = pack_cell(cell_of(c, g, xi));
  }
  // this block's wall adjoints, summed in thread order
  for (int k = 0; k < 6; ++k) wall[k][threadIdx.x] = w6[k];
  __syncthreads();
  if (threadIdx.x < 6) {
    float sum = 0.f;
    for (int k = 0; k < kThreads; ++k) sum += wall[threadIdx.x][k];
    a.wall_part[blockIdx.x * 6 + threadIdx.x] = sum;
  }
}

template <int L>
__global__ void __launch_bounds__(kThreads)
k_bwd_dp2(BackwardArgs a, const float4* __restrict__ X, const float* __restrict__ lam) {
  const StepConsts& c = a.c;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / L, lane = tid % L;
  if (i >= a.n) return;
  const float4 xi = ld4(X, i), pbi4 = ld4(a.pbar, i);
  const Vec pbi = {pbi4.x, pbi4.y, pbi4.z};
  const float li = lam[i];
  const unsigned long long gci = a.gcell[i];
  const SceneGeom g = geom_of(c, a.G, i);
  Vec xb = {0.f, 0.f, 0.f};
  float lb = 0.f;
  for_window(g, a.cs, a.n, cell_of(c, g, xi), [&](int j) {
    if (j == i) return;
    const float4 xj = ld4(X, j);
    const Vec r = vsub(xi, xj);
    const float q = vdot(r, r);
    if (!(q < c.h2) || q < c.keps2) return;
    float phi, k;
    spiky_parts(c, sqrtf(q), phi, k);
    const Vec F = {phi * r.x, phi * r.y, phi * r.z};
    const float wq = poly6_inside(c, q);
    const float lsum = li + __ldg(lam + j) + c.coef_corr * pow_corr(c, wq);
    const float dsdq = c.npow == 4 ? 4.f * c.coef_corr * wq * wq * wq * dpoly6(c, q)
                                   : c.coef_corr * c.n_corr * powf(wq, c.n_corr - 1.f) * dpoly6(c, q);
    // P_i's term (lambda_i + lambda_j + s_ij) F(r_ij): its adjoint on lambda_i and x_i
    const float fi = vdot(F, pbi);
    const Vec Ji = jac(phi, k, r, pbi);
    const Vec oi = {lsum * Ji.x + 2.f * dsdq * r.x * fi, lsum * Ji.y + 2.f * dsdq * r.y * fi,
                    lsum * Ji.z + 2.f * dsdq * r.z * fi};
    lb += fi;
    xb.x += oi.x;
    xb.y += oi.y;
    xb.z += oi.z;
    if (near_cell(gci, a.kcell[j])) {
      // P_j's term on lambda_i and x_i (F and r change sign, J does not)
      const float4 pbj4 = ld4(a.pbar, j);
      const Vec pbj = {pbj4.x, pbj4.y, pbj4.z};
      const float fj = vdot(F, pbj);
      const Vec Jj = jac(phi, k, r, pbj);
      lb -= fj;
      xb.x -= lsum * Jj.x + 2.f * dsdq * r.x * fj;
      xb.y -= lsum * Jj.y + 2.f * dsdq * r.y * fj;
      xb.z -= lsum * Jj.z + 2.f * dsdq * r.z * fj;
    } else {
      // j cannot gather P_i's term: scatter its adjoint on lambda_j and x_j
      scatter_term(a, 0, j, -oi.x, -oi.y, -oi.z, fi);
    }
  }, lane, L);
  xb = lane_sum<L>(xb);
  lb = lane_sum<L>(lb);
  if (lane != 0) return;
  const float4 u = ld4(a.gx_next, i);
  a.gx_next[i] = make_float4(u.x + xb.x, u.y + xb.y, u.z + xb.z, 0.f);
  a.lbar[i] = lb;
}

// ---- lambda ------------------------------------------------------------------------

template <int L>
__global__ void __launch_bounds__(kThreads)
k_bwd_lam1(BackwardArgs a, const float4* __restrict__ X, const float* __restrict__ lam, int last) {
  const StepConsts& c = a.c;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / L, lane = tid % L;
  if (i >= a.n) return;
  const float4 xi = ld4(X, i);
  const SceneGeom g = geom_of(c, a.G, i);
  float gx = 0.f, gy = 0.f, gz = 0.f, gl2 = 0.f;
  for_window(g, a.cs, a.n, cell_of(c, g, xi), [&](int j) {
    const float4 xj = ld4(X, j);
    const float ex = xi.x - xj.x, ey = xi.y - xj.y, ez = xi.z - xj.z;
    const float r2 = dist2(ex, ey, ez);
    if (!(r2 >= c.h2) && !(r2 < c.keps2)) {
      const float ir = rsqrtf(r2);
      const float t = c.h - r2 * ir;
      const float sc = c.spiky_coef_rho0 * t * t * ir;
      gx += sc * ex;
      gy += sc * ey;
      gz += sc * ez;
      if (j != i) gl2 += dist2(sc * ex, sc * ey, sc * ez);
    }
  }, lane, L);
  gx = lane_sum<L>(gx);
  gy = lane_sum<L>(gy);
  gz = lane_sum<L>(gz);
  gl2 = lane_sum<L>(gl2);
  if (lane != 0) return;
  const float D = gl2 + dist2(gx, gy, gz) + c.lambda_eps;
  const float lb = a.lbar[i];
  const float cbar = -lb / D;
  const float sbar = -lb * lam[i] / D;
  a.gs[i] = make_float4(gx, gy, gz, sbar);
  a.rtot[i] = (last ? a.grho[i] : 0.f) + cbar / c.pho0;
}

template <int L>
__global__ void __launch_bounds__(kThreads)
k_bwd_lam2(BackwardArgs a, const float4* __restrict__ X) {
  const StepConsts& c = a.c;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tid / L, lane = tid % L;
  if (i >= a.n) return;
  const float4 xi = ld4(X, i), gsi = ld4(a.gs, i);
  const float rti = a.rtot[i];
  const unsigned long long gci = a.gcell[i];
  const SceneGeom g = geom_of(c, a.G, i);
  Vec xb = {0.f, 0.f, 0.f};
  for_window(g, a.cs, a.n, cell_of(c, g, xi), [&](int j) {
    if (j == i) return;
    const float4 xj = ld4(X, j);
    const Vec r = vsub(xi, xj);
    const float q = vdot(r, r);
    if (!(q < c.h2)) return;
    const bool recip = near_cell(gci, a.kcell[j]);
    // rho_i's term W(q): 2 W'(q) r rhobar_i on x_i; rho_j's the same with rhobar_j
    const float dw = 2.f * dpoly6(c, q);
    float wt = dw * rti;
    if (recip) wt += dw * a.rtot[j];
    xb.x += wt * r.x;
    xb.y += wt * r.y;
    xb.z += wt * r.z;
    // what j cannot gather: rho_i's (and below S_i's) terms on x_j
    float sx = recip ? 0.f : -dw * rti * r.x, sy = recip ? 0.f : -dw * rti * r.y,
          sz = recip ? 0.f : -dw * rti * r.z;
    if (!(q < c.keps2)) {
      // S_i's terms |g_ij|^2 + the g_ij part of |G_i|^2, g_ij = F / pho0:
      // a_ij = 2 Sbar_i (g_ij + G_i); J a_ij / pho0 on x_i, minus that on x_j
      float phi, k;
      spiky_parts(c, sqrtf(q), phi, k);
      const float si = gsi.w;
      const Vec ai = {2.f * si * (phi * r.x * c.inv_pho0 + gsi.x), 2.f * si * (phi * r.y * c.inv_pho0 + gsi.y),
                      2.f * si * (phi * r.z * c.inv_pho0 + gsi.z)};
      const Vec Ji = jac(phi, k, r, ai);
      xb.x += Ji.x * c.inv_pho0;
      xb.y += Ji.y * c.inv_pho0;
      xb.z += Ji.z * c.inv_pho0;
      if (recip) {
        // S_j's: a_ji = 2 Sbar_j (-g_ij + G_j); -J a_ji / pho0 on x_i
        const float4 gsj = ld4(a.gs, j);
        const float sj = gsj.w;
        const Vec aj = {2.f * sj * (-phi * r.x * c.inv_pho0 + gsj.x), 2.f * sj * (-phi * r.y * c.inv_pho0 + gsj.y),
                        2.f * sj * (-phi * r.z * c.inv_pho0 + gsj.z)};
        const Vec Jj = jac(phi, k, r, aj);
        xb.x -= Jj.x * c.inv_pho0;
        xb.y -= Jj.y * c.inv_pho0;
        xb.z -= Jj.z * c.inv_pho0;
      } else {
        sx -= Ji.x * c.inv_pho0;
        sy -= Ji.y * c.inv_pho0;
        sz -= Ji.z * c.inv_pho0;
      }
    }
    if (!recip) scatter_term(a, 0, j, sx, sy, sz, 0.f);
  }, lane, L);
  xb = lane_sum<L>(xb);
  if (lane != 0) return;
  const float4 u = ld4(a.gx_next, i);
  a.gx_next[i] = make_float4(u.x + xb.x, u.y + xb.y, u.z + xb.z, 0.f);
}

// ---- advection and the permutation ---------------------------------------------------

// x* = x + dt v + dt^2 g: adjoints of the (sorted) inputs, scattered back to
// the caller's input order through the sort permutation.
__global__ void __launch_bounds__(256)
k_bwd_out(BackwardArgs a, const uint32_t* __restrict__ perm, float4* __restrict__ g_pos,
          float4* __restrict__ g_vel) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const float4 gs = ld4(a.gx, k), g0 = ld4(a.gx0, k);
  const uint32_t p = min(perm[k], (uint32_t)(a.n - 1));
  g_pos[p] = make_float4(gs.x + g0.x, gs.y + g0.y, gs.z + g0.z, 0.f);
  g_vel[p] = make_float4(a.c.dt * gs.x, a.c.dt * gs.y, a.c.dt * gs.z, 0.f);
}

// Sums the blocks' wall adjoints into g_lim[6] (accumulating) in a fixed
// order: thread t of one block adds the parts of blocks t, t + kWallThreads,
// ... in turn, then the threads' sums are added pairwise in a fixed tree.
constexpr int kWallThreads = 256;
__global__ void __launch_bounds__(kWallThreads)
k_bwd_wall(const float* __restrict__ part, int blocks, float* __restrict__ g_lim) {
  __shared__ float s[6][kWallThreads];
  float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int b = threadIdx.x; b < blocks; b += kWallThreads)
#pragma unroll
    for (int k = 0; k < 6; ++k) acc[k] += part[b * 6 + k];
#pragma unroll
  for (int k = 0; k < 6; ++k) s[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = kWallThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int k = 0; k < 6; ++k) s[k][threadIdx.x] += s[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 6) g_lim[threadIdx.x] += s[threadIdx.x][0];
}

// ---- density grid ---------------------------------------------------------------------

struct Lattice {
  float lo[3], step[3];
  int dims[3];
  float h, h2, coef;  // poly6 radius and coefficient
};

Lattice make_lattice(const float lo[3], const float hi[3], const int dims[3], float h) {
  Lattice L;
  for (int a = 0; a < 3; ++a) {
    L.lo[a] = lo[a];
    L.dims[a] = dims[a];
    L.step[a] = (hi[a] - lo[a]) / (float)dims[a];
  }
  L.h = h;
  L.h2 = h * h;
  L.coef = (float)(315.0 / (64.0 * kRefPi * (double)h * h * h * h * h * h * h * h * h));
  return L;
}

__device__ __forceinline__ float node_coord(const Lattice& L, int a, int k) {
  return L.lo[a] + ((float)k + 0.5f) * L.step[a];
}

// One node per thread; the particles stream through shared memory in tiles
// (every node reads every particle once per tile: n is small for this loss).
constexpr int kSplatTile = 256;

__global__ void __launch_bounds__(kSplatTile)
k_density_grid(const float4* __restrict__ pos, int n, Lattice L, float* __restrict__ grid) {
  __shared__ float4 tile[kSplatTile];
  const int nodes = L.dims[0] * L.dims[1] * L.dims[2];
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int cx = c / (L.dims[1] * L.dims[2]), cy = (c / L.dims[2]) % L.dims[1], cz = c % L.dims[2];
  const float px = node_coord(L, 0, cx), py = node_coord(L, 1, cy), pz = node_coord(L, 2, cz);
  float d = 0.f;
  for (int base = 0; base < n; base += kSplatTile) {
    const int k = base + threadIdx.x;
    tile[threadIdx.x] = k < n ? pos[k] : make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f);
    __syncthreads();
    const int m = min(kSplatTile, n - base);
    for (int t = 0; t < m; ++t) {
      const float4 x = tile[t];
      const float q = dist2(x.x - px, x.y - py, x.z - pz);
      if (q < L.h2) {
        const float w = L.h2 - q;
        d += L.coef * w * w * w;
      }
    }
    __syncthreads();
  }
  if (c < nodes) grid[c] = d;
}

// Per particle: the nodes within h (a box of lattice indices around it).
__global__ void __launch_bounds__(256)
k_density_grid_backward(const float4* __restrict__ pos, int n, Lattice L,
                        const float* __restrict__ g_grid, float4* __restrict__ g_pos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 x = pos[i];
  const float p[3] = {x.x, x.y, x.z};
  int klo[3], khi[3];
  for (int a = 0; a < 3; ++a) {
    klo[a] = max((int)floorf((p[a] - L.h - L.lo[a]) / L.step[a] - 0.5f), 0);
    khi[a] = min((int)ceilf((p[a] + L.h - L.lo[a]) / L.step[a] - 0.5f), L.dims[a] - 1);
  }
  float gx = 0.f, gy = 0.f, gz = 0.f;
  for (int a = klo[0]; a <= khi[0]; ++a)
    for (int b = klo[1]; b <= khi[1]; ++b)
      for (int cz = klo[2]; cz <= khi[2]; ++cz) {
        const float rx = x.x - node_coord(L, 0, a), ry = x.y - node_coord(L, 1, b),
                    rz = x.z - node_coord(L, 2, cz);
        const float q = dist2(rx, ry, rz);
        if (!(q < L.h2)) continue;
        const float w = L.h2 - q;
        const float gq = g_grid[(a * L.dims[1] + b) * L.dims[2] + cz] * (-3.f * L.coef * w * w) * 2.f;
        gx += gq * rx;
        gy += gq * ry;
        gz += gq * rz;
      }
  g_pos[i] = make_float4(gx, gy, gz, 0.f);
}

}  // namespace

cudaError_t density_grid(const float4* pos, int n, const float lo[3], const float hi[3],
                         const int dims[3], float h, float* grid, cudaStream_t stream) {
  const Lattice L = make_lattice(lo, hi, dims, h);
  const int nodes = dims[0] * dims[1] * dims[2];
  k_density_grid<<<(nodes + kSplatTile - 1) / kSplatTile, kSplatTile, 0, stream>>>(pos, n, L, grid);
  return cudaGetLastError();
}

cudaError_t density_grid_backward(const float4* pos, int n, const float lo[3], const float hi[3],
                                  const int dims[3], float h, const float* g_grid, float4* g_pos,
                                  cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const Lattice L = make_lattice(lo, hi, dims, h);
  k_density_grid_backward<<<(n + 255) / 256, 256, 0, stream>>>(pos, n, L, g_grid, g_pos);
  return cudaGetLastError();
}

template <int L>
cudaError_t run_backward(BackwardArgs a, const BackwardTape& t, const uint32_t* perm, void* g_pos,
                         void* g_vel, float* g_lim, cudaStream_t stream) {
  const int blocks = (int)(((long long)a.n * L + kThreads - 1) / kThreads);
  const int blocks256 = (a.n + 255) / 256;
  const int acc_blocks = a.c.dense_grid;
  k_bwd_xsph<L><<<blocks, kThreads, 0, stream>>>(a);
  k_bwd_acc<<<acc_blocks, 256, 0, stream>>>(a);
  k_bwd_fix_xsph<<<blocks256, 256, 0, stream>>>(a);
  for (int k = t.niter - 1; k >= 0; --k) {
    const float4* X = t.X[k];
    const float* lam = t.lambda[k];
    k_bwd_dp1<L><<<blocks, kThreads, 0, stream>>>(a, X, lam);  // also the packed cells of X_k
    k_bwd_wall<<<1, kWallThreads, 0, stream>>>(a.wall_part, blocks, g_lim);
    k_bwd_dp2<L><<<blocks, kThreads, 0, stream>>>(a, X, lam);
    k_bwd_acc<<<acc_blocks, 256, 0, stream>>>(a);
    k_bwd_fix<true><<<blocks256, 256, 0, stream>>>(a);
    k_bwd_lam1<L><<<blocks, kThreads, 0, stream>>>(a, X, lam, k == t.niter - 1);
    k_bwd_lam2<L><<<blocks, kThreads, 0, stream>>>(a, X);
    k_bwd_acc<<<acc_blocks, 256, 0, stream>>>(a);
    k_bwd_fix<false><<<blocks256, 256, 0, stream>>>(a);
    // the adjoint of X_k becomes the input of the next (earlier) iteration
    float4* tmp = a.gx;
    a.gx = a.gx_next;
    a.gx_next = tmp;
  }
  k_bwd_out<<<(a.n + 255) / 256, 256, 0, stream>>>(a, perm, (float4*)g_pos, (float4*)g_vel);
  return cudaGetLastError();
}


cudaError_t backward(const BackwardArgs& args, const BackwardTape& t, const uint32_t* perm,
                     const void* g_npos, const void* g_nvel, void* g_pos, void* g_vel,
                     float* g_lim, cudaStream_t stream) {
  BackwardArgs a = args;
  a.g_npos = (const float4*)g_npos;
  a.g_nvel = (const float4*)g_nvel;
  cudaError_t e = cudaMemsetAsync(g_lim, 0, sizeof(float) * 6, stream);
  if (e != cudaSuccess) return e;
  a.XK = t.X[t.niter];
  a.X0 = t.X[0];
  const int blocks256 = (a.n + 255) / 256;
  k_bwd_cells<<<blocks256, 256, 0, stream>>>(a, a.X0, a.gcell);
  k_bwd_cells<<<blocks256, 256, 0, stream>>>(a, a.XK, a.kcell);
  if (a.n < kWarpPerParticleBelow) {
    if (a.lanes == 8) return run_backward<8>(a, t, perm, g_pos, g_vel, g_lim, stream);
    if (a.lanes == 16) return run_backward<16>(a, t, perm, g_pos, g_vel, g_lim, stream);
    return run_backward<32>(a, t, perm, g_pos, g_vel, g_lim, stream);
  }
  return run_backward<1>(a, t, perm, g_pos, g_vel, g_lim, stream);
}

}  // namespace pbf
