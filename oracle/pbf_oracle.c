/*
 * pbf_oracle.c — CPU restatement of naeioi/PBF-CUDA's Simulator::step.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference leg load this library: as the checker
 * the CUDA path is compared against, or as the timed CPU baseline.  The CUDA
 * product path never links, loads or falls back to it.
 *
 * The same source is compiled twice (oracle/build_oracle.py):
 *   ORACLE_F64 defined -> oracle_*_f64: every continuous quantity in double.
 *                         This is the FP64 oracle.
 *   otherwise          -> oracle_*_f32: float arithmetic in the order of the
 *                         reference's kernels, parallel over particles with
 *                         OpenMP.  This is the CPU port of the reference (it
 *                         has no CPU path of its own) and the timed CPU baseline.
 * Both are compiled with -ffp-contract=off, so the only fused multiply-adds are
 * the explicit fma() calls of the advection step.  Those reproduce the fused
 * multiply-adds nvcc emits for the reference's advect_kernel, which makes the
 * predicted positions, and so the cell ids, bit-identical to the GPU's.
 *
 * Parity pinning: the reference ships no tests or fixtures and has no CPU
 * path, so this restatement is pinned against outputs of the reference's own
 * kernels (fluids/Simulator.cu, fluids/Simulator_kernel.cuh compiled
 * unmodified for sm_103a and run on a GB300 by oracle/ref_harness), recorded
 * in tests/golden/ by tests/golden/make_golden.py: cell ids, order and ranges
 * bit-exact, positions within 1e-7 (tests/test_golden.py).
 *
 * Layout: all particle arrays are stride-4 (x, y, z, w) in the oracle's real
 * type; iid is uint32.  The step permutes pos/vel/iid in place exactly like
 * the reference's thrust::sort_by_key over zip(pos, vel, npos, nvel, iid).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/pbf.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORACLE_F64
typedef double real;
#define SFX(name) name##_f64
#define RSQRT(x) sqrt(x)
#define RFMA(a, b, c) fma((a), (b), (c))
#define RMIN(a, b) fmin((a), (b))
#define RMAX(a, b) fmax((a), (b))
#define RPOW(a, b) pow((a), (b))
#else
typedef float real;
#define SFX(name) name##_f32
#define RSQRT(x) sqrtf(x)
#define RFMA(a, b, c) fmaf((a), (b), (c))
#define RMIN(a, b) fminf((a), (b))
#define RMAX(a, b) fmaxf((a), (b))
#define RPOW(a, b) powf((a), (b))
#endif

/* fluids/helper.h:4 — the reference's truncated pi. */
#define REF_PI 3.14159265359

typedef struct {
  int dims[3];
  int cells;
} grid_dims;

/* Solver constants, restating the host-side set-up of the reference. */
typedef struct {
  real h, h2;
  real poly6_coef;  /* getPoly6 ctor, fluids/Simulator.cu:77-83 */
  real spiky_coef;  /* getSpikyGrad ctor, fluids/Simulator.cu:94-98 */
  real coef_corr;   /* fluids/Simulator.cu:235 */
  real inv_dt;      /* h_updateVelocity ctor, fluids/Simulator.cu:129 */
  real g[3];
  real lo[3], hi[3]; /* wall clamp bounds, fluids/Simulator_kernel.cuh:190-192 */
  double kernel_eps; /* compared in double, as KERNAL_EPS (fluids/helper.h:7) */
  real max_dp;
  float llim[3], ulim[3];
  grid_dims gd;
} consts;

/* float -> int conversion with round-toward-zero that saturates and maps NaN
 * to 0, as the GPU's cvt.rzi.s32 does for the reference's (int) casts. */
static int f2i_rz(double v) {
  if (v != v) return 0;
  if (v >= 2147483647.0) return 2147483647;
  if (v <= -2147483648.0) return (-2147483647 - 1);
  return (int)v;
}

/* A float parameter as the double it was typed as: the shortest decimal that
 * rounds to it.  The reference's LIM_EPS is the double literal 1e-3
 * (fluids/helper.h:5); the float field 1e-3f promotes back to exactly 1e-3. */
static double promote_decimal(float f) {
  char buf[32];
  for (int prec = 1; prec <= 9; ++prec) {
    snprintf(buf, sizeof(buf), "%.*g", prec, (double)f);
    double d = strtod(buf, NULL);
    if ((float)d == f) return d;
  }
  return (double)f;
}

/* fluids/Simulator.cu:187-188: dims = ceil((ulim - llim) / h), in float. */
static grid_dims make_dims(const float ulim[3], const float llim[3], float h) {
  grid_dims g;
  for (int a = 0; a < 3; ++a) {
    float diff = ulim[a] - llim[a];
    g.dims[a] = f2i_rz((double)ceilf(diff / h));
    if (g.dims[a] < 1) g.dims[a] = 1;
  }
  g.cells = g.dims[0] * g.dims[1] * g.dims[2];
  return g;
}

/* getPoly6::operator(), fluids/Simulator.cu:84-89. */
static inline real poly6(const consts* c, real r2) {
  if (r2 >= c->h2) return 0;
  real d = c->h2 - r2;
  return c->poly6_coef * d * d * d;
}

/* getSpikyGrad::operator(), fluids/Simulator.cu:100-106: out = grad W(r). */
static inline void spiky(const consts* c, const real r[3], real out[3]) {
  real rlen = RSQRT(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  if (rlen >= c->h || (double)rlen < c->kernel_eps) {
    out[0] = out[1] = out[2] = 0;
    return;
  }
  real d = c->h - rlen;
  real s = c->spiky_coef * d * d / rlen;
  out[0] = s * r[0];
  out[1] = s * r[1];
  out[2] = s * r[2];
}

/* DensityBoundary::densityAt, fluids/Simulator.cu:144-149 (double constant,
 * float return). */
static inline real density_at(real d, real h) {
  if (d > h) return 0;
  if (d <= 0) return (real)(2 * REF_PI / 3);
  return (real)((2 * REF_PI / 3) * (h - d) * (h - d) * (h + d));
}

/* DensityBoundary::operator(), fluids/Simulator.cu:151-160. */
static inline real boundary_density(const consts* c, const real p[3]) {
  real up[3], lo[3];
  for (int a = 0; a < 3; ++a) {
    up[a] = (real)c->ulim[a];
    lo[a] = (real)c->llim[a];
  }
  return density_at(up[0] - p[0], c->h) + density_at(p[0] - lo[0], c->h) +
         density_at(up[1] - p[1], c->h) + density_at(p[1] - lo[1], c->h) +
         density_at(up[2] - p[2], c->h) + density_at(p[2] - lo[2], c->h);
}

/* getGridxyz::operator(), fluids/Simulator.cu:30-36 (also getGridId :65-71). */
static inline void cell_xyz(const consts* c, const real* p, int out[3]) {
  for (int a = 0; a < 3; ++a) {
    real diff = p[a] - (real)c->llim[a];
    int v = f2i_rz((double)(diff / c->h));
    if (v < 0) v = 0;
    if (v > c->gd.dims[a] - 1) v = c->gd.dims[a] - 1;
    out[a] = v;
  }
}

/* xyzToId::operator(), fluids/Simulator.cu:44-53. */
static inline int cell_id(const consts* c, const int xyz[3]) {
  return xyz[0] * c->gd.dims[1] * c->gd.dims[2] + xyz[1] * c->gd.dims[2] + xyz[2];
}

static void make_consts(consts* c, const pbf_params* p, const float ulim[3],
                        const float llim[3]) {
  memcpy(c->ulim, ulim, sizeof(float) * 3);
  memcpy(c->llim, llim, sizeof(float) * 3);
  c->gd = make_dims(ulim, llim, p->h);
#ifdef ORACLE_F64
  double h = p->h;
  c->h = h;
  c->h2 = h * h;
  c->poly6_coef = 315.0 / (64.0 * REF_PI * pow(h, 9));
  c->spiky_coef = -45.0 / (REF_PI * pow(h, 6));
  {
    double dq2 = (double)p->delta_q * (double)p->delta_q;
    double w = dq2 >= c->h2 ? 0.0 : c->poly6_coef * pow(c->h2 - dq2, 3);
    c->coef_corr = -(double)p->k_corr / pow(w, (double)p->n_corr);
  }
  c->inv_dt = 1.0 / (double)p->dt;
  for (int a = 0; a < 3; ++a) {
    c->lo[a] = (double)llim[a] + promote_decimal(p->lim_eps);
    c->hi[a] = (double)ulim[a] - promote_decimal(p->lim_eps);
  }
#else
  float h = p->h;
  c->h = h;
  c->h2 = h * h;
  {
    float ih = 1.f / h;
    float ih3 = ih * ih * ih;
    float ih9 = ih3 * ih3 * ih3;
    c->poly6_coef = (float)((double)(315.f * ih9) / (64.0 * REF_PI));
  }
  {
    float h6 = h * h;
    h6 = h6 * h6 * h6;
    c->spiky_coef = (float)(-45.0 / (REF_PI * (double)h6));
  }
  c->coef_corr = -p->k_corr / powf(poly6(c, p->delta_q * p->delta_q), p->n_corr);
  c->inv_dt = 1.f / p->dt;
  for (int a = 0; a < 3; ++a) {
    c->lo[a] = (float)((double)llim[a] + promote_decimal(p->lim_eps));
    c->hi[a] = (float)((double)ulim[a] - promote_decimal(p->lim_eps));
  }
#endif
  for (int a = 0; a < 3; ++a) c->g[a] = -(real)p->g * (real)p->up[a];
  c->kernel_eps = promote_decimal(p->kernel_eps);
  c->max_dp = (real)p->max_dp;
}

/*
 * Cell ids, stable order and ranges (fluids/Simulator.cu:178-204 with
 * computeGridRange, fluids/Simulator_kernel.cuh:21-50).  The stable sort is a
 * counting sort by cell id; start/end use the reference's 0/0 for empty cells.
 * keys[n] input order; perm[n] input index of each sorted slot; start/end
 * hold gd.cells entries and may be NULL.
 */
static void build_grid(const consts* c, const real* xstar, int n, uint32_t* keys, uint32_t* perm,
                       uint32_t* start, uint32_t* end) {
  int cells = c->gd.cells;
  uint32_t* cnt = (uint32_t*)calloc((size_t)cells + 1, sizeof(uint32_t));
  for (int i = 0; i < n; ++i) {
    int xyz[3];
    cell_xyz(c, xstar + 4 * (size_t)i, xyz);
    keys[i] = (uint32_t)cell_id(c, xyz);
    cnt[keys[i] + 1]++;
  }
  for (int k = 0; k < cells; ++k) cnt[k + 1] += cnt[k];
  if (start && end) {
    for (int k = 0; k < cells; ++k) {
      if (cnt[k + 1] > cnt[k]) {
        start[k] = cnt[k];
        end[k] = cnt[k + 1];
      } else {
        start[k] = end[k] = 0;
      }
    }
  }
  {
    uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)cells + 1));
    memcpy(fill, cnt, sizeof(uint32_t) * ((size_t)cells + 1));
    for (int i = 0; i < n; ++i) perm[fill[keys[i]]++] = (uint32_t)i;
    free(fill);
  }
  free(cnt);
}

int SFX(oracle_grid)(const pbf_params* p, const float ulim[3], const float llim[3],
                     const real* xstar, int n, uint32_t* keys, uint32_t* perm, uint32_t* start,
                     uint32_t* end, int dims[3]) {
  consts c;
  make_consts(&c, p, ulim, llim);
  if (dims) memcpy(dims, c.gd.dims, sizeof(int) * 3);
  if (n < 0) return 1;
  if (n == 0) {
    if (start && end)
      for (int k = 0; k < c.gd.cells; ++k) start[k] = end[k] = 0;
    return 0;
  }
  build_grid(&c, xstar, n, keys, perm, start, end);
  return 0;
}

/* advect_kernel's predicted positions only (fluids/Simulator_kernel.cuh:14-15). */
int SFX(oracle_predict)(const pbf_params* p, const real* pos, const real* vel, int n, real* xstar) {
  if (!p || n < 0) return 1;
  consts c;
  float z[3] = {0, 0, 0};
  make_consts(&c, p, z, z);
  const real dt = (real)p->dt;
  for (int i = 0; i < n; ++i) {
    for (int a = 0; a < 3; ++a) {
      real v = RFMA(dt, c.g[a], vel[4 * (size_t)i + a]);
      xstar[4 * (size_t)i + a] = RFMA(dt, v, pos[4 * (size_t)i + a]);
    }
    xstar[4 * (size_t)i + 3] = pos[4 * (size_t)i + 3];
  }
  return 0;
}

/* Sorted index range of the three z-consecutive cells (x, y, zlo..zhi): with
 * the reference's loop order (dz innermost, fluids/Simulator_kernel.cuh:78-88)
 * these cells are visited in a row, so their particles form one run. */
static inline void column_run(const consts* c, const uint32_t* cs, int x, int y, int z, int* s,
                              int* e) {
  int zlo = z > 0 ? z - 1 : 0;
  int zhi = z + 1 < c->gd.dims[2] ? z + 1 : c->gd.dims[2] - 1;
  int base = (x * c->gd.dims[1] + y) * c->gd.dims[2];
  *s = (int)cs[base + zlo];
  *e = (int)cs[base + zhi + 1];
}

/* computeLambda, fluids/Simulator_kernel.cuh:52-129.  cs = exclusive prefix
 * of cell counts (cells + 1 entries): cell k holds sorted slots [cs[k], cs[k+1]). */
static void lambda_pass(const consts* c, const pbf_params* p, const real* X, const uint32_t* cs,
                        int n, real* lambda, real* rho) {
  const real pho0 = (real)p->pho0;
  const real eps = (real)p->lambda_eps;
  const real kb = (real)p->k_boundaryDensity;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const real* xi = X + 4 * (size_t)i;
    int ind[3];
    cell_xyz(c, xi, ind);
    real pho = 0, gradj_l2 = 0;
    real gi[3] = {0, 0, 0};
    for (int dx = -1; dx <= 1; ++dx) {
      int x = ind[0] + dx;
      if (x < 0 || x >= c->gd.dims[0]) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        int y = ind[1] + dy;
        if (y < 0 || y >= c->gd.dims[1]) continue;
        int s, e;
        column_run(c, cs, x, y, ind[2], &s, &e);
        for (int j = s; j < e; ++j) {
          const real* xj = X + 4 * (size_t)j;
          real d[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
          real r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
          pho += poly6(c, r2);
          real g[3];
          spiky(c, d, g);
          g[0] /= pho0;
          g[1] /= pho0;
          g[2] /= pho0;
          gi[0] += g[0];
          gi[1] += g[1];
          gi[2] += g[2];
          if (j != i) gradj_l2 += g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
        }
      }
    }
    pho += kb * boundary_density(c, xi);
    real grad_l2 = gradj_l2 + gi[0] * gi[0] + gi[1] * gi[1] + gi[2] * gi[2];
    lambda[i] = -(pho / pho0 - 1) / (grad_l2 + eps);
    rho[i] = pho;
  }
}

/* computetpos, fluids/Simulator_kernel.cuh:131-194 (s_corr with powf). */
static void dp_pass(const consts* c, const pbf_params* p, const real* X, const uint32_t* cs,
                    int n, const real* lambda, real* T) {
  const real pho0 = (real)p->pho0;
  const real n_corr = (real)p->n_corr;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const real* xi = X + 4 * (size_t)i;
    int ind[3];
    cell_xyz(c, xi, ind);
    real li = lambda[i];
    real d[3] = {0, 0, 0};
    for (int dx = -1; dx <= 1; ++dx) {
      int x = ind[0] + dx;
      if (x < 0 || x >= c->gd.dims[0]) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        int y = ind[1] + dy;
        if (y < 0 || y >= c->gd.dims[1]) continue;
        int s, e;
        column_run(c, cs, x, y, ind[2], &s, &e);
        for (int j = s; j < e; ++j) {
          if (j == i) continue;
          const real* xj = X + 4 * (size_t)j;
          real r[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
          real corr = c->coef_corr * RPOW(poly6(c, r[0] * r[0] + r[1] * r[1] + r[2] * r[2]), n_corr);
          real g[3];
          spiky(c, r, g);
          real f = li + lambda[j] + corr;
          d[0] += f * g[0];
          d[1] += f * g[1];
          d[2] += f * g[2];
        }
      }
    }
    real* ti = T + 4 * (size_t)i;
    for (int a = 0; a < 3; ++a) {
      real v = d[a] / pho0;
      v = RMAX(RMIN(v, c->max_dp), -c->max_dp);
      v = xi[a] + v;
      ti[a] = RMAX(RMIN(v, c->hi[a]), c->lo[a]);
    }
    ti[3] = xi[3];
  }
}

/* computeXSPH, fluids/Simulator_kernel.cuh:196-239. */
static void xsph_pass(const consts* c, const pbf_params* p, const real* X, const real* V,
                      const real* rho, const uint32_t* cs, int n, real* NV) {
  const real cx = (real)p->c_XSPH;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    const real* xi = X + 4 * (size_t)i;
    const real* vi = V + 4 * (size_t)i;
    real ci = rho[i];
    int ind[3];
    cell_xyz(c, xi, ind);
    real av[3] = {0, 0, 0};
    for (int dx = -1; dx <= 1; ++dx) {
      int x = ind[0] + dx;
      if (x < 0 || x >= c->gd.dims[0]) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        int y = ind[1] + dy;
        if (y < 0 || y >= c->gd.dims[1]) continue;
        int s, e;
        column_run(c, cs, x, y, ind[2], &s, &e);
        for (int j = s; j < e; ++j) {
          const real* xj = X + 4 * (size_t)j;
          const real* vj = V + 4 * (size_t)j;
          real dp[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
          real w = poly6(c, dp[0] * dp[0] + dp[1] * dp[1] + dp[2] * dp[2]);
          real den = ci + rho[j];
          for (int a = 0; a < 3; ++a) av[a] += (real)2 * (vj[a] - vi[a]) * w / den;
        }
      }
    }
    real* o = NV + 4 * (size_t)i;
    for (int a = 0; a < 3; ++a) o[a] = vi[a] + cx * av[a];
  }
}

/* Vorticity confinement (no counterpart in the reference; Macklin and
 * Mueller 2013, eqs. 15-16) after XSPH, on its output U (positions X):
 * omega_i = sum_{j != i} (u_j - u_i) x g_ij, eta_i = sum_{j != i} |omega_j| g_ij
 * with g_ij = spiky(x_i - x_j) over the same windows, then
 * u_i += dt eps (eta_i / |eta_i|) x omega_i. */
static void vorticity_pass(const consts* c, const pbf_params* p, const real* X, const uint32_t* cs, int n,
                           real* U) {
  real* W = (real*)malloc(sizeof(real) * 4 * (size_t)(n > 0 ? n : 1));
  for (int pass = 0; pass < 2; ++pass) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      const real* xi = X + 4 * (size_t)i;
      const real* ui = U + 4 * (size_t)i;
      int ind[3];
      cell_xyz(c, xi, ind);
      real acc[3] = {0, 0, 0};
      for (int dx = -1; dx <= 1; ++dx) {
        int x = ind[0] + dx;
        if (x < 0 || x >= c->gd.dims[0]) continue;
        for (int dy = -1; dy <= 1; ++dy) {
          int y = ind[1] + dy;
          if (y < 0 || y >= c->gd.dims[1]) continue;
          int s, e;
          column_run(c, cs, x, y, ind[2], &s, &e);
          for (int j = s; j < e; ++j) {
            if (j == i) continue;
            const real* xj = X + 4 * (size_t)j;
            real r[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
            real g[3];
            spiky(c, r, g);
            if (pass == 0) {
              const real* uj = U + 4 * (size_t)j;
              real d[3] = {uj[0] - ui[0], uj[1] - ui[1], uj[2] - ui[2]};
              acc[0] += d[1] * g[2] - d[2] * g[1];
              acc[1] += d[2] * g[0] - d[0] * g[2];
              acc[2] += d[0] * g[1] - d[1] * g[0];
            } else {
              const real m = W[4 * (size_t)j + 3];
              for (int a = 0; a < 3; ++a) acc[a] += m * g[a];
            }
          }
        }
      }
      if (pass == 0) {
        real* w = W + 4 * (size_t)i;
        w[0] = acc[0], w[1] = acc[1], w[2] = acc[2];
        w[3] = RSQRT(acc[0] * acc[0] + acc[1] * acc[1] + acc[2] * acc[2]);
      } else {
        real len = RSQRT(acc[0] * acc[0] + acc[1] * acc[1] + acc[2] * acc[2]);
        if (!(len > 0) || !isfinite(len)) continue;
        const real* w = W + 4 * (size_t)i;
        real nx = acc[0] / len, ny = acc[1] / len, nz = acc[2] / len;
        real sc = (real)p->dt * (real)p->vorticity_eps;
        real* u = U + 4 * (size_t)i;
        u[0] += sc * (ny * w[2] - nz * w[1]);
        u[1] += sc * (nz * w[0] - nx * w[2]);
        u[2] += sc * (nx * w[1] - ny * w[0]);
      }
    }
  }
  free(W);
}

/*
 * One Simulator::step (fluids/Simulator.cpp:10-99) on host arrays, with the
 * same in/out contract as the GPU entry point pbf_step.  rho_out/lambda_out
 * (optional, n entries, cell order) receive the last lambda pass.
 * Returns 0 on success, nonzero on bad arguments.
 */
int SFX(oracle_step)(const pbf_params* p, const float ulim[3], const float llim[3], real* pos,
                     real* npos, real* vel, real* nvel, uint32_t* iid, int n, real* rho_out,
                     real* lambda_out) {
  if (!p || n < 0 || p->niter < 1) return 1;
  if (n == 0) return 0;
  consts c;
  make_consts(&c, p, ulim, llim);
  size_t n4 = 4 * (size_t)n;
  real* X = (real*)malloc(sizeof(real) * n4);    /* x, sorted */
  real* V = (real*)malloc(sizeof(real) * n4);    /* v after gravity, sorted */
  real* A = (real*)malloc(sizeof(real) * n4);    /* npos ping */
  real* B = (real*)malloc(sizeof(real) * n4);    /* tpos pong */
  real* S = (real*)malloc(sizeof(real) * n4);    /* predicted, input order */
  real* lam = (real*)malloc(sizeof(real) * (size_t)n);
  real* rho = (real*)malloc(sizeof(real) * (size_t)n);
  uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t* perm = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t* cs = (uint32_t*)calloc((size_t)c.gd.cells + 1, sizeof(uint32_t));

  /* advect_kernel, fluids/Simulator_kernel.cuh:7-19: v += dt g; x* = x + dt v. */
  const real dt = (real)p->dt;
  for (int i = 0; i < n; ++i) {
    real* v = vel + 4 * (size_t)i;
    real* x = pos + 4 * (size_t)i;
    real* s = S + 4 * (size_t)i;
    for (int a = 0; a < 3; ++a) {
      v[a] = RFMA(dt, c.g[a], v[a]);
      s[a] = RFMA(dt, v[a], x[a]);
    }
    s[3] = x[3];
  }
  /* buildGridHash: ids, stable sort of zip(pos, vel, npos, nvel, iid), ranges. */
  build_grid(&c, S, n, keys, perm, NULL, NULL);
  for (int i = 0; i < n; ++i) cs[keys[i] + 1]++;
  for (int k = 0; k < c.gd.cells; ++k) cs[k + 1] += cs[k];
  for (int k = 0; k < n; ++k) {
    uint32_t q = perm[k];
    memcpy(X + 4 * (size_t)k, pos + 4 * (size_t)q, sizeof(real) * 4);
    memcpy(V + 4 * (size_t)k, vel + 4 * (size_t)q, sizeof(real) * 4);
    memcpy(A + 4 * (size_t)k, S + 4 * (size_t)q, sizeof(real) * 4);
    ids[k] = iid[q];
  }
  /* correctDensity x niter (fluids/Simulator.cu:213-249): Jacobi update. */
  for (int it = 0; it < p->niter; ++it) {
    lambda_pass(&c, p, A, cs, n, lam, rho);
    dp_pass(&c, p, A, cs, n, lam, B);
    real* t = A;
    A = B;
    B = t;
  }
  /* updateVelocity (fluids/Simulator.cu:267-273): v = (x* - x) * (1/dt). */
  for (int k = 0; k < n; ++k) {
    for (int a = 0; a < 3; ++a) V[4 * (size_t)k + a] = (A[4 * (size_t)k + a] - X[4 * (size_t)k + a]) * c.inv_dt;
  }
  /* correctVelocity: XSPH with rho of the last lambda pass. */
  xsph_pass(&c, p, A, V, rho, cs, n, B);
  if (p->vorticity_eps > 0) vorticity_pass(&c, p, A, cs, n, B);

  for (int k = 0; k < n; ++k) {
    size_t o = 4 * (size_t)k;
    pos[o] = X[o];
    pos[o + 1] = X[o + 1];
    pos[o + 2] = X[o + 2];
    pos[o + 3] = X[o + 3];
    npos[o] = A[o];
    npos[o + 1] = A[o + 1];
    npos[o + 2] = A[o + 2];
    npos[o + 3] = X[o + 3];
    vel[o] = V[o];
    vel[o + 1] = V[o + 1];
    vel[o + 2] = V[o + 2];
    nvel[o] = B[o];
    nvel[o + 1] = B[o + 1];
    nvel[o + 2] = B[o + 2];
    nvel[o + 3] = 0;
    vel[o + 3] = 0;
    iid[k] = ids[k];
    if (rho_out) rho_out[k] = rho[k];
    if (lambda_out) lambda_out[k] = lam[k];
  }
  free(X);
  free(V);
  free(A);
  free(B);
  free(S);
  free(lam);
  free(rho);
  free(keys);
  free(perm);
  free(ids);
  free(cs);
  return 0;
}

/* Number of OpenMP threads the parallel passes use (1 without OpenMP). */
int SFX(oracle_threads)(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ---- reverse pass of one step (adjoint) ------------------------------------------
 *
 * The reference has no adjoint; this is the exact transpose of the step above
 * with the neighbour sets (windows, r < h, |r| >= KERNAL_EPS) and the clamp
 * states held fixed, written as a scatter over the forward's own pairs.
 * Kernels: W(q) = a (h^2 - q)^3, W'(q) = -3a (h^2 - q)^2 (q = |r|^2);
 * spiky F(r) = phi(s) r with phi = b (h - s)^2 / s, s = |r|, whose Jacobian
 * is J(r) = phi I + (phi'(s) / s) r r^T, phi' = -b (h - s)(h + s) / s^2.
 * Not supported with k_boundaryDensity != 0 (returns 2).
 */

typedef struct {
  real J[6]; /* symmetric 3x3: xx, yy, zz, xy, xz, yz */
} sym3;

static inline void spiky_jac(const consts* c, const real r[3], real s, sym3* out) {
  real d = c->h - s;
  real phi = c->spiky_coef * d * d / s;
  real dphi = -c->spiky_coef * d * (c->h + s) / (s * s);
  real k = dphi / s;
  out->J[0] = phi + k * r[0] * r[0];
  out->J[1] = phi + k * r[1] * r[1];
  out->J[2] = phi + k * r[2] * r[2];
  out->J[3] = k * r[0] * r[1];
  out->J[4] = k * r[0] * r[2];
  out->J[5] = k * r[1] * r[2];
}

static inline void sym3_mul(const sym3* m, const real v[3], real out[3]) {
  out[0] = m->J[0] * v[0] + m->J[3] * v[1] + m->J[4] * v[2];
  out[1] = m->J[3] * v[0] + m->J[1] * v[1] + m->J[5] * v[2];
  out[2] = m->J[4] * v[0] + m->J[5] * v[1] + m->J[2] * v[2];
}

static inline real dpoly6(const consts* c, real q) { /* dW/dq inside the support */
  real d = c->h2 - q;
  return -3 * c->poly6_coef * d * d;
}

/* Visit the window pairs (i, j) of slot i at positions P (cell of P[i]). */
#define FOR_WINDOW(c, cs, P, i, j)                                      \
  for (int dx_ = -1, ind_[3] = {0, 0, 0}; dx_ <= 1; ++dx_)              \
    if (dx_ == -1 ? (cell_xyz((c), (P) + 4 * (size_t)(i), ind_), 1) : 1) \
      for (int dy_ = -1; dy_ <= 1; ++dy_)                               \
        for (int s_ = 0, e_ = 0, ok_ = ((ind_[0] + dx_) >= 0 && (ind_[0] + dx_) < (c)->gd.dims[0] && \
                                        (ind_[1] + dy_) >= 0 && (ind_[1] + dy_) < (c)->gd.dims[1]) \
                                           ? (column_run((c), (cs), ind_[0] + dx_, ind_[1] + dy_, ind_[2], &s_, &e_), 1) \
                                           : 0;                         \
             ok_; ok_ = 0)                                              \
          for (int j = s_; j < e_; ++j)

int SFX(oracle_step_backward)(const pbf_params* p, const float ulim[3], const float llim[3],
                              const real* pos_in, const real* vel_in, const uint32_t* iid_in, int n,
                              const real* g_npos, const real* g_nvel, real* g_pos, real* g_vel,
                              real* g_ulim, real* g_llim) {
  if (!p || n < 0 || p->niter < 1) return 1;
  if (p->k_boundaryDensity != 0.f) return 2;
  for (int a = 0; a < 3; ++a) g_ulim[a] = g_llim[a] = 0;
  if (n == 0) return 0;
  (void)iid_in;
  consts c;
  make_consts(&c, p, ulim, llim);
  const int K = p->niter;
  const size_t n4 = 4 * (size_t)n;
  const real dt = (real)p->dt, pho0 = (real)p->pho0, eps = (real)p->lambda_eps;
  const real n_corr = (real)p->n_corr, cx = (real)p->c_XSPH;
  real* S = (real*)malloc(sizeof(real) * n4);
  real* X0 = (real*)malloc(sizeof(real) * n4); /* sorted input positions */
  real* XK = (real*)malloc(sizeof(real) * n4 * (size_t)(K + 1)); /* X_0 .. X_K */
  real* LAM = (real*)malloc(sizeof(real) * (size_t)n * (size_t)K);
  real* RHO = (real*)malloc(sizeof(real) * (size_t)n * (size_t)K);
  real* V = (real*)malloc(sizeof(real) * n4);
  real* gX = (real*)calloc(n4, sizeof(real));    /* adjoint of the current X_k */
  real* gXn = (real*)calloc(n4, sizeof(real));   /* adjoint of X_{k+1} */
  real* gX0 = (real*)calloc(n4, sizeof(real));   /* adjoint of the sorted input positions */
  real* gV = (real*)calloc(n4, sizeof(real));
  real* gl = (real*)calloc((size_t)n, sizeof(real));
  real* gr = (real*)calloc((size_t)n, sizeof(real));
  real* Pb = (real*)calloc(n4, sizeof(real));
  real* G = (real*)calloc(n4, sizeof(real));
  real* Sbar = (real*)calloc((size_t)n, sizeof(real));
  real* Rtot = (real*)calloc((size_t)n, sizeof(real));
  uint32_t* keys = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t* perm = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)n);
  uint32_t* cs = (uint32_t*)calloc((size_t)c.gd.cells + 1, sizeof(uint32_t));

  /* ---- forward, recorded ---- */
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      real v = RFMA(dt, c.g[a], vel_in[4 * (size_t)i + a]);
      S[4 * (size_t)i + a] = RFMA(dt, v, pos_in[4 * (size_t)i + a]);
    }
  build_grid(&c, S, n, keys, perm, NULL, NULL);
  for (int i = 0; i < n; ++i) cs[keys[i] + 1]++;
  for (int k = 0; k < c.gd.cells; ++k) cs[k + 1] += cs[k];
  for (int k = 0; k < n; ++k) {
    memcpy(X0 + 4 * (size_t)k, pos_in + 4 * (size_t)perm[k], sizeof(real) * 4);
    memcpy(XK + 4 * (size_t)k, S + 4 * (size_t)perm[k], sizeof(real) * 4);
  }
  for (int k = 0; k < K; ++k) {
    lambda_pass(&c, p, XK + n4 * k, cs, n, LAM + (size_t)n * k, RHO + (size_t)n * k);
    dp_pass(&c, p, XK + n4 * k, cs, n, LAM + (size_t)n * k, XK + n4 * (k + 1));
  }
  const real* XF = XK + n4 * K;
  const real* rho = RHO + (size_t)n * (K - 1);
  for (int k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) V[4 * (size_t)k + a] = (XF[4 * (size_t)k + a] - X0[4 * (size_t)k + a]) * c.inv_dt;

  /* ---- XSPH: nv_i = v_i + c sum_j (v_j - v_i) w_ij, w = 2 W(q) / (rho_i + rho_j) ---- */
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      gV[4 * (size_t)i + a] += g_nvel[4 * (size_t)i + a];
      gXn[4 * (size_t)i + a] = g_npos[4 * (size_t)i + a];
    }
  for (int i = 0; i < n; ++i) {
    const real* xi = XF + 4 * (size_t)i;
    const real* vi = V + 4 * (size_t)i;
    const real* gn = g_nvel + 4 * (size_t)i;
    FOR_WINDOW(&c, cs, XF, i, j) {
      if (j == i) continue;
      const real* xj = XF + 4 * (size_t)j;
      const real* vj = V + 4 * (size_t)j;
      real r[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
      real q = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
      if (q >= c.h2) continue;
      real den = rho[i] + rho[j];
      real w = 2 * poly6(&c, q) / den;
      real wb = 0;
      for (int a = 0; a < 3; ++a) {
        gV[4 * (size_t)i + a] -= cx * w * gn[a];
        gV[4 * (size_t)j + a] += cx * w * gn[a];
        wb += cx * gn[a] * (vj[a] - vi[a]);
      }
      real gq = wb * 2 * dpoly6(&c, q) / den;
      for (int a = 0; a < 3; ++a) {
        gXn[4 * (size_t)i + a] += gq * 2 * r[a];
        gXn[4 * (size_t)j + a] -= gq * 2 * r[a];
      }
      real grho = wb * (-2 * poly6(&c, q) / (den * den));
      gr[i] += grho;
      gr[j] += grho;
    }
  }
  /* ---- v = (X_K - X0) / dt ---- */
  for (int k = 0; k < n; ++k)
    for (int a = 0; a < 3; ++a) {
      gXn[4 * (size_t)k + a] += gV[4 * (size_t)k + a] * c.inv_dt;
      gX0[4 * (size_t)k + a] -= gV[4 * (size_t)k + a] * c.inv_dt;
    }

  /* ---- iterations, last to first ---- */
  for (int k = K - 1; k >= 0; --k) {
    const real* X = XK + n4 * k;
    const real* lam = LAM + (size_t)n * k;
    const real* rk = RHO + (size_t)n * k;
    memset(gX, 0, sizeof(real) * n4);
    memset(gl, 0, sizeof(real) * (size_t)n);
    /* delta_p and its clamps: X_{k+1} = box(X_k + clamp(P / pho0)) */
    for (int i = 0; i < n; ++i) {
      const real* xi = X + 4 * (size_t)i;
      real P[3] = {0, 0, 0};
      FOR_WINDOW(&c, cs, X, i, j) {
        if (j == i) continue;
        const real* xj = X + 4 * (size_t)j;
        real r[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
        real corr = c.coef_corr * RPOW(poly6(&c, r[0] * r[0] + r[1] * r[1] + r[2] * r[2]), n_corr);
        real f[3];
        spiky(&c, r, f);
        for (int a = 0; a < 3; ++a) P[a] += (lam[i] + lam[j] + corr) * f[a];
      }
      for (int a = 0; a < 3; ++a) {
        real dpa = P[a] / pho0;
        real d = RMAX(RMIN(dpa, c.max_dp), -c.max_dp);
        real u = xi[a] + d;
        real gu;
        if (u > c.hi[a]) {
          g_ulim[a] += gXn[4 * (size_t)i + a];
          gu = 0;
        } else if (u < c.lo[a]) {
          g_llim[a] += gXn[4 * (size_t)i + a];
          gu = 0;
        } else {
          gu = gXn[4 * (size_t)i + a];
        }
        gX[4 * (size_t)i + a] += gu;
        Pb[4 * (size_t)i + a] = (dpa < c.max_dp && dpa > -c.max_dp) ? gu / pho0 : 0;
      }
    }
    for (int i = 0; i < n; ++i) {
      const real* xi = X + 4 * (size_t)i;
      const real* pb = Pb + 4 * (size_t)i;
      FOR_WINDOW(&c, cs, X, i, j) {
        if (j == i) continue;
        const real* xj = X + 4 * (size_t)j;
        real r[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
        real q = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        real s = RSQRT(q);
        if (s >= c.h || (double)s < c.kernel_eps) continue;
        real wq = poly6(&c, q);
        real corr = c.coef_corr * RPOW(wq, n_corr);
        real f[3];
        spiky(&c, r, f);
        real fp = f[0] * pb[0] + f[1] * pb[1] + f[2] * pb[2];
        gl[i] += fp;
        gl[j] += fp;
        sym3 Jm;
        spiky_jac(&c, r, s, &Jm);
        real jp[3];
        sym3_mul(&Jm, pb, jp);
        real ds = 2 * c.coef_corr * n_corr * RPOW(wq, n_corr - 1) * dpoly6(&c, q);
        real lsum = lam[i] + lam[j] + corr;
        for (int a = 0; a < 3; ++a) {
          real m = lsum * jp[a] + ds * r[a] * fp;
          gX[4 * (size_t)i + a] += m;
          gX[4 * (size_t)j + a] -= m;
        }
      }
    }
    /* lambda: lambda_i = -(rho_i / pho0 - 1) / (S_i + eps) */
    for (int i = 0; i < n; ++i) {
      const real* xi = X + 4 * (size_t)i;
      real gi[3] = {0, 0, 0}, gj2 = 0;
      FOR_WINDOW(&c, cs, X, i, j) {
        const real* xj = X + 4 * (size_t)j;
        real r[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
        real f[3];
        spiky(&c, r, f);
        for (int a = 0; a < 3; ++a) gi[a] += f[a] / pho0;
        if (j != i) gj2 += (f[0] * f[0] + f[1] * f[1] + f[2] * f[2]) / (pho0 * pho0);
      }
      real Sv = gj2 + gi[0] * gi[0] + gi[1] * gi[1] + gi[2] * gi[2];
      real D = Sv + eps;
      real Cb = -gl[i] / D;
      Sbar[i] = -gl[i] * lam[i] / D;
      Rtot[i] = (k == K - 1 ? gr[i] : 0) + Cb / pho0;
      memcpy(G + 4 * (size_t)i, gi, sizeof(real) * 3);
      (void)rk;
    }
    for (int i = 0; i < n; ++i) {
      const real* xi = X + 4 * (size_t)i;
      FOR_WINDOW(&c, cs, X, i, j) {
        if (j == i) continue;
        const real* xj = X + 4 * (size_t)j;
        real r[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
        real q = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        if (q >= c.h2) continue;
        real dw = dpoly6(&c, q);
        for (int a = 0; a < 3; ++a) {
          gX[4 * (size_t)i + a] += Rtot[i] * dw * 2 * r[a];
          gX[4 * (size_t)j + a] -= Rtot[i] * dw * 2 * r[a];
        }
        real s = RSQRT(q);
        if (s >= c.h || (double)s < c.kernel_eps) continue;
        real f[3];
        spiky(&c, r, f);
        real av[3];
        for (int a = 0; a < 3; ++a) av[a] = Sbar[i] * (2 * f[a] / pho0 + 2 * G[4 * (size_t)i + a]);
        sym3 Jm;
        spiky_jac(&c, r, s, &Jm);
        real ja[3];
        sym3_mul(&Jm, av, ja);
        for (int a = 0; a < 3; ++a) {
          gX[4 * (size_t)i + a] += ja[a] / pho0;
          gX[4 * (size_t)j + a] -= ja[a] / pho0;
        }
      }
    }
    memcpy(gXn, gX, sizeof(real) * n4); /* becomes the adjoint of X_k */
  }
  /* ---- x* = x + dt v + dt^2 g, then un-permute ---- */
  for (int k = 0; k < n; ++k) {
    const uint32_t q = perm[k];
    for (int a = 0; a < 3; ++a) {
      g_pos[4 * (size_t)q + a] = gXn[4 * (size_t)k + a] + gX0[4 * (size_t)k + a];
      g_vel[4 * (size_t)q + a] = dt * gXn[4 * (size_t)k + a];
    }
    g_pos[4 * (size_t)q + 3] = 0;
    g_vel[4 * (size_t)q + 3] = 0;
  }
  free(S); free(X0); free(XK); free(LAM); free(RHO); free(V); free(gX); free(gXn); free(gX0);
  free(gV); free(gl); free(gr); free(Pb); free(G); free(Sbar); free(Rtot); free(keys); free(perm); free(cs);
  return 0;
}
