/*
 * ssf_oracle.c — CPU restatement of naeioi/PBF-CUDA's screen-space fluid
 * renderer (fluids/SSFRenderer.cpp:113-358 and the shaders
 * fluids/shader/SSF*.glsl), the oracle for include/pbf_ssf.h.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/ and bench.py's CPU
 * baseline load this library, as the checker or the timed CPU baseline.  The
 * CUDA product path never links, loads or falls back to it.
 *
 * Compiled twice (oracle/build_oracle.py), like pbf_oracle.c:
 *   ORACLE_F64 -> oracle_ssf_*_f64: every quantity in double (the FP64 oracle);
 *   otherwise  -> oracle_ssf_*_f32: float, each operation rounded on its own
 *                 (-ffp-contract=off; fused multiply-adds only where written as
 *                 fmaf) in the order of the shader source, which
 *                 is also the order of the CUDA kernels' explicitly rounded
 *                 operations.  So the splats (depth, thickness) agree with the
 *                 GPU bit for bit, and so do the normals and the shading options
 *                 without exp when given the same input images; smoothing and
 *                 the depth, thickness, full and tinted-refraction shading differ
 *                 from the GPU only through the libraries' expf.
 *   The stage entry points (oracle_ssf_smooth / _normals / _shade) take the
 *   previous stage's image as input, so each stage is checked on the GPU's own
 *   input (tests/test_gpu_ssf.py).
 *
 * Parity pinned against the reference's own shader code: its renderer is
 * OpenGL and no graphics stack exists here, but its SSF shaders
 * (fluids/shader/SSF*.glsl) are plain arithmetic, and oracle/ref_harness
 * compiles them as C++ and runs them on the CPU with the fixed-function steps
 * made explicit (ssf_ref.cpp).  Their outputs, recorded in
 * tests/golden/ssf_ref_*.npz by tests/golden/make_ssf_golden.py, agree with
 * this restatement stage by stage (tests/test_ssf_ref.py: the same fragments
 * and pixels, splat depth within 1e-6 relative, smoothing and normals
 * bit-identical here, shading within 1e-5).  GL implementation details are
 * fixed the way include/pbf_ssf.h states them (exact depth minimum,
 * fixed-point thickness, half-open sprite squares, GL point clipping, 0
 * outside the image in smoothing, wrap-around in normal restoration, shading
 * only where the depth is below the far plane).  Known answers check the
 * formulas besides (tests/test_ssf_oracle.py).
 *
 * Images: row-major W x H, row 0 at the bottom; depth/thickness 1 float per
 * pixel, normal_D and colour 4.  Particles: stride-4 float (x, y, z, w).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/pbf_ssf.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef ORACLE_F64
typedef double real;
#define SFX(name) name##_f64
#define RSQRT(x) sqrt(x)
#define REXP(x) exp(x)
#define RCEIL(x) ceil(x)
#define RFLOOR(x) floor(x)
#define RABS(x) fabs(x)
#define RMAX(a, b) fmax((a), (b))
#define RMIN(a, b) fmin((a), (b))
#define RINF HUGE_VAL
#define RFMA(a, b, c) fma((a), (b), (c))
#else
typedef float real;
#define SFX(name) name##_f32
#define RSQRT(x) sqrtf(x)
#define REXP(x) expf(x)
#define RCEIL(x) ceilf(x)
#define RFLOOR(x) floorf(x)
#define RABS(x) fabsf(x)
#define RMAX(a, b) fmaxf((a), (b))
#define RMIN(a, b) fminf((a), (b))
#define RINF HUGE_VALF
#define RFMA(a, b, c) fmaf((a), (b), (c))
#endif

#define CLEAR_DEPTH ((real)100)     /* glClearTexImage(d_depth_a/b, 100), SSFRenderer.cpp:159-162 */
#define BACKGROUND ((real)99)       /* SSFsmooth_depth.f.glsl:68 */

typedef struct {
  int W, H;
  real V[16], P[16], IV[16];
  real p_n, p_f, p_t, p_r, r;
  int kernel_r, keep_edge, blur_option, shading;
  real blur_r, blur_z, r0, sky[3];
  const float* sky_map; /* [6][S][S][3] */
  int sky_size;
} ssf_consts;

/* 4 x 4 inverse by cofactors in double (column-major). */
static int invert4(const double* a, double* out) {
  double inv[16];
  inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] +
           a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
  inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] -
           a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
  inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] +
           a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
  inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] -
            a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
  inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] -
           a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
  inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] +
           a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
  inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] -
           a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
  inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] +
            a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
  inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] +
           a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
  inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] -
           a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
  inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] +
            a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
  inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] -
            a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
  inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] -
           a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
  inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] +
           a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
  inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] -
            a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
  inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] +
            a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
  const double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
  if (!(det != 0.0) || !isfinite(det)) return 0;
  for (int i = 0; i < 16; ++i) out[i] = inv[i] / det;
  return 1;
}

static int make_consts(const pbf_ssf_params* p, const float* sky, int sky_size, ssf_consts* c) {
  double v[16], iv[16];
  c->W = p->width, c->H = p->height;
  for (int i = 0; i < 16; ++i) {
    c->V[i] = p->view[i], c->P[i] = p->proj[i];
    v[i] = p->view[i];
  }
  if (!invert4(v, iv)) return 0;
  for (int i = 0; i < 16; ++i) c->IV[i] = (real)iv[i];
  c->p_n = p->p_n, c->p_f = p->p_f, c->p_t = p->p_t, c->p_r = p->p_r, c->r = p->radius;
  c->kernel_r = p->kernel_r, c->keep_edge = p->keep_edge, c->blur_option = p->blur_option;
  c->shading = p->shading_option;
  /* loadParams: blur_r = 1 / sigma_r, blur_z = 1 / sigma_z (SSFRenderer.cpp:286-287) */
  c->blur_r = (real)1 / (real)p->sigma_r;
  c->blur_z = (real)1 / (real)p->sigma_z;
  c->r0 = p->r0;
  for (int a = 0; a < 3; ++a) c->sky[a] = p->sky[a];
  c->sky_map = sky;
  c->sky_size = sky ? sky_size : 0;
  return 1;
}

/* Row r of M (column-major) times (x, y, z, w), left to right as GLSL writes it. */
static inline real mrow(const real* M, int r, real x, real y, real z, real w) {
  return M[r] * x + M[4 + r] * y + M[8 + r] * z + M[12 + r] * w;
}

/* ---- 1-2. depth and thickness splats (SSFget_depth.*.glsl, SSFget_thick.*.glsl) ---- */

/* Splats every particle: depth[k] = min(100, -nviewPos.z of the covering
 * fragments) (SSFget_depth.f.glsl:21-37 under GL_LESS, SSFRenderer.cpp:183-190),
 * thick[k] = the fixed-point sum of 2 r z (SSFget_thick.f.glsl:21-25 under
 * additive blending, SSFRenderer.cpp:216-218).  Returns the fragment count. */
static long long splat(const ssf_consts* c, const float* pos, int n, real* depth, long long* tfx) {
  const int W = c->W, H = c->H;
  long long frags = 0;
  for (size_t k = 0; k < (size_t)W * H; ++k) depth[k] = CLEAR_DEPTH, tfx[k] = 0;
  for (int i = 0; i < n; ++i) {
    const real px_ = pos[4 * i], py_ = pos[4 * i + 1], pz_ = pos[4 * i + 2];
    /* vertex shader: viewPos = view * (aPos, 1), gl_Position = proj * viewPos */
    const real vx = mrow(c->V, 0, px_, py_, pz_, 1), vy = mrow(c->V, 1, px_, py_, pz_, 1);
    const real vz = mrow(c->V, 2, px_, py_, pz_, 1), vw = mrow(c->V, 3, px_, py_, pz_, 1);
    const real cx = mrow(c->P, 0, vx, vy, vz, vw), cy = mrow(c->P, 1, vx, vy, vz, vw);
    const real cz = mrow(c->P, 2, vx, vy, vz, vw), cw = mrow(c->P, 3, vx, vy, vz, vw);
    /* GL point clipping */
    if (!(cw > 0) || !(cw < RINF)) continue;
    if (!(-cw <= cx && cx <= cw && -cw <= cy && cy <= cw && -cw <= cz && cz <= cw)) continue;
    const real hw = (real)0.5f * (real)W, hh = (real)0.5f * (real)H;
    const real xw = hw * (cx / cw) + hw, yw = hh * (cy / cw) + hh;
    /* gl_PointSize = r * p_n * s_h / (-viewPos.z * p_t) (SSFget_depth.v.glsl:24), >= 1 */
    real size = c->r * c->p_n * (real)H / (-vz * c->p_t);
    if (!(size < RINF)) continue;
    size = RMAX(size, (real)1);
    const real s2 = (real)2 / size;
    const real lox = xw - (real)0.5f * size, loy = yw - (real)0.5f * size;
    const real fx0 = RCEIL(lox - (real)0.5f), fx1 = RCEIL(lox + size - (real)0.5f) - (real)1;
    const real fy0 = RCEIL(loy - (real)0.5f), fy1 = RCEIL(loy + size - (real)0.5f) - (real)1;
    const int x0 = (int)RMAX(fx0, (real)0), x1 = (int)RMIN(fx1, (real)(W - 1));
    const int y0 = (int)RMAX(fy0, (real)0), y1 = (int)RMIN(fy1, (real)(H - 1));
    for (int py = y0; py <= y1; ++py)
      for (int px = x0; px <= x1; ++px) {
        /* gl_PointCoord (upper-left origin), one reciprocal of the point size per
         * sprite: x = 2 s - 1 = (px + 1/2 - xw) 2 / size, y = 2 t - 1 = (yw - py - 1/2) 2 / size */
        const real x = ((real)px + (real)0.5f - xw) * s2;
        const real y = (yw - ((real)py + (real)0.5f)) * s2;
        const real pho = RFMA(x, x, y * y);
        if (pho > 1) continue; /* discard */
        const real z = RSQRT((real)1 - pho);
        const real d = -RFMA(z, c->r, vz); /* -nviewPos.z, nviewPos = viewPos + (x, y, z) r */
        const real th = (real)2 * c->r * z;
        const size_t k = (size_t)py * W + px;
        if (d < depth[k]) depth[k] = d;
        tfx[k] += llrint((double)th * 4294967296.0);
        ++frags;
      }
  }
  return frags;
}

/* ---- 3. smoothing (SSFsmooth_depth.f.glsl:26-75) ---- */

static void smooth(const ssf_consts* c, const real* src, real* dst) {
  const int W = c->W, H = c->H, R = c->kernel_r;
#pragma omp parallel for schedule(dynamic, 4)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const real z = src[(size_t)y * W + x];
      if (z > BACKGROUND) continue; /* dst keeps its content */
      real sum = 0, wsum = 0;
      for (int dx = -R; dx <= R; ++dx)
        for (int dy = -R; dy <= R; ++dy) {
          const int sx = x + dx, sy = y + dy;
          const real s = (sx >= 0 && sx < W && sy >= 0 && sy < H) ? src[(size_t)sy * W + sx] : (real)0;
          const real w = REXP((real)(-(dx * dx + dy * dy)) * c->blur_r * c->blur_r);
          if (c->blur_option == 0) {
            const real r2 = (s - z) * c->blur_z;
            const real g = REXP(-r2 * r2);
            const real wg = w * g;
            sum += s * wg;
            wsum += wg;
          } else {
            sum += s * w;
            wsum += w;
          }
        }
      if (wsum > 0) sum /= wsum;
      dst[(size_t)y * W + x] = sum;
    }
}

/* ---- 4. normals (SSFrestore_normal.f.glsl:31-58) ---- */

static void normals(const ssf_consts* c, const real* depth, real* nd) {
  const int W = c->W, H = c->H;
  const real f_x = c->p_n / c->p_r, f_y = c->p_n / c->p_t;
  const real c_x = (real)2 / ((real)W * f_x), c_y = (real)2 / ((real)H * f_y);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      /* getZ = -texture(zTex); texture coordinates wrap (REPEAT) */
      const int xp = x + 1 == W ? 0 : x + 1, xm = x == 0 ? W - 1 : x - 1;
      const int yp = y + 1 == H ? 0 : y + 1, ym = y == 0 ? H - 1 : y - 1;
      const real z = -depth[(size_t)y * W + x];
      real dzdx = -depth[(size_t)y * W + xp] - z, dzdy = -depth[(size_t)yp * W + x] - z;
      const real dzdx2 = z - -depth[(size_t)y * W + xm], dzdy2 = z - -depth[(size_t)ym * W + x];
      if (c->keep_edge == 1) {
        if (RABS(dzdx2) < RABS(dzdx)) dzdx = dzdx2;
        if (RABS(dzdy2) < RABS(dzdy)) dzdy = dzdy2;
      }
      const real nx = -c_y * dzdx, ny = -c_x * dzdy, nz = -(c_x * c_y * z);
      const real d = RSQRT(nx * nx + ny * ny + nz * nz);
      real* o = nd + 4 * ((size_t)y * W + x);
      o[0] = nx / d, o[1] = ny / d, o[2] = nz / d, o[3] = d;
    }
}

/* ---- 5. shading (SSFshading.f.glsl) ---- */

static void sky_color(const ssf_consts* c, const real d[3], real out[3]) {
  if (c->sky_size <= 0) {
    out[0] = c->sky[0], out[1] = c->sky[1], out[2] = c->sky[2];
    return;
  }
  const real ax = RABS(d[0]), ay = RABS(d[1]), az = RABS(d[2]);
  int face;
  real sc, tc, ma;
  /* the GL specification's cube-map face table */
  if (ax >= ay && ax >= az) {
    face = d[0] >= 0 ? 0 : 1, ma = ax;
    sc = d[0] >= 0 ? -d[2] : d[2], tc = -d[1];
  } else if (ay >= az) {
    face = d[1] >= 0 ? 2 : 3, ma = ay;
    sc = d[0], tc = d[1] >= 0 ? d[2] : -d[2];
  } else {
    face = d[2] >= 0 ? 4 : 5, ma = az;
    sc = d[2] >= 0 ? d[0] : -d[0], tc = -d[1];
  }
  if (!(ma > 0) || !(ma < RINF)) {
    out[0] = c->sky[0], out[1] = c->sky[1], out[2] = c->sky[2];
    return;
  }
  const int S = c->sky_size;
  const real s = (real)0.5f * (sc / ma + 1), t = (real)0.5f * (tc / ma + 1);
  const real u = s * (real)S - (real)0.5f, v = t * (real)S - (real)0.5f;
  const real fu = RFLOOR(u), fv = RFLOOR(v);
  const real a = u - fu, b = v - fv;
  int i0 = (int)fu, i1 = (int)fu + 1, j0 = (int)fv, j1 = (int)fv + 1;
  i0 = i0 < 0 ? 0 : (i0 > S - 1 ? S - 1 : i0);
  i1 = i1 < 0 ? 0 : (i1 > S - 1 ? S - 1 : i1);
  j0 = j0 < 0 ? 0 : (j0 > S - 1 ? S - 1 : j0);
  j1 = j1 < 0 ? 0 : (j1 > S - 1 ? S - 1 : j1);
  const float* F = c->sky_map + (size_t)face * S * S * 3;
  for (int ch = 0; ch < 3; ++ch)
    out[ch] = (1 - a) * (1 - b) * F[((size_t)j0 * S + i0) * 3 + ch] + a * (1 - b) * F[((size_t)j0 * S + i1) * 3 + ch] +
              (1 - a) * b * F[((size_t)j1 * S + i0) * 3 + ch] + a * b * F[((size_t)j1 * S + i1) * 3 + ch];
}

/* trace_color (SSFshading.f.glsl:50-72) */
static void trace_color(const ssf_consts* c, const real p[3], const real d[3], real out[3]) {
  const real* M = c->IV;
  real wp[3], wd[3], its[3];
  for (int r = 0; r < 3; ++r) {
    wp[r] = M[r] * p[0] + M[4 + r] * p[1] + M[8 + r] * p[2] + M[12 + r];
    wd[r] = M[r] * d[0] + M[4 + r] * d[1] + M[8 + r] * d[2];
  }
  const real t = -wp[2] / wd[2];
  for (int r = 0; r < 3; ++r) its[r] = wp[r] + t * wd[r];
  if (t > 0 && RABS(its[0]) < 5 && RABS(its[1]) < 5) {
    const real uvx = (real)10 * (its[0] - (real)-5) / (real)10, uvy = (real)10 * (its[1] - (real)-5) / (real)10;
    const real u = uvx - RFLOOR(uvx), v = uvy - RFLOOR(uvy);
    int flip = 1;
    if (u > (real)0.5f) flip = 1 - flip;
    if (v > (real)0.5f) flip = 1 - flip;
    const real g = flip == 1 ? (real)0.8f : (real)0.6f;
    out[0] = out[1] = out[2] = g;
    return;
  }
  sky_color(c, wd, out);
}

static void shade(const ssf_consts* c, const real* depth, const real* nd, const real* thick, float* color) {
  const int W = c->W, H = c->H;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t k = (size_t)y * W + x;
      const real ze = depth[k];
      if (!(ze < c->p_f)) continue; /* the depth test against the cleared buffer */
      const real u = ((real)x + (real)0.5f) / (real)W, v = ((real)y + (real)0.5f) / (real)H;
      const real n[3] = {nd[4 * k], nd[4 * k + 1], nd[4 * k + 2]};
      /* getPos */
      const real p[3] = {((real)2 * u - 1) * c->p_r * ze / c->p_n, ((real)2 * v - 1) * c->p_t * ze / c->p_n, -ze};
      real out[3];
      const real pl = RSQRT(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
      const real e[3] = {-p[0] / pl, -p[1] / pl, -p[2] / pl}; /* normalize(-p) */
      const real ne = n[0] * e[0] + n[1] * e[1] + n[2] * e[2];
      switch (c->shading) {
        case PBF_SSF_DEPTH: {
          if (ze > 50) continue;
          const real ez = REXP(ze);
          out[0] = out[1] = out[2] = (ez / (ez + 1) - (real)0.5f) * 2;
          break;
        }
        case PBF_SSF_THICK: {
          if (ze > 50) continue;
          const real et = REXP(thick[k]);
          out[0] = out[1] = out[2] = (et / (et + 1) - (real)0.5f) * 2;
          break;
        }
        case PBF_SSF_NORMAL:
          out[0] = n[0], out[1] = n[1], out[2] = n[2];
          break;
        case PBF_SSF_FRESNEL: {
          const real q = 1 - ne;
          out[0] = out[1] = out[2] = c->r0 + (1 - c->r0) * (q * q);
          break;
        }
        default: {
          const real q = 1 - ne;
          const real r = c->r0 + (1 - c->r0) * (q * q * q);
          real refl[3], refr[3], cl[3], cr[3];
          for (int a = 0; a < 3; ++a) {
            refl[a] = -e[a] + (real)2 * ne * n[a];
            refr[a] = -e[a] - (real)0.2f * n[a];
          }
          if (c->shading == PBF_SSF_REFLECT) {
            trace_color(c, p, refl, out);
          } else if (c->shading == PBF_SSF_REFRACT) {
            trace_color(c, p, refr, out);
          } else {
            const real att = RMAX(REXP((real)0.5f * -thick[k]), (real)0.2f);
            const real tint[3] = {(real)6 / 256, (real)105 / 256, (real)217 / 256};
            trace_color(c, p, refr, cr);
            for (int a = 0; a < 3; ++a) cr[a] = (1 - att) * tint[a] + att * cr[a];
            if (c->shading == PBF_SSF_REFRACT_TINTED) {
              for (int a = 0; a < 3; ++a) out[a] = cr[a];
            } else {
              trace_color(c, p, refl, cl);
              for (int a = 0; a < 3; ++a) out[a] = (1 - r) * cr[a] + r * cl[a];
            }
          }
        }
      }
      color[4 * k] = (float)out[0], color[4 * k + 1] = (float)out[1], color[4 * k + 2] = (float)out[2];
      color[4 * k + 3] = 1.f;
    }
}

/*
 * The whole render (SSFRenderer::render, fluids/SSFRenderer.cpp:113-146).
 * Outputs (each may be NULL): depth_raw (the splat, before smoothing), depth
 * (the smoothed depth shading reads: the m_ab ping-pong's last target),
 * thick, normal_D, color (written where drawn, else left as given).  Returns
 * the number of fragments that passed the circle test, or -1 on bad input.
 */
long long SFX(oracle_ssf_render)(const pbf_ssf_params* p, const float* pos, int n, const float* sky, int sky_size,
                                 float* depth_raw, float* depth, float* thick, float* normal_D, float* color) {
  ssf_consts c;
  if (!p || p->width < 1 || p->height < 1 || n < 0 || !make_consts(p, sky, sky_size, &c)) return -1;
  const size_t npix = (size_t)c.W * c.H;
  real* a = (real*)malloc(sizeof(real) * npix);
  real* b = (real*)malloc(sizeof(real) * npix);
  long long* tfx = (long long*)malloc(sizeof(long long) * npix);
  real* nd = (real*)malloc(sizeof(real) * 4 * npix);
  real* th = (real*)malloc(sizeof(real) * npix);
  if (!a || !b || !tfx || !nd || !th) {
    free(a), free(b), free(tfx), free(nd), free(th);
    return -1;
  }
  const long long frags = splat(&c, pos, n, a, tfx);
  for (size_t k = 0; k < npix; ++k) {
    b[k] = CLEAR_DEPTH;
    th[k] = (real)((double)tfx[k] * 0x1p-32);
  }
  if (depth_raw)
    for (size_t k = 0; k < npix; ++k) depth_raw[k] = (float)a[k];
  const real* fin = a;
  for (int it = 1; it <= p->smooth_niter; ++it) {
    const real* src = (it & 1) ? a : b;
    real* dst = (it & 1) ? b : a;
    smooth(&c, src, dst);
    fin = dst;
  }
  normals(&c, fin, nd);
  if (color) shade(&c, fin, nd, th, color);
  if (depth)
    for (size_t k = 0; k < npix; ++k) depth[k] = (float)fin[k];
  if (thick)
    for (size_t k = 0; k < npix; ++k) thick[k] = (float)th[k];
  if (normal_D)
    for (size_t k = 0; k < 4 * npix; ++k) normal_D[k] = (float)nd[k];
  free(a), free(b), free(tfx), free(nd), free(th);
  return frags;
}

/* ---- single stages on given images (for stage-by-stage parity) ---- */

static real* to_real(const float* src, size_t count) {
  real* out = (real*)calloc(count ? count : 1, sizeof(real));
  if (out)
    for (size_t k = 0; k < count; ++k) out[k] = src[k];
  return out;
}

/* smooth_niter smoothing passes from a splatted depth image (the m_ab
 * ping-pong, SSFRenderer.cpp:130-137): out = the last pass's target. */
int SFX(oracle_ssf_smooth)(const pbf_ssf_params* p, const float* raw, float* out) {
  ssf_consts c;
  if (!p || !raw || !out || !make_consts(p, NULL, 0, &c)) return -1;
  const size_t npix = (size_t)c.W * c.H;
  real* a = to_real(raw, npix);
  real* b = (real*)malloc(sizeof(real) * npix);
  if (!a || !b) {
    free(a), free(b);
    return -1;
  }
  for (size_t k = 0; k < npix; ++k) b[k] = CLEAR_DEPTH;
  const real* fin = a;
  for (int it = 1; it <= p->smooth_niter; ++it) {
    const real* src = (it & 1) ? a : b;
    real* dst = (it & 1) ? b : a;
    smooth(&c, src, dst);
    fin = dst;
  }
  for (size_t k = 0; k < npix; ++k) out[k] = (float)fin[k];
  free(a), free(b);
  return 0;
}

/* Normal restoration (SSFrestore_normal.f.glsl) of a depth image. */
int SFX(oracle_ssf_normals)(const pbf_ssf_params* p, const float* depth, float* normal_D) {
  ssf_consts c;
  if (!p || !depth || !normal_D || !make_consts(p, NULL, 0, &c)) return -1;
  const size_t npix = (size_t)c.W * c.H;
  real* d = to_real(depth, npix);
  real* nd = (real*)malloc(sizeof(real) * 4 * npix);
  if (!d || !nd) {
    free(d), free(nd);
    return -1;
  }
  normals(&c, d, nd);
  for (size_t k = 0; k < 4 * npix; ++k) normal_D[k] = (float)nd[k];
  free(d), free(nd);
  return 0;
}

/* Shading (SSFshading.f.glsl) of given depth, normal_D and thickness images. */
int SFX(oracle_ssf_shade)(const pbf_ssf_params* p, const float* depth, const float* normal_D, const float* thick,
                          const float* sky, int sky_size, float* color) {
  ssf_consts c;
  if (!p || !depth || !normal_D || !thick || !color || !make_consts(p, sky, sky_size, &c)) return -1;
  const size_t npix = (size_t)c.W * c.H;
  real* d = to_real(depth, npix);
  real* nd = to_real(normal_D, 4 * npix);
  real* th = to_real(thick, npix);
  if (!d || !nd || !th) {
    free(d), free(nd), free(th);
    return -1;
  }
  shade(&c, d, nd, th, color);
  free(d), free(nd), free(th);
  return 0;
}
