// ssf.cu — the screen-space fluid surface pipeline of include/pbf_ssf.h: the
// reference's OpenGL SSFRenderer (fluids/SSFRenderer.cpp:113-358, shaders
// fluids/shader/SSF*.glsl) as CUDA kernels over headless device images.
//
// One render = clear, splat (depth + thickness of every sprite fragment),
// resolve, smooth_niter smoothing passes, normals, shading: 5 + smooth_niter
// launches on the caller's stream.
//
//   k_ssf_splat   a warp takes 32 particles; each lane projects one (the vertex
//                 shader), then the warp rasterises the 32 sprites one after the
//                 other, its lanes spread over the sprite's pixels (the fragment
//                 shaders).  A pixel keeps the smallest eye depth (atomicMin on
//                 an order-preserving integer image of the float) and the sum of
//                 2 r z in 64-bit fixed point (2^-32 per unit): both independent
//                 of the order fragments arrive in, so renders are deterministic.
//                 The vertex and fragment arithmetic is written with explicitly
//                 rounded operations (fused multiply-adds only where written
//                 out) in the order of the shader source, so the float oracle,
//                 written the same way, reproduces depth and thickness bit for
//                 bit.  gl_PointCoord takes one reciprocal of the point size per
//                 sprite (GL leaves its precision to the implementation).
//   k_ssf_smooth  32 x 16 output pixels per 256-thread block, the source tile
//                 and its kernel_r halo staged in shared memory with the spatial
//                 weights; taps summed in the shader's order (dx outer, dy inner).
//   k_ssf_normal  one thread per pixel, neighbours wrapping at the image edges.
//   k_ssf_shade   one thread per pixel; trace_color's floor and sky cube map.
//
// All kernels are bounded loops over in-range indices: no waits, no device
// asserts.
#include <cmath>
#include <cstring>
#include <new>

#include "pbf_internal.cuh"
#include "../../include/pbf_ssf.h"

namespace pbf {
pbf_status set_error(pbf_status s, const char* msg);
pbf_status set_cuda_error(cudaError_t e, const char* what);
}  // namespace pbf

namespace {

constexpr int kMaxKernelR = 20;            // GUI range of kernel_r (fluids/Renderer.cpp:103-105)
constexpr int kMaxSmoothIter = 64;
constexpr int kMaxImageSide = 16384;
constexpr float kClearDepth = 100.f;       // glClearTexImage(d_depth_a/b, ..., 100) (SSFRenderer.cpp:159-162)
constexpr float kBackground = 99.f;        // smoothing skips z > 99 (SSFsmooth_depth.f.glsl:68)
constexpr float kThickScale = 4294967296.f;  // 2^32: fixed-point units per unit of thickness
constexpr int kSmoothTileW = 32, kSmoothTileH = 16, kSmoothThreadsY = 8;

struct SsfConsts {
  int W, H;
  float V[16], P[16], IV[16];
  float p_n, p_f, p_t, p_r;
  float r;
  int kernel_r;
  float blur_r, blur_z;
  int keep_edge, blur_option, shading;
  float r0;
  float sky[3];
  const float4* sky_map;  // [6][S][S], rgb in xyz
  int sky_size;
};

// ---- explicitly rounded float arithmetic (the splat path) --------------------------------

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

// Row r of M (column-major) times (x, y, z, w), summed left to right as the
// GLSL mat4 * vec4 product is written out: ((m0 x + m1 y) + m2 z) + m3 w.
__device__ __forceinline__ float mrow(const float* M, int r, float x, float y, float z, float w) {
  return fa(fa(fa(fm(M[r], x), fm(M[4 + r], y)), fm(M[8 + r], z)), fm(M[12 + r], w));
}

// Order-preserving map of a float onto uint32 (atomicMin on the integers is
// min on the floats; NaN never reaches it).
__device__ __forceinline__ uint32_t depth_key(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float depth_of_key(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// One particle's sprite: the vertex shader (SSFget_depth.v.glsl:15-24) and
// the point's window-space square, clipped to the image.
struct Sprite {
  float xw, yw, s2, vz;  // s2 = 2 / gl_PointSize
  int x0, x1, y0, y1;    // inclusive pixel ranges; empty when x0 > x1
};

__device__ __forceinline__ bool make_sprite(const SsfConsts& c, float4 p, Sprite& s) {
  const float vx = mrow(c.V, 0, p.x, p.y, p.z, 1.f), vy = mrow(c.V, 1, p.x, p.y, p.z, 1.f);
  const float vz = mrow(c.V, 2, p.x, p.y, p.z, 1.f), vw = mrow(c.V, 3, p.x, p.y, p.z, 1.f);
  const float cx = mrow(c.P, 0, vx, vy, vz, vw), cy = mrow(c.P, 1, vx, vy, vz, vw);
  const float cz = mrow(c.P, 2, vx, vy, vz, vw), cw = mrow(c.P, 3, vx, vy, vz, vw);
  // GL point clipping: a point outside the clip volume is not drawn (NaN fails too)
  if (!(cw > 0.f) || !(cw < INFINITY)) return false;
  if (!(-cw <= cx && cx <= cw && -cw <= cy && cy <= cw && -cw <= cz && cz <= cw)) return false;
  const float hw = 0.5f * (float)c.W, hh = 0.5f * (float)c.H;
  s.xw = fa(fm(hw, fd(cx, cw)), hw);
  s.yw = fa(fm(hh, fd(cy, cw)), hh);
  // gl_PointSize = r * p_n * s_h / (-viewPos.z * p_t), at least one pixel
  const float size = fd(fm(fm(c.r, c.p_n), (float)c.H), fm(-vz, c.p_t));
  if (!(size < INFINITY)) return false;
  const float sz = fmaxf(size, 1.f);
  s.s2 = fd(2.f, sz);
  s.vz = vz;
  // pixels whose centres lie in [xw - size/2, xw + size/2)
  const float lox = fs(s.xw, fm(0.5f, sz)), loy = fs(s.yw, fm(0.5f, sz));
  const float fx0 = ceilf(fs(lox, 0.5f)), fx1 = ceilf(fs(fa(lox, sz), 0.5f)) - 1.f;
  const float fy0 = ceilf(fs(loy, 0.5f)), fy1 = ceilf(fs(fa(loy, sz), 0.5f)) - 1.f;
  s.x0 = (int)fmaxf(fx0, 0.f);
  s.x1 = (int)fminf(fx1, (float)(c.W - 1));
  s.y0 = (int)fmaxf(fy0, 0.f);
  s.y1 = (int)fminf(fy1, (float)(c.H - 1));
  return s.x0 <= s.x1 && s.y0 <= s.y1;
}

__global__ void __launch_bounds__(256) k_ssf_clear(int npix, uint32_t* __restrict__ zkey,
                                                   unsigned long long* __restrict__ tfx) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npix) return;
  zkey[k] = depth_key(kClearDepth);
  tfx[k] = 0ull;
}

__global__ void __launch_bounds__(256) k_ssf_splat(SsfConsts c, const float4* __restrict__ pos, int n,
                                                   uint32_t* __restrict__ zkey,
                                                   unsigned long long* __restrict__ tfx,
                                                   unsigned long long* __restrict__ frag_count) {
  const int lane = threadIdx.x & 31;
  const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x));
  Sprite me = {};
  const bool ok = i < n && make_sprite(c, pos[i], me);
  unsigned frags = 0;
  // thickness 2 r z in fixed point: z (2 r 2^32), the same value as (2 r z) 2^32
  const float qscale = fm(fm(2.f, c.r), kThickScale);
  unsigned todo = __ballot_sync(0xffffffffu, ok);
  while (todo) {
    const int src = __ffs(todo) - 1;
    todo &= todo - 1u;
    const float xw = __shfl_sync(0xffffffffu, me.xw, src), yw = __shfl_sync(0xffffffffu, me.yw, src);
    const float s2 = __shfl_sync(0xffffffffu, me.s2, src), vz = __shfl_sync(0xffffffffu, me.vz, src);
    const int x0 = __shfl_sync(0xffffffffu, me.x0, src), x1 = __shfl_sync(0xffffffffu, me.x1, src);
    const int y0 = __shfl_sync(0xffffffffu, me.y0, src), y1 = __shfl_sync(0xffffffffu, me.y1, src);
    const int w = x1 - x0 + 1;                 // 1 .. W
    const int total = w * (y1 - y0 + 1);       // <= W H < 2^31
    // fragment f = row * w + col, lanes strided by 32 (row, col stepped incrementally)
    int row = lane / w, col = lane - (lane / w) * w;
    const int drow = 32 / w, dcol = 32 - drow * w;
    for (int f = lane; f < total; f += 32) {
      const int px = x0 + col, py = y0 + row;
      // the fragment shader (SSFget_depth.f.glsl:21-37) at gl_PointCoord (upper-left
      // origin): x = 2 s - 1 = (px + 1/2 - xw) 2 / size, y = 2 t - 1 = (yw - py - 1/2) 2 / size
      const float x = fm(fs(fa((float)px, 0.5f), xw), s2);
      const float y = fm(fs(yw, fa((float)py, 0.5f)), s2);
      const float pho = __fmaf_rn(x, x, fm(y, y));
      if (!(pho > 1.f)) {
        const float z = __fsqrt_rn(fs(1.f, pho));
        const float depth = -__fmaf_rn(z, c.r, vz);  // -nviewPos.z, nviewPos = viewPos + (x, y, z) r
        const size_t k = (size_t)py * c.W + px;
        atomicMin(zkey + k, depth_key(depth));
        // 2 r dot((x, y, z), (0, 0, 1)) (SSFget_thick.f.glsl:24-25)
        const long long q = __float2ll_rn(fm(z, qscale));
        if (q) atomicAdd(tfx + k, (unsigned long long)q);
        ++frags;
      }
      col += dcol;
      row += drow;
      if (col >= w) {
        col -= w;
        ++row;
      }
    }
  }
  if (frag_count) {
    for (int o = 16; o > 0; o >>= 1) frags += __shfl_xor_sync(0xffffffffu, frags, o);
    if (lane == 0 && frags) atomicAdd(frag_count, (unsigned long long)frags);
  }
}

// depth_a <- the splat's depth, depth_b <- the clear value, thickness <- the
// fixed-point sums (SSFRenderer.cpp:159-162, 207).
__global__ void __launch_bounds__(256) k_ssf_resolve(int npix, const uint32_t* __restrict__ zkey,
                                                     const unsigned long long* __restrict__ tfx,
                                                     float* __restrict__ depth_a, float* __restrict__ depth_b,
                                                     float* __restrict__ thick) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npix) return;
  depth_a[k] = depth_of_key(zkey[k]);
  depth_b[k] = kClearDepth;
  thick[k] = __double2float_rn(__ll2double_rn((long long)tfx[k]) * 0x1p-32);
}

// One smoothing pass (SSFsmooth_depth.f.glsl:26-75): dst keeps its content where
// the source depth is background (> 99).  Taps in the shader's order; the
// range weight through exp2f and fused multiply-adds (within 1e-5 of the float
// oracle's expf and separate roundings).
__global__ void __launch_bounds__(kSmoothTileW * kSmoothThreadsY)
k_ssf_smooth(SsfConsts c, const float* __restrict__ src, float* __restrict__ dst) {
  constexpr int kTW = kSmoothTileW + 2 * kMaxKernelR, kTH = kSmoothTileH + 2 * kMaxKernelR;
  constexpr int kK = 2 * kMaxKernelR + 1;
  __shared__ float tile[kTW * kTH];
  __shared__ float wsp[kK * kK];
  const int R = c.kernel_r, K = 2 * R + 1;
  const int tw = kSmoothTileW + 2 * R, th = kSmoothTileH + 2 * R;
  const int gx0 = blockIdx.x * kSmoothTileW - R, gy0 = blockIdx.y * kSmoothTileH - R;
  const int tid = threadIdx.y * kSmoothTileW + threadIdx.x;
  constexpr int kThreads = kSmoothTileW * kSmoothThreadsY;
  for (int k = tid; k < tw * th; k += kThreads) {
    const int ty = k / tw, tx = k - ty * tw;
    const int gx = gx0 + tx, gy = gy0 + ty;
    tile[k] = (gx >= 0 && gx < c.W && gy >= 0 && gy < c.H) ? src[(size_t)gy * c.W + gx] : 0.f;  // texelFetch out of range: 0
  }
  for (int k = tid; k < K * K; k += kThreads) {
    const int a = k / K, b = k - a * K;
    const int dx = a - R, dy = b - R;
    // exp(-(dx*dx + dy*dy) * blur_r * blur_r)
    wsp[k] = expf(fm(fm((float)(-(dx * dx + dy * dy)), c.blur_r), c.blur_r));
  }
  __syncthreads();
  const int px = blockIdx.x * kSmoothTileW + threadIdx.x;
  for (int row = threadIdx.y; row < kSmoothTileH; row += kSmoothThreadsY) {
    const int py = blockIdx.y * kSmoothTileH + row;
    if (px >= c.W || py >= c.H) continue;
    const float* center = tile + (row + R) * tw + threadIdx.x + R;
    const float z = *center;
    if (z > kBackground) continue;
    float sum = 0.f, wsum = 0.f;
    if (c.blur_option == 0) {
      // g = exp(-((s - z) blur_z)^2) = 2^-((s - z) blur_z sqrt(log2 e))^2
      const float bz = c.blur_z * 1.2011224087864498f;
      for (int dx = -R; dx <= R; ++dx) {
        const float* wrow = wsp + (dx + R) * K + R;
        for (int dy = -R; dy <= R; ++dy) {
          const float s = center[dy * tw + dx];
          const float r2 = (s - z) * bz;
          const float wg = wrow[dy] * exp2f(-r2 * r2);
          sum = fmaf(s, wg, sum);
          wsum += wg;
        }
      }
    } else {
      for (int dx = -R; dx <= R; ++dx) {
        const float* wrow = wsp + (dx + R) * K + R;
        for (int dy = -R; dy <= R; ++dy) {
          const float w = wrow[dy];
          sum = fmaf(center[dy * tw + dx], w, sum);
          wsum += w;
        }
      }
    }
    if (wsum > 0.f) sum = fd(sum, wsum);
    dst[(size_t)py * c.W + px] = sum;
  }
}

// SSFrestore_normal.f.glsl:31-58; getZ returns -depth, neighbours wrap (REPEAT).
// Explicitly rounded in the float oracle's order: the same depth image gives
// the same normals bit for bit.
__global__ void __launch_bounds__(256) k_ssf_normal(SsfConsts c, const float* __restrict__ depth,
                                                    float4* __restrict__ normal_D) {
  const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
  if (px >= c.W || py >= c.H) return;
  const int xp = px + 1 == c.W ? 0 : px + 1, xm = px == 0 ? c.W - 1 : px - 1;
  const int yp = py + 1 == c.H ? 0 : py + 1, ym = py == 0 ? c.H - 1 : py - 1;
  const size_t row = (size_t)py * c.W;
  const float z = -depth[row + px];
  float dzdx = fs(-depth[row + xp], z), dzdy = fs(-depth[(size_t)yp * c.W + px], z);
  const float dzdx2 = fs(z, -depth[row + xm]), dzdy2 = fs(z, -depth[(size_t)ym * c.W + px]);
  if (c.keep_edge == 1) {
    if (fabsf(dzdx2) < fabsf(dzdx)) dzdx = dzdx2;
    if (fabsf(dzdy2) < fabsf(dzdy)) dzdy = dzdy2;
  }
  const float f_x = fd(c.p_n, c.p_r), f_y = fd(c.p_n, c.p_t);
  const float c_x = fd(2.f, fm((float)c.W, f_x)), c_y = fd(2.f, fm((float)c.H, f_y));
  const float nx = fm(-c_y, dzdx), ny = fm(-c_x, dzdy), nz = -fm(fm(c_x, c_y), z);
  const float d = __fsqrt_rn(fa(fa(fm(nx, nx), fm(ny, ny)), fm(nz, nz)));
  normal_D[row + px] = make_float4(fd(nx, d), fd(ny, d), fd(nz, d), d);
}

// ---- shading (SSFshading.f.glsl) ------------------------------------------------------
// Explicitly rounded in the float oracle's order: with the same depth, normal
// and thickness images the colours agree bit for bit except through expf
// (depth, thickness, full and tinted-refraction options).

// GL cube-map face selection and (s, t) (the major-axis table of the GL
// specification), then bilinear filtering clamped to the face's edge.
__device__ void sky_color(const SsfConsts& c, const float d[3], float out[3]) {
  if (c.sky_size <= 0) {
    out[0] = c.sky[0], out[1] = c.sky[1], out[2] = c.sky[2];
    return;
  }
  const float ax = fabsf(d[0]), ay = fabsf(d[1]), az = fabsf(d[2]);
  int face;
  float sc, tc, ma;
  if (ax >= ay && ax >= az) {
    face = d[0] >= 0.f ? 0 : 1, ma = ax;
    sc = d[0] >= 0.f ? -d[2] : d[2], tc = -d[1];
  } else if (ay >= az) {
    face = d[1] >= 0.f ? 2 : 3, ma = ay;
    sc = d[0], tc = d[1] >= 0.f ? d[2] : -d[2];
  } else {
    face = d[2] >= 0.f ? 4 : 5, ma = az;
    sc = d[2] >= 0.f ? d[0] : -d[0], tc = -d[1];
  }
  if (!(ma > 0.f) || !(ma < INFINITY)) {
    out[0] = c.sky[0], out[1] = c.sky[1], out[2] = c.sky[2];
    return;
  }
  const int S = c.sky_size;
  const float s = fm(0.5f, fa(fd(sc, ma), 1.f)), t = fm(0.5f, fa(fd(tc, ma), 1.f));
  const float u = fs(fm(s, (float)S), 0.5f), v = fs(fm(t, (float)S), 0.5f);
  const float fu = floorf(u), fv = floorf(v);
  const float a = fs(u, fu), b = fs(v, fv);
  const int i0 = min(max((int)fu, 0), S - 1), i1 = min(max((int)fu + 1, 0), S - 1);
  const int j0 = min(max((int)fv, 0), S - 1), j1 = min(max((int)fv + 1, 0), S - 1);
  const float4* F = c.sky_map + (size_t)face * S * S;
  const float4 t00 = F[(size_t)j0 * S + i0], t01 = F[(size_t)j0 * S + i1];
  const float4 t10 = F[(size_t)j1 * S + i0], t11 = F[(size_t)j1 * S + i1];
  const float w00 = fm(fs(1.f, a), fs(1.f, b)), w01 = fm(a, fs(1.f, b));
  const float w10 = fm(fs(1.f, a), b), w11 = fm(a, b);
  out[0] = fa(fa(fa(fm(w00, t00.x), fm(w01, t01.x)), fm(w10, t10.x)), fm(w11, t11.x));
  out[1] = fa(fa(fa(fm(w00, t00.y), fm(w01, t01.y)), fm(w10, t10.y)), fm(w11, t11.y));
  out[2] = fa(fa(fa(fm(w00, t00.z), fm(w01, t01.z)), fm(w10, t10.z)), fm(w11, t11.z));
}

// trace_color (SSFshading.f.glsl:50-72): a 10 x 10 checker floor at world z = 0,
// else the sky.
__device__ void trace_color(const SsfConsts& c, const float p[3], const float d[3], float out[3]) {
  const float* M = c.IV;
  float wp[3], wd[3], its[3];
  for (int r = 0; r < 3; ++r) {
    wp[r] = fa(fa(fa(fm(M[r], p[0]), fm(M[4 + r], p[1])), fm(M[8 + r], p[2])), M[12 + r]);
    wd[r] = fa(fa(fm(M[r], d[0]), fm(M[4 + r], d[1])), fm(M[8 + r], d[2]));
  }
  const float t = fd(-wp[2], wd[2]);
  for (int r = 0; r < 3; ++r) its[r] = fa(wp[r], fm(t, wd[r]));
  if (t > 0.f && fabsf(its[0]) < 5.f && fabsf(its[1]) < 5.f) {
    const float uvx = fd(fm(10.f, fs(its[0], -5.f)), 10.f), uvy = fd(fm(10.f, fs(its[1], -5.f)), 10.f);
    const float u = fs(uvx, floorf(uvx)), v = fs(uvy, floorf(uvy));  // mod(., 1)
    int flip = 1;
    if (u > 0.5f) flip = 1 - flip;
    if (v > 0.5f) flip = 1 - flip;
    out[0] = out[1] = out[2] = flip == 1 ? 0.8f : 0.6f;
    return;
  }
  sky_color(c, wd, out);
}

__global__ void __launch_bounds__(256) k_ssf_shade(SsfConsts c, const float* __restrict__ depth,
                                                   const float4* __restrict__ normal_D,
                                                   const float* __restrict__ thick, float4* __restrict__ color) {
  const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
  if (px >= c.W || py >= c.H) return;
  const size_t k = (size_t)py * c.W + px;
  const float ze = depth[k];
  // gl_FragDepth from ze against the cleared depth buffer: drawn iff ze < far
  if (!(ze < c.p_f)) return;
  const float u = fd(fa((float)px, 0.5f), (float)c.W), v = fd(fa((float)py, 0.5f), (float)c.H);
  const float4 nd = normal_D[k];
  const float n[3] = {nd.x, nd.y, nd.z};
  // getPos: right-handed eye position of the pixel's surface point
  const float p[3] = {fd(fm(fm(fs(fm(2.f, u), 1.f), c.p_r), ze), c.p_n),
                      fd(fm(fm(fs(fm(2.f, v), 1.f), c.p_t), ze), c.p_n), -ze};
  const float pl = __fsqrt_rn(fa(fa(fm(p[0], p[0]), fm(p[1], p[1])), fm(p[2], p[2])));
  const float e[3] = {fd(-p[0], pl), fd(-p[1], pl), fd(-p[2], pl)};  // normalize(-p)
  const float ne = fa(fa(fm(n[0], e[0]), fm(n[1], e[1])), fm(n[2], e[2]));
  float out[3];
  switch (c.shading) {
    case PBF_SSF_DEPTH: {
      if (ze > 50.f) return;
      const float ez = expf(ze);
      out[0] = out[1] = out[2] = fm(fs(fd(ez, fa(ez, 1.f)), 0.5f), 2.f);
      break;
    }
    case PBF_SSF_THICK: {
      if (ze > 50.f) return;
      const float et = expf(thick[k]);
      out[0] = out[1] = out[2] = fm(fs(fd(et, fa(et, 1.f)), 0.5f), 2.f);
      break;
    }
    case PBF_SSF_NORMAL:
      out[0] = n[0], out[1] = n[1], out[2] = n[2];
      break;
    case PBF_SSF_FRESNEL: {
      const float q = fs(1.f, ne);
      out[0] = out[1] = out[2] = fa(c.r0, fm(fs(1.f, c.r0), fm(q, q)));
      break;
    }
    default: {
      const float q = fs(1.f, ne);
      const float r = fa(c.r0, fm(fs(1.f, c.r0), fm(fm(q, q), q)));
      float refl[3], refr[3], cl[3], cr[3];
      for (int a = 0; a < 3; ++a) {
        refl[a] = fa(-e[a], fm(fm(2.f, ne), n[a]));
        refr[a] = fs(-e[a], fm(0.2f, n[a]));
      }
      if (c.shading == PBF_SSF_REFLECT) {
        trace_color(c, p, refl, out);
      } else if (c.shading == PBF_SSF_REFRACT) {
        trace_color(c, p, refr, out);
      } else {
        const float att = fmaxf(expf(fm(0.5f, -thick[k])), 0.2f);
        const float tint[3] = {6.f / 256.f, 105.f / 256.f, 217.f / 256.f};
        trace_color(c, p, refr, cr);
        for (int a = 0; a < 3; ++a) cr[a] = fa(fm(fs(1.f, att), tint[a]), fm(att, cr[a]));
        if (c.shading == PBF_SSF_REFRACT_TINTED) {
          for (int a = 0; a < 3; ++a) out[a] = cr[a];
        } else {
          trace_color(c, p, refl, cl);
          for (int a = 0; a < 3; ++a) out[a] = fa(fm(fs(1.f, r), cr[a]), fm(r, cl[a]));
        }
      }
    }
  }
  color[k] = make_float4(out[0], out[1], out[2], 1.f);
}

// ---- host side ------------------------------------------------------------------------

bool finite_all(const float* v, int k) {
  for (int i = 0; i < k; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

pbf_status check_ssf_params(const pbf_ssf_params* p) {
  if (!p) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf params is NULL");
  if (p->width < 1 || p->height < 1 || p->width > kMaxImageSide || p->height > kMaxImageSide)
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: width and height must be in 1..16384");
  if (!finite_all(p->view, 16) || !finite_all(p->proj, 16))
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: camera matrices must be finite");
  const float pos_vals[] = {p->p_n, p->p_f, p->p_t, p->p_r, p->radius, p->sigma_r, p->sigma_z};
  for (float v : pos_vals)
    if (!(v > 0.f) || !std::isfinite(v))
      return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: p_n, p_f, p_t, p_r, radius, sigma_r, sigma_z must be > 0");
  if (!(p->p_f > p->p_n)) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: p_f must exceed p_n");
  // thickness sums are 64-bit fixed point, 2 r 2^32 per fragment (pbf_ssf_render
  // also bounds n * radius, so that a pixel's sum stays below 2^63)
  if (!(p->radius <= 100.f)) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: radius must be <= 100");
  if (p->kernel_r < 0 || p->kernel_r > kMaxKernelR)
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: kernel_r must be in 0..20");
  if (p->smooth_niter < 0 || p->smooth_niter > kMaxSmoothIter)
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: smooth_niter must be in 0..64");
  if (p->blur_option != 0 && p->blur_option != 1)
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: blur_option must be 0 (bilateral) or 1 (gaussian)");
  if (p->shading_option < 0 || p->shading_option > 7)
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: shading_option must be in 0..7");
  if (!std::isfinite(p->r0) || !finite_all(p->sky, 3))
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf: r0 and sky must be finite");
  return PBF_OK;
}

// 4 x 4 inverse (cofactors, in double), column-major in and out.
bool invert4(const float* m, float* out) {
  double a[16], inv[16];
  for (int i = 0; i < 16; ++i) a[i] = m[i];
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
  if (!(det != 0.0) || !std::isfinite(det)) return false;
  for (int i = 0; i < 16; ++i) out[i] = (float)(inv[i] / det);
  return true;
}

}  // namespace

struct pbf_ssf {
  pbf_ssf_params p;
  float iview[16];
  uint32_t* zkey = nullptr;
  unsigned long long* tfx = nullptr;
  float* depth_a = nullptr;
  float* depth_b = nullptr;
  float* thick = nullptr;
  float4* normal_D = nullptr;
  float4* sky = nullptr;
  int sky_size = 0;
  unsigned long long* frag_count = nullptr;
  const float* final_depth = nullptr;  // the image shading read in the last render
  int profile = 0;
  bool have_events = false;
  bool events_recorded = false;
  cudaEvent_t ev[5] = {};
  int last_launches = 0;
};

namespace {

void ssf_free(pbf_ssf* s) {
  void* ptrs[] = {s->zkey, s->tfx, s->depth_a, s->depth_b, s->thick, s->normal_D, s->sky, s->frag_count};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (s->have_events)
    for (cudaEvent_t& e : s->ev)
      if (e) cudaEventDestroy(e);
}

SsfConsts consts_of(const pbf_ssf* s) {
  const pbf_ssf_params& p = s->p;
  SsfConsts c;
  c.W = p.width, c.H = p.height;
  std::memcpy(c.V, p.view, sizeof(c.V));
  std::memcpy(c.P, p.proj, sizeof(c.P));
  std::memcpy(c.IV, s->iview, sizeof(c.IV));
  c.p_n = p.p_n, c.p_f = p.p_f, c.p_t = p.p_t, c.p_r = p.p_r;
  c.r = p.radius;
  c.kernel_r = p.kernel_r;
  // loadParams: blur_r = 1 / sigma_r, blur_z = 1 / sigma_z (fluids/SSFRenderer.cpp:286-287)
  c.blur_r = 1.f / p.sigma_r;
  c.blur_z = 1.f / p.sigma_z;
  c.keep_edge = p.keep_edge, c.blur_option = p.blur_option, c.shading = p.shading_option;
  c.r0 = p.r0;
  for (int a = 0; a < 3; ++a) c.sky[a] = p.sky[a];
  c.sky_map = s->sky;
  c.sky_size = s->sky_size;
  return c;
}

}  // namespace

extern "C" {

void pbf_ssf_params_default(pbf_ssf_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->width = 1600;                      // WINDOW_WIDTH  (fluids/Renderer.h:12)
  p->height = 1200;                     // WINDOW_HEIGHT (fluids/Renderer.h:13)
  p->radius = 0.1f * 0.5f;              // setUnif("r", 0.1f * 0.5f) (fluids/SSFRenderer.cpp:180)
  p->smooth_niter = 2;                  // fluids/FluidSystem.cpp:26-32
  p->kernel_r = 10;
  p->sigma_r = 6.f;
  p->sigma_z = 0.1f;
  p->keep_edge = 1;
  p->blur_option = 0;
  p->shading_option = PBF_SSF_FULL;
  const float n1 = 1.3333f, t = (n1 - 1.f) / (n1 + 1.f);  // fluids/SSFRenderer.cpp:25-29
  p->r0 = t * t;
  p->sky[0] = 0.62f, p->sky[1] = 0.75f, p->sky[2] = 0.90f;
  const float pos[3] = {1.f, -5.f, 2.f}, focus[3] = {0.f, 0.f, 1.5f};  // fluids/FluidSystem.cpp:41
  pbf_ssf_look_at(p, pos, focus, 60.f);
}

pbf_status pbf_ssf_look_at(pbf_ssf_params* p, const float pos[3], const float focus[3], float fov_deg) {
  if (!p || !pos || !focus) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf look_at: NULL argument");
  if (p->width < 1 || p->height < 1) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf look_at: width/height < 1");
  if (!(fov_deg > 0.f && fov_deg < 180.f)) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf look_at: fov in (0, 180)");
  double e[3], f[3];
  for (int a = 0; a < 3; ++a) e[a] = pos[a], f[a] = (double)focus[a] - pos[a];
  auto cross = [](const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1], o[1] = a[2] * b[0] - a[0] * b[2], o[2] = a[0] * b[1] - a[1] * b[0];
  };
  auto norm = [](double* a) {
    const double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (!(l > 0.0)) return false;
    a[0] /= l, a[1] /= l, a[2] /= l;
    return true;
  };
  // Camera(pos, focus, aspect): up = cross(front, cross((0, 0, 1), front)), normalised
  const double zup[3] = {0.0, 0.0, 1.0};
  double t[3], up[3];
  cross(zup, f, t);
  cross(f, t, up);
  double fn[3] = {f[0], f[1], f[2]};
  if (!norm(up) || !norm(fn)) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf look_at: degenerate camera");
  // lookAt(eye, eye + front, up): s = f x up, u = s x f
  double s[3], u[3];
  cross(fn, up, s);
  if (!norm(s)) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf look_at: degenerate camera");
  cross(s, fn, u);
  float* V = p->view;
  std::memset(V, 0, sizeof(p->view));
  V[0] = (float)s[0], V[4] = (float)s[1], V[8] = (float)s[2];
  V[1] = (float)u[0], V[5] = (float)u[1], V[9] = (float)u[2];
  V[2] = (float)-fn[0], V[6] = (float)-fn[1], V[10] = (float)-fn[2];
  V[12] = (float)-(s[0] * e[0] + s[1] * e[1] + s[2] * e[2]);
  V[13] = (float)-(u[0] * e[0] + u[1] * e[1] + u[2] * e[2]);
  V[14] = (float)(fn[0] * e[0] + fn[1] * e[1] + fn[2] * e[2]);
  V[15] = 1.f;
  // perspective(radians(fov), aspect, 0.1, 100) and getProjectionInfo
  const double n = 0.1, fa_ = 100.0, aspect = (double)p->width / (double)p->height;
  const double th = std::tan(fov_deg * 3.14159265358979323846 / 180.0 * 0.5);
  float* P = p->proj;
  std::memset(P, 0, sizeof(p->proj));
  P[0] = (float)(1.0 / (aspect * th));
  P[5] = (float)(1.0 / th);
  P[10] = (float)(-(fa_ + n) / (fa_ - n));
  P[11] = -1.f;
  P[14] = (float)(-(2.0 * fa_ * n) / (fa_ - n));
  p->p_n = (float)n;
  p->p_f = (float)fa_;
  p->p_t = (float)(th * n);
  p->p_r = (float)(aspect * th * n);
  return PBF_OK;
}

pbf_status pbf_ssf_create(const pbf_ssf_params* p, pbf_ssf** out) {
  if (!out) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf create: out is NULL");
  *out = nullptr;
  pbf_status st = check_ssf_params(p);
  if (st != PBF_OK) return st;
  pbf_ssf* s = new (std::nothrow) pbf_ssf();
  if (!s) return pbf::set_error(PBF_ERR_CAPACITY, "ssf create: out of host memory");
  s->p = *p;
  if (!invert4(p->view, s->iview)) {
    delete s;
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf create: view matrix is singular");
  }
  const size_t npix = (size_t)p->width * p->height;
  cudaError_t e = cudaMalloc(&s->zkey, 4 * npix);
  if (e == cudaSuccess) e = cudaMalloc(&s->tfx, 8 * npix);
  if (e == cudaSuccess) e = cudaMalloc(&s->depth_a, 4 * npix);
  if (e == cudaSuccess) e = cudaMalloc(&s->depth_b, 4 * npix);
  if (e == cudaSuccess) e = cudaMalloc(&s->thick, 4 * npix);
  if (e == cudaSuccess) e = cudaMalloc(&s->normal_D, 16 * npix);
  if (e == cudaSuccess) e = cudaMalloc(&s->frag_count, 8);
  if (e == cudaSuccess) e = cudaMemset(s->frag_count, 0, 8);
  for (int k = 0; e == cudaSuccess && k < 5; ++k) e = cudaEventCreate(&s->ev[k]);
  if (e == cudaSuccess) s->have_events = true;
  if (e != cudaSuccess) {
    ssf_free(s);
    delete s;
    return pbf::set_cuda_error(e, "ssf create");
  }
  *out = s;
  return PBF_OK;
}

void pbf_ssf_destroy(pbf_ssf* s) {
  if (!s) return;
  ssf_free(s);
  delete s;
}

pbf_status pbf_ssf_set_params(pbf_ssf* s, const pbf_ssf_params* p) {
  if (!s) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf is NULL");
  pbf_status st = check_ssf_params(p);
  if (st != PBF_OK) return st;
  if (p->width != s->p.width || p->height != s->p.height)
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf set_params: width and height are fixed at create");
  float iv[16];
  if (!invert4(p->view, iv)) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf set_params: view matrix is singular");
  s->p = *p;
  std::memcpy(s->iview, iv, sizeof(iv));
  return PBF_OK;
}

pbf_status pbf_ssf_get_params(const pbf_ssf* s, pbf_ssf_params* p) {
  if (!s || !p) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf get_params: NULL argument");
  *p = s->p;
  return PBF_OK;
}

pbf_status pbf_ssf_set_sky(pbf_ssf* s, const float* faces, int size) {
  if (!s) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf is NULL");
  if (size < 0 || size > 4096) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf set_sky: size must be in 0..4096");
  if (s->sky) {
    cudaError_t e = cudaFree(s->sky);
    s->sky = nullptr;
    s->sky_size = 0;
    if (e != cudaSuccess) return pbf::set_cuda_error(e, "ssf set_sky: free");
  }
  if (!faces || size == 0) return PBF_OK;
  const size_t texels = (size_t)6 * size * size;
  float4* host = new (std::nothrow) float4[texels];
  if (!host) return pbf::set_error(PBF_ERR_CAPACITY, "ssf set_sky: out of host memory");
  for (size_t k = 0; k < texels; ++k) {
    host[k] = make_float4(faces[3 * k], faces[3 * k + 1], faces[3 * k + 2], 0.f);
    if (!std::isfinite(host[k].x) || !std::isfinite(host[k].y) || !std::isfinite(host[k].z)) {
      delete[] host;
      return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf set_sky: non-finite texel");
    }
  }
  cudaError_t e = cudaMalloc(&s->sky, sizeof(float4) * texels);
  if (e == cudaSuccess) e = cudaMemcpy(s->sky, host, sizeof(float4) * texels, cudaMemcpyHostToDevice);
  delete[] host;
  if (e != cudaSuccess) {
    if (s->sky) cudaFree(s->sky);
    s->sky = nullptr;
    return pbf::set_cuda_error(e, "ssf set_sky");
  }
  s->sky_size = size;
  return PBF_OK;
}

pbf_status pbf_ssf_render(pbf_ssf* s, const void* pos, int n, void* color, void* stream) {
  const pbf::NvtxRange range("pbf_ssf_render");
  if (!s) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf is NULL");
  if (n < 0) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf render: n < 0");
  if (n > 0 && !pos) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf render: pos is NULL");
  // a pixel's thickness sum is at most n fragments of 2 r 2^32 each: below 2^63
  if ((double)n * s->p.radius >= 1073741824.0)
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf render: n * radius must stay below 2^30");
  if (((uintptr_t)pos & 15u) || ((uintptr_t)color & 15u))
    return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf render: pos and color must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  const SsfConsts c = consts_of(s);
  const int npix = c.W * c.H;
  const bool prof = s->profile != 0;
  int launches = 0;
  cudaError_t e = cudaSuccess;
  if (prof) {
    e = cudaMemsetAsync(s->frag_count, 0, 8, st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[0], st);
  }
  // 1-2. depth and thickness splats, resolved into depth_a / depth_b / thick
  if (e == cudaSuccess) {
    k_ssf_clear<<<(npix + 255) / 256, 256, 0, st>>>(npix, s->zkey, s->tfx);
    ++launches;
    if (n > 0) {
      k_ssf_splat<<<(int)(((long long)n + 255) / 256), 256, 0, st>>>(c, (const float4*)pos, n, s->zkey, s->tfx,
                                                   prof ? s->frag_count : nullptr);
      ++launches;
    }
    k_ssf_resolve<<<(npix + 255) / 256, 256, 0, st>>>(npix, s->zkey, s->tfx, s->depth_a, s->depth_b, s->thick);
    ++launches;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && prof) e = cudaEventRecord(s->ev[1], st);
  // 3. smoothing: pass k reads a and writes b for odd k, the reverse for even k
  //    (the m_ab ping-pong, fluids/SSFRenderer.cpp:130-137, 407-408)
  const float* final_depth = s->depth_a;
  if (e == cudaSuccess) {
    const dim3 grid((c.W + kSmoothTileW - 1) / kSmoothTileW, (c.H + kSmoothTileH - 1) / kSmoothTileH);
    const dim3 block(kSmoothTileW, kSmoothThreadsY);
    for (int it = 1; it <= s->p.smooth_niter; ++it) {
      const float* src = (it & 1) ? s->depth_a : s->depth_b;
      float* dst = (it & 1) ? s->depth_b : s->depth_a;
      k_ssf_smooth<<<grid, block, 0, st>>>(c, src, dst);
      ++launches;
      final_depth = dst;
    }
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && prof) e = cudaEventRecord(s->ev[2], st);
  // 4. normals
  const dim3 pgrid((c.W + 255) / 256, c.H);
  if (e == cudaSuccess) {
    k_ssf_normal<<<pgrid, 256, 0, st>>>(c, final_depth, s->normal_D);
    ++launches;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && prof) e = cudaEventRecord(s->ev[3], st);
  // 5. shading
  if (e == cudaSuccess && color) {
    k_ssf_shade<<<pgrid, 256, 0, st>>>(c, final_depth, s->normal_D, s->thick, (float4*)color);
    ++launches;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && prof) e = cudaEventRecord(s->ev[4], st);
  if (e != cudaSuccess) return pbf::set_cuda_error(e, "ssf render");
  s->final_depth = final_depth;
  s->last_launches = launches;
  s->events_recorded = prof;
  return PBF_OK;
}

pbf_status pbf_ssf_images(pbf_ssf* s, void* depth, void* thick, void* normal_D, void* stream) {
  if (!s) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf is NULL");
  if (!s->final_depth) return pbf::set_error(PBF_ERR_NOT_READY, "ssf images: nothing rendered yet");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t npix = (size_t)s->p.width * s->p.height;
  cudaError_t e = cudaSuccess;
  if (depth) e = cudaMemcpyAsync(depth, s->final_depth, 4 * npix, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && thick) e = cudaMemcpyAsync(thick, s->thick, 4 * npix, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && normal_D)
    e = cudaMemcpyAsync(normal_D, s->normal_D, 16 * npix, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return pbf::set_cuda_error(e, "ssf images");
  return PBF_OK;
}

pbf_status pbf_ssf_profile_enable(pbf_ssf* s, int on) {
  if (!s) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf is NULL");
  s->profile = on != 0;
  if (!s->profile) s->events_recorded = false;
  return PBF_OK;
}

pbf_status pbf_ssf_profile_read(pbf_ssf* s, pbf_ssf_profile* out) {
  if (!s || !out) return pbf::set_error(PBF_ERR_INVALID_ARG, "ssf profile_read: NULL argument");
  if (!s->events_recorded) return pbf::set_error(PBF_ERR_NOT_READY, "ssf profile_read: no profiled render");
  cudaError_t e = cudaEventSynchronize(s->ev[4]);
  float ms[4] = {};
  for (int k = 0; e == cudaSuccess && k < 4; ++k) e = cudaEventElapsedTime(&ms[k], s->ev[k], s->ev[k + 1]);
  unsigned long long frags = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&frags, s->frag_count, 8, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return pbf::set_cuda_error(e, "ssf profile_read");
  out->splat_ms = ms[0];
  out->smooth_ms = ms[1];
  out->normal_ms = ms[2];
  out->shade_ms = ms[3];
  out->total_ms = ms[0] + ms[1] + ms[2] + ms[3];
  out->launches = s->last_launches;
  out->fragments = (long long)frags;
  return PBF_OK;
}

}  // extern "C"
