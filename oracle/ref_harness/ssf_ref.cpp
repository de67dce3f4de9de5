// ssf_ref.cpp — runs the reference's SSF shaders (fluids/shader/SSF*.glsl,
// compiled as C++ through ssf_glsl.hpp; build_ref.py generates ssf_shaders.inc
// from them into oracle/_ref/) on the CPU, with the fixed-function OpenGL
// steps SSFRenderer relies on (fluids/SSFRenderer.cpp:148-358) made explicit.
//
// TEST INFRASTRUCTURE, NOT PRODUCT CODE: the reference side that pins
// oracle/ssf_oracle.c (tests/test_ssf_ref.py, tests/golden/make_ssf_golden.py).
//
// Fixed-function steps, by the rules include/pbf_ssf.h states:
//   points: clipped by their centre, window coordinates by the viewport
//     transform, size gl_PointSize (at least 1), pixel centres in the half-open
//     square, gl_PointCoord = (1/2 + (x_f + 1/2 - x_w) / size, 1/2 - (y_f + 1/2 - y_w) / size);
//   depth pass: GL_LESS on gl_FragDepth (clamped to [0, 1]) against a buffer
//     cleared to 1, the colour target d_depth_a cleared to 100;
//   thickness pass: additive blending into a target cleared to 0, in draw order;
//   full-screen passes: texCoord = pixel centre / size, gl_FragCoord = pixel centre;
//   shading: drawn where gl_FragDepth (clamped) is below the cleared 1.
// Uniforms are set as SSFRenderer sets them (renderDepth, renderThick,
// smoothDepth, restoreNormal, shading, loadParams).
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/pbf_ssf.h"
#include "ssf_glsl.hpp"
#include "ssf_shaders.inc"  // generated: namespaces ref_depth_v, ref_depth_f, ref_thick_v,
                            // ref_thick_f, ref_smooth_f, ref_normal_f, ref_shading_f

namespace {

glsl::mat4 mat(const float* m) {
  glsl::mat4 a;
  std::memcpy(a.m, m, sizeof(a.m));
  return a;
}

bool invert4(const float* mf, float* out) {
  double a[16], inv[16];
  for (int i = 0; i < 16; ++i) a[i] = mf[i];
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

// One point through a vertex shader: its window square, or false when clipped.
struct Point {
  float xw, yw, size;
  int x0, x1, y0, y1;
};

bool rasterise_point(int W, int H, Point& pt) {
  const glsl::vec4 c = glsl::gl_Position;
  if (!(c.w > 0.f) || !std::isfinite(c.w)) return false;
  if (!(-c.w <= c.x && c.x <= c.w && -c.w <= c.y && c.y <= c.w && -c.w <= c.z && c.z <= c.w)) return false;
  const float hw = 0.5f * (float)W, hh = 0.5f * (float)H;
  pt.xw = hw * (c.x / c.w) + hw;
  pt.yw = hh * (c.y / c.w) + hh;
  if (!(glsl::gl_PointSize < INFINITY)) return false;
  pt.size = std::fmax(glsl::gl_PointSize, 1.f);
  const float lox = pt.xw - 0.5f * pt.size, loy = pt.yw - 0.5f * pt.size;
  pt.x0 = (int)std::fmax(std::ceil(lox - 0.5f), 0.f);
  pt.x1 = (int)std::fmin(std::ceil(lox + pt.size - 0.5f) - 1.f, (float)(W - 1));
  pt.y0 = (int)std::fmax(std::ceil(loy - 0.5f), 0.f);
  pt.y1 = (int)std::fmin(std::ceil(loy + pt.size - 0.5f) - 1.f, (float)(H - 1));
  return pt.x0 <= pt.x1 && pt.y0 <= pt.y1;
}

void point_coord(const Point& pt, int px, int py) {
  glsl::gl_PointCoord = glsl::vec2(0.5f + ((float)px + 0.5f - pt.xw) / pt.size,
                                   0.5f - ((float)py + 0.5f - pt.yw) / pt.size);
}

}  // namespace

extern "C" {

// renderDepth + renderThick (fluids/SSFRenderer.cpp:148-238): depth (the
// colour target d_depth_a, cleared to 100) and thickness (cleared to 0).
// Returns the depth pass's fragments that were not discarded.
long long ssf_ref_splat(const pbf_ssf_params* p, const float* pos, int n, float* depth, float* thick) {
  const int W = p->width, H = p->height;
  const size_t npix = (size_t)W * H;
  std::vector<float> zbuf(npix, 1.f);
  for (size_t k = 0; k < npix; ++k) depth[k] = 100.f, thick[k] = 0.f;
  long long frags = 0;
  // renderDepth's uniforms (camera->use: view, proj; s_h, p_t, p_n, p_f, r)
  ref_depth_v::view = mat(p->view), ref_depth_v::proj = mat(p->proj);
  ref_depth_v::s_h = H, ref_depth_v::p_t = p->p_t, ref_depth_v::p_n = p->p_n, ref_depth_v::r = p->radius;
  ref_depth_f::proj = mat(p->proj), ref_depth_f::p_n = p->p_n, ref_depth_f::p_f = p->p_f, ref_depth_f::r = p->radius;
  for (int i = 0; i < n; ++i) {
    ref_depth_v::aPos = glsl::vec3(pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]);
    ref_depth_v::shader_main();
    Point pt;
    if (!rasterise_point(W, H, pt)) continue;
    ref_depth_f::viewPos = ref_depth_v::viewPos, ref_depth_f::projPos = ref_depth_v::projPos;
    for (int py = pt.y0; py <= pt.y1; ++py)
      for (int px = pt.x0; px <= pt.x1; ++px) {
        point_coord(pt, px, py);
        glsl::gl_discarded = false;
        ref_depth_f::shader_main();
        if (glsl::gl_discarded) continue;
        ++frags;
        const float d = std::fmin(std::fmax(glsl::gl_FragDepth, 0.f), 1.f);
        const size_t k = (size_t)py * W + px;
        if (d < zbuf[k]) {
          zbuf[k] = d;
          depth[k] = ref_depth_f::FragColor.x;
        }
      }
  }
  // renderThick: the same uniforms, no depth test, GL_ONE / GL_ONE blending
  ref_thick_v::view = mat(p->view), ref_thick_v::proj = mat(p->proj);
  ref_thick_v::s_h = H, ref_thick_v::p_t = p->p_t, ref_thick_v::p_n = p->p_n, ref_thick_v::r = p->radius;
  ref_thick_f::proj = mat(p->proj), ref_thick_f::p_n = p->p_n, ref_thick_f::p_f = p->p_f, ref_thick_f::r = p->radius;
  for (int i = 0; i < n; ++i) {
    ref_thick_v::aPos = glsl::vec3(pos[4 * i], pos[4 * i + 1], pos[4 * i + 2]);
    ref_thick_v::shader_main();
    Point pt;
    if (!rasterise_point(W, H, pt)) continue;
    ref_thick_f::viewPos = ref_thick_v::viewPos, ref_thick_f::projPos = ref_thick_v::projPos;
    for (int py = pt.y0; py <= pt.y1; ++py)
      for (int px = pt.x0; px <= pt.x1; ++px) {
        point_coord(pt, px, py);
        glsl::gl_discarded = false;
        ref_thick_f::shader_main();
        if (glsl::gl_discarded) continue;
        thick[(size_t)py * W + px] += ref_thick_f::thickness;
      }
  }
  return frags;
}

// smooth_niter smoothDepth passes (fluids/SSFRenderer.cpp:130-137, 325-358)
// from the splatted depth: the m_ab ping-pong, d_depth_b cleared to 100.
int ssf_ref_smooth(const pbf_ssf_params* p, const float* raw, float* out) {
  const int W = p->width, H = p->height;
  const size_t npix = (size_t)W * H;
  std::vector<float> a(raw, raw + npix), b(npix, 100.f);
  ref_smooth_f::p_f = p->p_f, ref_smooth_f::p_n = p->p_n, ref_smooth_f::s_w = W, ref_smooth_f::s_h = H;
  ref_smooth_f::blur_option = p->blur_option, ref_smooth_f::kernel_r = p->kernel_r;
  ref_smooth_f::blur_r = 1.f / p->sigma_r, ref_smooth_f::blur_z = 1.f / p->sigma_z;  // loadParams
  const float* fin = a.data();
  for (int it = 1; it <= p->smooth_niter; ++it) {
    std::vector<float>& src = (it & 1) ? a : b;
    std::vector<float>& dst = (it & 1) ? b : a;
    ref_smooth_f::zA = glsl::sampler2D{src.data(), W, H, 1, false};
    ref_smooth_f::zB = glsl::image2D{dst.data(), W, H};
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        glsl::gl_FragCoord = glsl::vec4((float)x + 0.5f, (float)y + 0.5f, 0.f, 1.f);
        ref_smooth_f::shader_main();
      }
    fin = dst.data();
  }
  std::memcpy(out, fin, sizeof(float) * npix);
  return 0;
}

// restoreNormal (fluids/SSFRenderer.cpp:290-323) of a depth image.
int ssf_ref_normals(const pbf_ssf_params* p, const float* depth, float* normal_D) {
  const int W = p->width, H = p->height;
  ref_normal_f::p_n = p->p_n, ref_normal_f::p_f = p->p_f, ref_normal_f::p_t = p->p_t, ref_normal_f::p_r = p->p_r;
  ref_normal_f::s_w = (float)W, ref_normal_f::s_h = (float)H, ref_normal_f::keep_edge = p->keep_edge;
  ref_normal_f::zTex = glsl::sampler2D{depth, W, H, 1, false};
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      ref_normal_f::texCoord = glsl::vec2(((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H);
      ref_normal_f::shader_main();
      float* o = normal_D + 4 * ((size_t)y * W + x);
      o[0] = ref_normal_f::normal_D.x, o[1] = ref_normal_f::normal_D.y;
      o[2] = ref_normal_f::normal_D.z, o[3] = ref_normal_f::normal_D.w;
    }
  return 0;
}

// shading (fluids/SSFRenderer.cpp:240-278) of the depth, normal_D and
// thickness images into color (drawn where the depth test passes).
int ssf_ref_shade(const pbf_ssf_params* p, const float* depth, const float* normal_D, const float* thick,
                  const float* sky, int sky_size, float* color) {
  const int W = p->width, H = p->height;
  float iv[16];
  if (!invert4(p->view, iv)) return -1;
  ref_shading_f::iview = mat(iv);
  ref_shading_f::p_n = p->p_n, ref_shading_f::p_f = p->p_f, ref_shading_f::p_t = p->p_t, ref_shading_f::p_r = p->p_r;
  ref_shading_f::r0 = p->r0, ref_shading_f::shading_option = p->shading_option;
  ref_shading_f::zTex = glsl::sampler2D{depth, W, H, 1, false};
  ref_shading_f::normalDTex = glsl::sampler2D{normal_D, W, H, 4, false};
  ref_shading_f::thickTex = glsl::sampler2D{thick, W, H, 1, true};
  ref_shading_f::skyTex = glsl::samplerCube{sky, sky ? sky_size : 0, glsl::vec3(p->sky[0], p->sky[1], p->sky[2])};
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      ref_shading_f::texCoord = glsl::vec2(((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H);
      glsl::gl_discarded = false;
      ref_shading_f::shader_main();
      if (glsl::gl_discarded) continue;
      if (!(std::fmin(std::fmax(glsl::gl_FragDepth, 0.f), 1.f) < 1.f)) continue;
      float* o = color + 4 * ((size_t)y * W + x);
      o[0] = ref_shading_f::FragColor.x, o[1] = ref_shading_f::FragColor.y;
      o[2] = ref_shading_f::FragColor.z, o[3] = ref_shading_f::FragColor.w;
    }
  return 0;
}

}  // extern "C"
