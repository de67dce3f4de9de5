/*
 * pbf_ssf.h — C ABI of the screen-space fluid (SSF) surface pipeline.
 *
 * Replaces the reference's OpenGL `SSFRenderer` (fluids/SSFRenderer.cpp:113-146
 * and the shaders under fluids/shader/SSF*.glsl) with CUDA kernels that write
 * into headless device images: no window, no GL context, no interop.  The
 * stages and their arithmetic are the reference's, per pixel:
 *
 *   1. depth splat   every particle is a sphere sprite; a pixel keeps the
 *                    smallest eye depth of the sphere fronts covering it
 *                    (SSFget_depth.v.glsl:15-24, SSFget_depth.f.glsl:19-37,
 *                    SSFRenderer.cpp:148-194);
 *   2. thickness     the sum over covering sprites of 2 r z (additive blend,
 *                    SSFget_thick.f.glsl:14-26, SSFRenderer.cpp:196-238);
 *   3. smoothing     smooth_niter bilateral (or gaussian) passes over the
 *                    depth, ping-pong (SSFsmooth_depth.f.glsl:26-75,
 *                    SSFRenderer.cpp:130-137, 325-358);
 *   4. normals       normal and its length from depth differences
 *                    (SSFrestore_normal.f.glsl:31-58);
 *   5. shading       one of the reference's eight shading options, Fresnel by
 *                    default (SSFshading.f.glsl:26-184).
 *
 * Images are row-major, W x H, row 0 at the bottom (OpenGL window
 * coordinates): pixel (x, y) is element y * W + x.  Depth and thickness are
 * float, normals float4 (nx, ny, nz, length), colour float4 RGBA.
 *
 * Where the reference depends on GL implementation details, this pipeline
 * fixes one exact rule (each is the exact-arithmetic reading of the GL rule):
 *  - depth test: the smallest eye depth wins (GL compares a fixed-point depth
 *    buffer, so near-equal fragments may resolve to either there);
 *  - thickness: summed in 64-bit fixed point, 2^-32 per unit, so the sum does
 *    not depend on the order fragments arrive in (GL's blend order is
 *    unspecified);
 *  - a sprite covers the pixels whose centres lie in the half-open square of
 *    side gl_PointSize (at least 1) around the projected centre; a particle
 *    whose centre is outside the clip volume is not drawn (GL point clipping);
 *  - smoothing reads 0 outside the image (texelFetch out of range);
 *  - normals wrap around the image edges (the texture's default REPEAT mode);
 *  - shading writes a pixel only where the smoothed depth is below the far
 *    plane (the depth test against a cleared depth buffer); the rest of the
 *    colour image keeps what the caller put there.
 */
#ifndef PBF_SSF_H_
#define PBF_SSF_H_

#include "pbf.h"

#ifdef __cplusplus
extern "C" {
#endif

/* GUIParams::ShadeOption (fluids/GUIParams.h:27-36) */
typedef enum pbf_ssf_shading {
  PBF_SSF_FULL = 0,          /* Fresnel mix of tinted refraction and reflection */
  PBF_SSF_DEPTH = 1,         /* depth as grey */
  PBF_SSF_THICK = 2,         /* thickness as grey */
  PBF_SSF_NORMAL = 3,        /* the normal */
  PBF_SSF_FRESNEL = 4,       /* the Fresnel factor (square law) */
  PBF_SSF_REFLECT = 5,       /* reflected colour */
  PBF_SSF_REFRACT = 6,       /* refracted colour */
  PBF_SSF_REFRACT_TINTED = 7 /* refracted colour, tinted by thickness */
} pbf_ssf_shading;

/*
 * Renderer parameters.  Camera matrices are column-major (element [c * 4 + r]
 * is column c, row r), as glm and OpenGL store them.  The defaults are the
 * reference's: its camera (fluids/FluidSystem.cpp:41, fluids/Camera.cpp:64-96,
 * 151-162), window (fluids/Renderer.h:12-13), sprite radius
 * (fluids/SSFRenderer.cpp:180), filter settings (fluids/FluidSystem.cpp:26-32)
 * and Schlick reflectance (fluids/SSFRenderer.cpp:25-29).
 */
typedef struct pbf_ssf_params {
  int width, height;      /* image size in pixels */
  float view[16];         /* world -> eye (glm::lookAt) */
  float proj[16];         /* eye -> clip (glm::perspective) */
  float p_n, p_f;         /* near / far plane distances   ProjectionInfo::n, f */
  float p_t, p_r;         /* near-plane half height / width ProjectionInfo::t, r */
  float radius;           /* sprite radius r, 0 < r <= 100 (reference: 0.1 * 0.5) */
  int smooth_niter;       /* smoothing passes                GUIParams::smooth_niter */
  int kernel_r;           /* filter radius in pixels, 0..20  GUIParams::kernel_r */
  float sigma_r;          /* spatial scale (blur_r = 1 / sigma_r)  GUIParams::sigma_r */
  float sigma_z;          /* depth scale (blur_z = 1 / sigma_z)    GUIParams::sigma_z */
  int keep_edge;          /* one-sided differences at silhouettes  GUIParams::keep_edge */
  int blur_option;        /* 0 bilateral, 1 gaussian              GUIParams::blur_option */
  int shading_option;     /* pbf_ssf_shading                      GUIParams::shading_option */
  float r0;               /* Schlick reflectance at normal incidence */
  float sky[3];           /* sky colour used when no cube map is set */
} pbf_ssf_params;

/* Phase times of the last render (pbf_ssf_profile_enable). */
typedef struct pbf_ssf_profile {
  float splat_ms;         /* clear, depth and thickness splat, resolve */
  float smooth_ms;        /* every smoothing pass */
  float normal_ms;
  float shade_ms;
  float total_ms;
  int launches;           /* kernels launched by the last render */
  long long fragments;    /* sprite pixels that passed the circle test (0 unless profiling) */
} pbf_ssf_profile;

typedef struct pbf_ssf pbf_ssf;

/* The reference's renderer settings with its default camera at 1600 x 1200. */
void pbf_ssf_params_default(pbf_ssf_params* p);

/*
 * Camera(pos, focus, aspect) (fluids/Camera.cpp:64-80) and Camera::use /
 * getProjectionInfo (fluids/Camera.cpp:87-96, 151-162): world up (0, 0, 1)
 * made orthogonal to the view direction, vertical field of view fov_deg
 * (reference: 60), aspect width / height, near 0.1, far 100.  Fills view,
 * proj, p_n, p_f, p_t and p_r of *p from its width and height.
 */
pbf_status pbf_ssf_look_at(pbf_ssf_params* p, const float pos[3], const float focus[3], float fov_deg);

/* SSFRenderer(camera, width, height, sky) (fluids/SSFRenderer.cpp:22-106):
 * allocates the device images for p->width x p->height. */
pbf_status pbf_ssf_create(const pbf_ssf_params* p, pbf_ssf** out);
void pbf_ssf_destroy(pbf_ssf* s);

/* loadParams (fluids/SSFRenderer.cpp:280-288) and the camera: new settings for
 * the next render; width and height must stay those of pbf_ssf_create. */
pbf_status pbf_ssf_set_params(pbf_ssf* s, const pbf_ssf_params* p);
pbf_status pbf_ssf_get_params(const pbf_ssf* s, pbf_ssf_params* p);

/*
 * The sky cube map sampled by trace_color (SSFshading.f.glsl:50-72; the
 * reference loads six images, fluids/Renderer.cpp:445-472): host RGB floats
 * [6][size][size][3], faces in GL order +x, -x, +y, -y, +z, -z, each face's
 * row 0 at t = 0; sampled bilinearly, clamped to each face's edge.  NULL (or
 * size 0) returns to the uniform colour p->sky.
 */
pbf_status pbf_ssf_set_sky(pbf_ssf* s, const float* faces, int size);

/*
 * SSFRenderer::render (fluids/SSFRenderer.cpp:113-146): n particles at device
 * positions pos (float4, xyz used) through the five stages on `stream`
 * (asynchronous).  color: device float4[width * height], written where the
 * fluid is drawn; may be NULL (the intermediate images are still made).
 * PBF_ERR_INVALID_ARG if n * radius >= 2^30 (the 64-bit fixed-point
 * thickness sum of a pixel covered by every sprite would overflow).
 */
pbf_status pbf_ssf_render(pbf_ssf* s, const void* pos, int n, void* color, void* stream);

/* Copies of the last render's images into caller device buffers (each may be
 * NULL): the smoothed depth that shading reads, thickness, normal_D. */
pbf_status pbf_ssf_images(pbf_ssf* s, void* depth, void* thick, void* normal_D, void* stream);

/* Phase times with CUDA events (on: 1); pbf_ssf_profile_read waits for the
 * last render's events. */
pbf_status pbf_ssf_profile_enable(pbf_ssf* s, int on);
pbf_status pbf_ssf_profile_read(pbf_ssf* s, pbf_ssf_profile* out);

#ifdef __cplusplus
}
#endif

#endif /* PBF_SSF_H_ */
