"""CPU tests of the SSF oracle (oracle/ssf_oracle.c) and the renderer's C ABI
(include/pbf_ssf.h) without a GPU.

The reference renders with OpenGL (fluids/SSFRenderer.cpp, fluids/shader/SSF*),
which cannot run here, so the oracle is pinned by known answers of the shader
formulas: a sphere sprite straight ahead of an identity camera has its nearest
depth D - r sqrt(1 - 2 / size^2) at the pixel next to its centre and thickness
2 r sqrt(...) there, covers about pi (size / 2)^2 pixels, its centre normal is
+z and its Fresnel factor r0; the refracted ray of that pixel misses the floor
and returns the sky.  The float and FP64 oracles agree away from sprite rims.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "pbf_ssf.h"


def identity_camera(p):
    for i in range(16):
        p.view[i] = 1.0 if i % 5 == 0 else 0.0
    return p


def small_params(pbf, w=160, h=120, **kw):
    p = pbf.ssf_default_params(w, h)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def sprite_size(p, depth):
    return p.radius * p.p_n * p.height / (depth * p.p_t)


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?[\s\*])(pbf_ssf_\w+)\s*\(", text, flags=re.M)


def test_header_declares_exported_list(pbf):
    assert declared_functions() == list(pbf.EXPORTED_SSF)
    L = pbf.lib()
    for name in declared_functions():
        assert hasattr(L, name), name


def test_ssf_params_layout_matches_c(pbf, tmp_path):
    import subprocess
    import textwrap

    fields = [f for f, _ in pbf.PbfSsfParams._fields_]
    src = tmp_path / "layout.c"
    src.write_text(textwrap.dedent(f"""
        #include <stdio.h>
        #include <stddef.h>
        #include "{HEADER}"
        int main(void) {{
          printf("%zu\\n", sizeof(pbf_ssf_params));
          {''.join(f'printf("%zu\\n", offsetof(pbf_ssf_params, {f}));' for f in fields)}
          printf("%zu\\n", sizeof(pbf_ssf_profile));
          return 0;
        }}
    """))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(pbf.PbfSsfParams)
    for f, off in zip(fields, vals[1:-1]):
        assert getattr(pbf.PbfSsfParams, f).offset == off, f
    assert vals[-1] == ctypes.sizeof(pbf.PbfSsfProfile)


def test_defaults_are_the_reference_settings(pbf):
    """fluids/FluidSystem.cpp:26-32, 41; fluids/Renderer.h:12-13; fluids/SSFRenderer.cpp:25-29, 180;
    fluids/Camera.cpp:151-162."""
    p = pbf.ssf_default_params()
    f = ctypes.c_float
    assert (p.width, p.height) == (1600, 1200)
    assert p.radius == f(0.1 * 0.5).value
    assert (p.smooth_niter, p.kernel_r, p.keep_edge, p.blur_option, p.shading_option) == (2, 10, 1, 0, 0)
    assert p.sigma_r == 6.0 and p.sigma_z == f(0.1).value
    t = (f(1.3333).value - 1) / (f(1.3333).value + 1)
    assert abs(p.r0 - t * t) < 1e-7
    assert p.p_n == f(0.1).value and p.p_f == 100.0
    assert abs(p.p_t - np.tan(np.radians(30)) * 0.1) < 1e-8
    assert abs(p.p_r - 4 / 3 * p.p_t) < 1e-8
    # the camera at (1, -5, 2) looks at (0, 0, 1.5): the focus maps onto the eye's -z axis
    V = np.array(p.view, np.float64).reshape(4, 4).T
    e = V @ np.array([0, 0, 1.5, 1.0])
    assert abs(e[0]) < 1e-6 and abs(e[1]) < 1e-6 and abs(-e[2] - np.sqrt(1 + 25 + 0.25)) < 1e-5
    P = np.array(p.proj, np.float64).reshape(4, 4).T
    c = P @ np.array([0, 0, -p.p_n, 1.0])
    assert abs(c[2] / c[3] + 1) < 1e-6  # near plane -> ndc -1


def test_argument_errors_need_no_gpu(pbf):
    L = pbf.lib()
    h = ctypes.c_void_p()
    assert L.pbf_ssf_create(None, ctypes.byref(h)) == pbf.PBF_ERR_INVALID_ARG
    for field, bad in (("width", 0), ("kernel_r", 21), ("smooth_niter", -1), ("blur_option", 2),
                       ("shading_option", 8), ("radius", 0.0), ("sigma_z", 0.0), ("p_f", 0.05)):
        p = pbf.ssf_default_params(64, 48)
        setattr(p, field, bad)
        assert L.pbf_ssf_create(ctypes.byref(p), ctypes.byref(h)) == pbf.PBF_ERR_INVALID_ARG, field
    p = pbf.ssf_default_params(64, 48)
    p.view[0] = float("nan")
    assert L.pbf_ssf_create(ctypes.byref(p), ctypes.byref(h)) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_ssf_render(None, None, 0, None, None) == pbf.PBF_ERR_INVALID_ARG


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_single_sprite_known_answers(pbf, oracle, prec):
    p = identity_camera(small_params(pbf))
    D = 2.0
    o = oracle.ssf_render(p, np.array([[0, 0, -D, 0]], np.float32), prec=prec)
    size = sprite_size(p, D)
    cov = o["depth_raw"] < 100
    # pixels next to the centre are half a pixel off it on both axes
    zc = np.sqrt(1 - 2 / size ** 2)
    assert abs(o["depth_raw"].min() - (D - p.radius * zc)) < 1e-6
    assert abs(o["thick"].max() - 2 * p.radius * zc) < 1e-6
    assert abs(cov.sum() - np.pi * (size / 2) ** 2) < np.pi * size + 4
    assert o["fragments"] == cov.sum()
    # symmetric about the image centre (W, H even: the centre lies on a pixel corner)
    assert np.array_equal(cov, cov[::-1, :]) and np.array_equal(cov, cov[:, ::-1])
    k = np.unravel_index(np.argmin(o["depth_raw"]), cov.shape)
    assert o["normal_D"][k][2] > 0.999
    # thickness at every covered pixel is 2 r z of that pixel's sphere point
    d = o["depth_raw"][cov]
    assert np.allclose(o["thick"][cov], 2 * (D - d), atol=2e-6)


def test_shading_known_answers(pbf, oracle):
    """At the sprite's centre pixel (identity camera): Fresnel = r0; the
    refracted ray points away from the floor and returns the sky colour; the
    tinted refraction mixes tint and sky by exp(-thickness / 2); the depth
    option shows tanh(z / 2)."""
    D = 2.0
    pos = np.array([[0, 0, -D, 0]], np.float32)
    base = identity_camera(small_params(pbf))
    out = {}
    for opt in range(8):
        p = base.copy()
        p.shading_option = opt
        out[opt] = oracle.ssf_render(p, pos, color=np.full((p.height, p.width, 4), -1, np.float32), prec="f64")
    o = out[0]
    k = np.unravel_index(np.argmin(o["depth"]), o["depth"].shape)
    z = o["depth"][k]
    assert abs(out[4]["color"][k][0] - base.r0) < 2e-4
    sky = np.array(base.sky[:], np.float64)
    assert np.allclose(out[6]["color"][k][:3], sky, atol=1e-6)
    att = max(np.exp(-0.5 * o["thick"][k]), 0.2)
    tint = np.array([6, 105, 217]) / 256
    assert np.allclose(out[7]["color"][k][:3], (1 - att) * tint + att * sky, atol=1e-5)
    assert abs(out[1]["color"][k][0] - np.tanh(z / 2)) < 1e-6
    assert np.allclose(out[3]["color"][k][:3], o["normal_D"][k][:3], atol=1e-7)
    # background keeps the caller's colour
    for opt in range(8):
        bg = out[opt]["depth"] >= 100
        assert (out[opt]["color"][bg] == -1).all()
        assert (out[opt]["color"][~bg][:, 3] == 1).all() or opt in (1, 2)


def test_sky_cube_map_face_lookup(pbf, oracle):
    """The refracted ray of the centre pixel runs along eye -z = world -z
    (identity camera): face 5 (-z), its centre texels."""
    p = identity_camera(small_params(pbf, shading_option=6))
    sky = np.zeros((6, 4, 4, 3), np.float32)
    for f in range(6):
        sky[f] = np.array([f / 10, 1 - f / 10, 0.5], np.float32)
    o = oracle.ssf_render(p, np.array([[0, 0, -2.0, 0]], np.float32), sky=sky, prec="f64")
    k = np.unravel_index(np.argmin(o["depth"]), o["depth"].shape)
    assert np.allclose(o["color"][k][:3], sky[5, 0, 0], atol=1e-6)


def test_nothing_drawn_outside_the_clip_volume(pbf, oracle):
    p = identity_camera(small_params(pbf))
    pos = np.array([[0, 0, 1.0, 0],         # behind the camera
                    [100, 0, -2.0, 0],      # far outside the frustum
                    [0, 0, -0.05, 0],       # in front of the near plane
                    [0, 0, -150.0, 0],      # beyond the far plane
                    [np.nan, 0, -2.0, 0]], np.float32)
    o = oracle.ssf_render(p, pos, prec="f32")
    assert o["fragments"] == 0
    assert (o["depth"] == 100).all() and (o["thick"] == 0).all()


def test_smoothing_stays_within_the_covered_range(pbf, oracle, ):
    """Bilateral and gaussian passes are weighted means: a covered pixel's
    smoothed depth lies between the covered depths (the bilateral weights of
    background and out-of-image zeros vanish for sigma_z = 0.1); background
    pixels stay at 100."""
    rng = np.random.default_rng(3)
    p = small_params(pbf, 96, 72)
    pos = np.zeros((400, 4), np.float32)
    pos[:, :3] = rng.uniform([-0.5, -0.5, 1.0], [0.5, 0.5, 2.0], (400, 3))
    raw = oracle.ssf_render(p.copy(), pos, prec="f64")
    cov = raw["depth_raw"] < 99
    lo, hi = raw["depth_raw"][cov].min(), raw["depth_raw"][cov].max()
    for niter in (1, 2, 3):
        q = p.copy()
        q.smooth_niter = niter
        o = oracle.ssf_render(q, pos, prec="f64")
        assert (o["depth"][~cov] == 100).all()
        assert o["depth"][cov].min() >= lo - 1e-9 and o["depth"][cov].max() <= hi + 1e-9
    q = p.copy()
    q.kernel_r = 0
    o = oracle.ssf_render(q, pos, prec="f64")
    assert np.array_equal(o["depth"], o["depth_raw"])  # a 1-tap filter is the identity


def test_float_and_fp64_oracles_agree_away_from_rims(pbf, oracle):
    rng = np.random.default_rng(5)
    p = small_params(pbf, 128, 96)
    pos = np.zeros((2000, 4), np.float32)
    pos[:, :3] = rng.uniform([-0.6, -0.6, 0.8], [0.6, 0.6, 2.2], (2000, 3))
    a = oracle.ssf_render(p, pos, prec="f32")
    b = oracle.ssf_render(p, pos, prec="f64")
    ca, cb = a["depth_raw"] < 100, b["depth_raw"] < 100
    assert (ca != cb).sum() <= 0.002 * cb.sum() + 2  # rim pixels only
    both = ca & cb
    assert np.abs(a["depth_raw"][both] - b["depth_raw"][both]).max() < 2e-6 * 6
    # a rim fragment (pho within a few ulp of 1) adds 2 r sqrt(1 - pho) <= ~5e-5 on one side only
    assert np.abs(a["thick"] - b["thick"]).max() < 1e-5 * b["thick"].max() + 1e-4


def test_write_ppm_orientation_and_background(pbf, tmp_path):
    """Row 0 of an image is its bottom row (GL window coordinates): the file
    starts with the top row; pixels with alpha 0 take the background colour."""
    img = np.zeros((2, 3, 4), np.float32)
    img[0, :, :] = (1.0, 0.0, 0.0, 1.0)   # bottom row red
    img[1, 0, :] = (0.0, 0.0, 1.0, 1.0)   # top-left blue, rest of the top row background
    path = pbf.ssf.write_ppm(tmp_path / "x.ppm", img, background=(0.0, 1.0, 0.0))
    data = path.read_bytes()
    header = b"P6 3 2 255\n"
    assert data.startswith(header)
    px = np.frombuffer(data[len(header):], np.uint8).reshape(2, 3, 3)
    assert px[0, 0].tolist() == [0, 0, 255] and px[0, 1].tolist() == [0, 255, 0]
    assert (px[1] == [255, 0, 0]).all()


def test_look_at_refuses_degenerate_cameras(pbf):
    """Camera(pos, focus, aspect) builds up = front x ((0, 0, 1) x front): a
    camera looking along the world's up axis, or at its own position, has no
    up direction (the reference would produce NaNs); pbf_ssf_look_at refuses."""
    L = pbf.lib()
    p = pbf.ssf_default_params(64, 48)
    f3 = lambda *v: (ctypes.c_float * 3)(*v)
    assert L.pbf_ssf_look_at(ctypes.byref(p), f3(0, 0, 5), f3(0, 0, 0), 60.0) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_ssf_look_at(ctypes.byref(p), f3(1, 1, 1), f3(1, 1, 1), 60.0) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_ssf_look_at(ctypes.byref(p), f3(1, -5, 2), f3(0, 0, 1.5), 0.0) == pbf.PBF_ERR_INVALID_ARG
    assert L.pbf_ssf_look_at(ctypes.byref(p), f3(1, -5, 2), f3(0, 0, 1.5), 60.0) == pbf.PBF_OK
