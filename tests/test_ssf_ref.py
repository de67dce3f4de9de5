"""The SSF oracle against the reference's own shaders.

The reference renders with OpenGL, but its SSF shaders (fluids/shader/SSF*.glsl)
are plain arithmetic: oracle/ref_harness compiles them as C++ and runs them on
the CPU with the fixed-function steps of fluids/SSFRenderer.cpp made explicit.
tests/golden/make_ssf_golden.py recorded their outputs (tests/golden/ssf_ref_*.npz);
the oracle is checked against them stage by stage, each stage fed the
reference's previous-stage output, and against a live build where the
reference sources are present.

Bars: the same fragments and covered pixels; splat depth within 1e-6 relative
(gl_PointCoord from one reciprocal of the point size here, a division there);
thickness within 1e-5 + 1e-6 |t| (fixed point here, float blending in draw
order there); smoothing within 1e-6 relative and normals within 1e-6 (the same
formulas; only the exp of another C library could differ); shading within 1e-5
on the fluid's pixels, drawn on the same pixels.  The GPU is held to the oracle
stage by stage in tests/test_gpu_ssf.py.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem.replace("ssf_ref_", "") for p in GOLDEN.glob("ssf_ref_*.npz"))


def params_from(oracle, g):
    p = oracle.OracleSsfParams()
    for name, ctype in p._fields_:
        v = g[f"param_{name}"]
        if hasattr(ctype, "_length_"):
            arr = getattr(p, name)
            for k in range(ctype._length_):
                arr[k] = float(v[k])
        else:
            setattr(p, name, v.item())
    return p


def with_(oracle, p, **kw):
    q = oracle.OracleSsfParams()
    for name, _ in p._fields_:
        setattr(q, name, getattr(p, name))
    for k, v in kw.items():
        setattr(q, k, v)
    return q


def check_stages(oracle, p, pos, sky, ref):
    """ref: dict with depth, thick, fragments, smooth, normal_D, colors (8 options)."""
    o = oracle.ssf_render(with_(oracle, p, smooth_niter=0), pos, prec="f32")
    assert o["fragments"] == int(ref["fragments"])
    cov = ref["depth"] < 99
    assert np.array_equal(o["depth_raw"] < 99, cov)
    assert (np.abs(o["depth_raw"][cov] - ref["depth"][cov]) <= 1e-6 * ref["depth"][cov]).all()
    assert (np.abs(o["thick"] - ref["thick"]) <= 1e-5 + 1e-6 * np.abs(ref["thick"])).all()
    sm = oracle.ssf_smooth(p, ref["depth"], prec="f32")
    bg = ref["smooth"] >= 99
    assert np.array_equal(sm >= 99, bg)
    assert (np.abs(sm[~bg] - ref["smooth"][~bg]) <= 1e-6 * ref["smooth"][~bg]).all()
    nd = oracle.ssf_normals(p, ref["smooth"], prec="f32")
    assert np.abs(nd - ref["normal_D"]).max() <= 1e-6 * max(1.0, float(np.abs(ref["normal_D"][..., 3]).max()))
    fluid = ref["smooth"] < 99
    for opt in range(8):
        q = with_(oracle, p, shading_option=opt)
        fill = np.full(ref["depth"].shape + (4,), -1.0, np.float32)
        c = oracle.ssf_shade(q, ref["smooth"], ref["normal_D"], ref["thick"], fill, sky=sky, prec="f32")
        rc = ref["colors"][opt]
        assert np.array_equal((c[..., 3] != -1) & fluid, (rc[..., 3] != -1) & fluid), opt
        m = (rc[..., 3] != -1) & fluid
        assert np.abs(c[m] - rc[m]).max(initial=0.0) <= 1e-5, opt


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_shader_golden(oracle, case):
    g = np.load(GOLDEN / f"ssf_ref_{case}.npz")
    p = params_from(oracle, g)
    sky = g["sky"] if g["sky"].size else None
    check_stages(oracle, p, g["pos"], sky, {k: g[k] for k in ("depth", "thick", "fragments", "smooth", "normal_D",
                                                              "colors")})
    assert int((g["depth"] < 99).sum()) > 200  # the fixture draws something


def test_golden_cases_present():
    assert set(CASES) >= {"block", "droplets", "gaussian"}


def test_oracle_matches_live_reference_shaders(pbf, oracle):
    """The dam-break start at 320 x 240 with the reference's settings, against
    the reference's shaders built from its sources (where they are present)."""
    if not oracle.ssf_ref_available():
        pytest.skip("the reference's shader sources are not on this machine")
    sc = pbf.scenes.dam_break(seed=0)
    pos = sc.pos.copy()
    pos[:, 1], pos[:, 2] = -sc.pos[:, 2], sc.pos[:, 1]
    p = pbf.ssf_default_params(320, 240)
    pbf.ssf.look_at(p, (2.6, -3.2, 1.8), (0.5, -0.5, 0.5))
    op = oracle.to_oracle_ssf_params(p)
    depth, thick, frags = oracle.ssf_ref_splat(op, pos)
    smooth = oracle.ssf_ref_smooth(op, depth)
    nd = oracle.ssf_ref_normals(op, smooth)
    colors = []
    for opt in range(8):
        fill = np.full(depth.shape + (4,), -1.0, np.float32)
        colors.append(oracle.ssf_ref_shade(with_(oracle, op, shading_option=opt), smooth, nd, thick, fill))
    check_stages(oracle, op, pos, None, {"depth": depth, "thick": thick, "fragments": frags, "smooth": smooth,
                                         "normal_D": nd, "colors": np.stack(colors)})
