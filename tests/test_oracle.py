"""CPU tests of the oracle: known answers derived from the reference's formulas
(fluids/Simulator.cu:75-161, fluids/Simulator_kernel.cuh:52-239), grid
properties, and agreement of the float port with the FP64 oracle."""
from __future__ import annotations

import numpy as np
import pytest

REF_PI = 3.14159265359  # fluids/helper.h:4


def poly6(r2, h):
    return 315.0 / (64.0 * REF_PI * h ** 9) * (h * h - r2) ** 3 if r2 < h * h else 0.0


def spiky(r, h):
    rl = float(np.linalg.norm(r))
    if rl >= h or rl < 1e-4:
        return np.zeros(3)
    return -45.0 / (REF_PI * h ** 6) * (h - rl) ** 2 / rl * np.asarray(r, float)


def ref_params(pbf, up=(0.0, 1.0, 0.0)):
    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = up
    return p


def one(x, y, z):
    return np.array([[x, y, z, 0.0]], np.float32)


def test_isolated_particle(pbf, oracle):
    """A lone particle: rho = W(0), zero gradient, lambda = -(W(0)/pho0 - 1)/eps,
    no correction; v = (x* - x)/dt; XSPH adds nothing."""
    p = ref_params(pbf)
    p.niter = 3
    box_u, box_l = (2.0, 2.0, 2.0), (0.0, 0.0, 0.0)
    pos = one(1.0, 1.0, 1.0)
    vel = np.array([[0.3, -0.2, 0.1, 0.0]], np.float32)
    r = oracle.step(p, box_u, box_l, pos, vel, np.zeros(1, np.uint32), prec="f64")
    h = float(p.h)
    w0 = poly6(0.0, h)
    assert r["rho"][0] == pytest.approx(w0, rel=1e-12)
    assert r["lambda"][0] == pytest.approx(-(w0 / float(p.pho0) - 1) / float(p.lambda_eps), rel=1e-12)
    dt = float(p.dt)
    g = np.array([0.0, -float(p.g), 0.0])
    v1 = vel[0, :3].astype(np.float64) + dt * g
    xs = pos[0, :3].astype(np.float64) + dt * v1
    np.testing.assert_allclose(r["npos"][0, :3], xs, rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["vel"][0, :3], (xs - pos[0, :3]) / dt, rtol=1e-9)
    np.testing.assert_allclose(r["nvel"][0, :3], r["vel"][0, :3], rtol=0, atol=0)


def test_particle_pair(pbf, oracle):
    """Two particles at r < h along x: rho, lambda and the s_corr-weighted
    delta_p of computeLambda / computetpos, in closed form."""
    p = ref_params(pbf)
    p.niter = 1
    p.g = 0.0
    h = float(p.h)
    d = 0.06
    pos = np.array([[1.0, 1.0, 1.0, 0.0], [1.0 + d, 1.0, 1.0, 0.0]], np.float32)
    d = float(pos[1, 0]) - float(pos[0, 0])
    vel = np.zeros_like(pos)
    r = oracle.step(p, (2.0, 2.0, 2.0), (0.0, 0.0, 0.0), pos, vel, np.arange(2, dtype=np.uint32), prec="f64")
    rho = poly6(0.0, h) + poly6(d * d, h)
    gr = spiky(np.array([-d, 0, 0]), h) / float(p.pho0)  # particle 0: x0 - x1
    lam = -(rho / float(p.pho0) - 1) / (2 * float(gr @ gr) + float(p.lambda_eps))
    np.testing.assert_allclose(r["rho"], [rho, rho], rtol=1e-12)
    np.testing.assert_allclose(r["lambda"], [lam, lam], rtol=1e-9)
    dq = float(p.delta_q)
    corr = -float(p.k_corr) / poly6(dq * dq, h) ** float(p.n_corr) * poly6(d * d, h) ** float(p.n_corr)
    dp0 = (2 * lam + corr) * spiky(np.array([-d, 0, 0]), h) / float(p.pho0)
    dp0 = np.clip(dp0, -float(p.max_dp), float(p.max_dp))
    # sorted order keeps input order (same cell or ascending cells)
    np.testing.assert_allclose(r["npos"][0, :3], pos[0, :3].astype(np.float64) + dp0, rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["npos"][1, :3], pos[1, :3].astype(np.float64) - dp0, rtol=0, atol=1e-12)


def test_wall_clamp(pbf, oracle):
    """A particle driven through the x-max wall ends at ulim - LIM_EPS
    (fluids/Simulator_kernel.cuh:190-192)."""
    p = ref_params(pbf)
    p.niter = 1
    pos = one(1.95, 1.0, 1.0)
    vel = np.array([[50.0, 0.0, 0.0, 0.0]], np.float32)
    for prec in ("f32", "f64"):
        r = oracle.step(p, (2.0, 2.0, 2.0), (0.0, 0.0, 0.0), pos, vel, np.zeros(1, np.uint32), prec=prec)
        # the bound is computed in double with LIM_EPS = 1e-3 (fluids/helper.h:5)
        want = np.float32(2.0 - 1e-3) if prec == "f32" else 2.0 - 1e-3
        assert r["npos"][0, 0] == want


def test_empty_and_single_cell(pbf, oracle):
    p = ref_params(pbf)
    r = oracle.step(p, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), np.zeros((0, 4), np.float32), np.zeros((0, 4), np.float32),
                    np.zeros(0, np.uint32))
    assert r["npos"].shape == (0, 4)
    rng = np.random.default_rng(3)
    xs = np.zeros((50, 4), np.float32)
    xs[:, :3] = 0.5 + rng.uniform(0.0, 0.09, size=(50, 3))
    g = oracle.grid(p, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0), xs)
    assert g["dims"] == (10, 10, 10)
    cell = 5 * 100 + 5 * 10 + 5
    assert np.all(g["keys"] == cell)
    np.testing.assert_array_equal(g["perm"], np.arange(50))
    assert g["start"][cell] == 0 and g["end"][cell] == 50
    assert g["start"].sum() == 0 and g["end"].sum() == 50


def _numpy_grid(xs, ulim, llim, h):
    """Independent numpy restatement of getGridId + stable sort + computeGridRange."""
    ulim = np.asarray(ulim, np.float32)
    llim = np.asarray(llim, np.float32)
    h = np.float32(h)
    dims = np.ceil((ulim - llim) / h).astype(np.int64)
    q = np.trunc((xs[:, :3] - llim) / h)
    q = np.nan_to_num(q, nan=0.0)
    q = np.clip(q, -2 ** 31, 2 ** 31 - 1).astype(np.int64)
    q = np.clip(q, 0, dims - 1)
    keys = (q[:, 0] * dims[1] + q[:, 1]) * dims[2] + q[:, 2]
    perm = np.argsort(keys, kind="stable")
    cells = int(np.prod(dims))
    cnt = np.bincount(keys, minlength=cells)
    cs = np.concatenate([[0], np.cumsum(cnt)])
    start = np.where(cnt > 0, cs[:-1], 0)
    end = np.where(cnt > 0, cs[1:], 0)
    return keys.astype(np.uint32), perm.astype(np.uint32), start, end, tuple(int(d) for d in dims)


def test_grid_matches_numpy_restatement(pbf, oracle):
    sc = pbf.scenes.double_dam(seed=1)
    p = sc.params
    xs = oracle.predict(p, sc.pos, sc.vel)
    rng = np.random.default_rng(0)
    # include out-of-box and NaN positions: clamped into edge cells / cell 0
    xs[:20, :3] = rng.uniform(-1.0, 5.0, size=(20, 3)).astype(np.float32)
    xs[20, 0] = np.nan
    g = oracle.grid(p, sc.ulim, sc.llim, xs)
    keys, perm, start, end, dims = _numpy_grid(xs, sc.ulim, sc.llim, p.h)
    assert g["dims"] == dims
    np.testing.assert_array_equal(g["keys"], keys)
    np.testing.assert_array_equal(g["perm"], perm)
    np.testing.assert_array_equal(g["start"], start)
    np.testing.assert_array_equal(g["end"], end)


def test_predict_is_fused(pbf, oracle):
    """x* = fma(dt, fma(dt, g, v), x) in float: differs from the unfused
    expression on some inputs, equals a float64 evaluation rounded once."""
    p = ref_params(pbf)
    rng = np.random.default_rng(5)
    pos = np.zeros((4096, 4), np.float32)
    vel = np.zeros((4096, 4), np.float32)
    pos[:, :3] = rng.uniform(0, 3, size=(4096, 3))
    vel[:, :3] = rng.normal(0, 2, size=(4096, 3))
    xs = oracle.predict(p, pos, vel)
    dt = np.float32(p.dt)
    g = np.float32(-p.g)
    vy = (np.float64(dt) * np.float64(g) + vel[:, 1].astype(np.float64)).astype(np.float32)
    want = (np.float64(dt) * vy.astype(np.float64) + pos[:, 1].astype(np.float64)).astype(np.float32)
    np.testing.assert_array_equal(xs[:, 1], want)
    np.testing.assert_array_equal(xs[:, 0], (np.float64(dt) * vel[:, 0] + pos[:, 0].astype(np.float64)).astype(np.float32))


@pytest.mark.parametrize("niter", [1, 4])
def test_port_matches_fp64_reference_params(pbf, oracle, niter):
    """With the reference's own parameters (fluids/FluidSystem.cpp:15-25) the
    float port stays within 1e-5 h of the FP64 oracle after a full step."""
    sc = pbf.scenes.dam_break(seed=0)
    p = ref_params(pbf)
    p.niter = niter
    iid = np.arange(sc.n, dtype=np.uint32)
    a = oracle.step(p, sc.ulim, sc.llim, sc.pos, sc.vel, iid, "f32")
    b = oracle.step(p, sc.ulim, sc.llim, sc.pos, sc.vel, iid, "f64")
    np.testing.assert_array_equal(a["iid"], b["iid"])
    assert np.abs(a["npos"][:, :3] - b["npos"][:, :3]).max() <= 1e-5 * p.h
    assert np.abs(a["rho"] - b["rho"]).max() <= 1e-5 * b["rho"].max()


def test_port_matches_fp64_scene_params_one_iteration(pbf, oracle):
    sc = pbf.scenes.dam_break(seed=0)
    p = sc.params
    p.niter = 1
    iid = np.arange(sc.n, dtype=np.uint32)
    a = oracle.step(p, sc.ulim, sc.llim, sc.pos, sc.vel, iid, "f32")
    b = oracle.step(p, sc.ulim, sc.llim, sc.pos, sc.vel, iid, "f64")
    assert np.abs(a["npos"][:, :3] - b["npos"][:, :3]).max() <= 1e-5 * p.h


def test_step_permutes_like_stable_sort(pbf, oracle):
    """pos/vel/iid come back permuted by the stable cell sort of x*."""
    sc = pbf.scenes.dam_break(seed=2)
    p = ref_params(pbf)
    rng = np.random.default_rng(1)
    order = rng.permutation(sc.n)
    pos, vel = sc.pos[order], sc.vel[order]
    iid = order.astype(np.uint32)
    r = oracle.step(p, sc.ulim, sc.llim, pos, vel, iid, "f32")
    xs = oracle.predict(p, pos, vel)
    keys, perm, _, _, _ = _numpy_grid(xs, sc.ulim, sc.llim, p.h)
    np.testing.assert_array_equal(r["iid"], iid[perm])
    np.testing.assert_array_equal(r["pos"], pos[perm])
    assert np.all(np.diff(keys[perm].astype(np.int64)) >= 0)


def test_threads(oracle):
    assert oracle.threads() >= 1
