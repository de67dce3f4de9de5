"""GPU tests of the inverse problem (pbf_cuda_gb300.inverse): the GPU
gradient of the reduced problem against the FP64 oracle's (itself checked
against finite differences on the CPU), and one optimisation step of the
full-size problem."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_inverse_gradient_matches_oracle(pbf, cuda):
    import torch
    from oracle import inverse as oinv
    from test_inverse_oracle import reduced_problem

    pb, target = reduced_problem(pbf, oinv)
    v0 = np.random.default_rng(3).normal(0.0, 0.05, size=(len(pb.pos0), 3))
    amp = 0.02
    L, gv, ga = oinv.loss_and_grad(pb, v0, amp, target)
    scene = pbf.scenes.Scene("reduced", pb.pos0.astype(np.float32), np.zeros_like(pb.pos0, np.float32), pb.box,
                             (0.0, 0.0, 0.0), params=pb.params)
    with pbf.inverse.InverseProblem(scene, frames=3, every=1, dims=pb.dims, period=pb.period) as ip:
        ip.target = torch.from_numpy(target.astype(np.float32)).cuda()
        Lg, gvg, gag = ip.loss_and_grad(torch.from_numpy(v0.astype(np.float32)), amp)
        torch.cuda.synchronize()
    assert abs(Lg - L) <= 1e-4 * L
    gvg = gvg.cpu().numpy()
    assert np.abs(gvg - gv).max() <= 2e-3 * np.abs(gv).max()
    assert abs(gag - ga) <= 2e-3 * abs(ga)


def test_inverse_full_size_short_horizon_descends(pbf, cuda):
    """15,625 particles (the inverse scene), the reference's default solver
    parameters, 2 frames: a small step along the negative gradient lowers the
    loss.  (Over tens of frames the step's adjoint grows by orders of
    magnitude per frame, in the FP64 oracle as on the GPU, and overflows
    float32; the horizon here keeps it finite.)"""
    import torch

    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    scene = pbf.scenes.inverse_scene()
    scene.params = p
    with pbf.inverse.InverseProblem(scene, frames=2, every=1) as ip:
        ip.make_target()
        v0 = torch.zeros((ip.n, 3), device="cuda")
        L0, gv, ga = ip.loss_and_grad(v0, 0.0)
        assert torch.isfinite(gv).all() and np.isfinite(ga)
        assert gv.abs().max() > 0
        step = 1e-3 / float(gv.abs().max())
        L1 = ip.loss(v0 - step * gv, 0.0)
        assert L1 < L0, (L0, L1)


def test_backward_full_size_one_step_matches_oracle(pbf, oracle, cuda):
    """One step of the inverse scene (15,625 particles, reference parameters,
    random velocities) through pbf_backward against the FP64 oracle."""
    import torch

    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    scene = pbf.scenes.inverse_scene()
    rng = np.random.default_rng(8)
    pos = scene.pos
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0, 0.2, size=(len(pos), 3))
    a = rng.normal(size=pos.shape).astype(np.float32)
    b = rng.normal(size=pos.shape).astype(np.float32)
    a[:, 3] = b[:, 3] = 0
    n = len(pos)
    with pbf.Simulator(p, scene.ulim, scene.llim, n) as sim:
        sim.tape(True)
        d_pos, d_vel = torch.from_numpy(pos.copy()).cuda(), torch.from_numpy(vel.copy()).cuda()
        iid = torch.arange(n, dtype=torch.int32, device="cuda")
        npos, nvel = torch.empty_like(d_pos), torch.empty_like(d_vel)
        sim.step(d_pos, npos, d_vel, nvel, iid, n)
        order = iid.long()
        g_pos, g_vel, _ = sim.backward(torch.from_numpy(a).cuda()[order].contiguous(),
                                       torch.from_numpy(b).cuda()[order].contiguous())
        torch.cuda.synchronize()
    ii = np.arange(n, dtype=np.uint32)
    r = oracle.step(p, scene.ulim, scene.llim, pos.astype(np.float64), vel.astype(np.float64), ii, "f64")
    want = oracle.step_backward(p, scene.ulim, scene.llim, pos.astype(np.float64), vel.astype(np.float64), ii,
                                a[r["iid"]].astype(np.float64), b[r["iid"]].astype(np.float64), "f64")
    for got, w in ((g_pos.cpu().numpy(), want["pos"]), (g_vel.cpu().numpy(), want["vel"])):
        assert np.abs(got[:, :3] - w[:, :3]).max() <= 2e-3 * np.abs(w[:, :3]).max()
