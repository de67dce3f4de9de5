"""GPU tests of the reverse pass (pbf_tape_enable / pbf_backward), the density
grid (pbf_density_grid / pbf_density_grid_backward) and the checkpointed
rollout, against the FP64 oracle's exact adjoint (itself checked against
finite differences on the CPU).

The GPU pass is FP32 and gathers transposed pair terms over the forward's
windows (exact when no particle crosses a cell boundary during a step's
iterations), so the bar is relative to the gradient's scale:
|gpu - oracle| <= 2e-3 * max|oracle| per component.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 2e-3


def setup(pbf, seed=0, n=(5, 5, 5), niter=3, speed=0.2, push_x=0.0, origin=(0.3, 0.3, 0.3)):
    rng = np.random.default_rng(seed)
    pos = pbf.scenes.lattice(n, origin, rng)
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0, speed, size=(len(pos), 3))
    vel[:, 0] += push_x
    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    p.niter = niter
    a = rng.normal(size=(len(pos), 4)).astype(np.float32)
    b = rng.normal(size=(len(pos), 4)).astype(np.float32)
    a[:, 3] = b[:, 3] = 0
    return rng, pos, vel, p, a, b


def close(got, want, what):
    scale = max(np.abs(want).max(), 1e-30)
    err = np.abs(got - want).max()
    assert err <= REL * scale, f"{what}: max err {err:.3e} vs scale {scale:.3e}"


def gpu_step_backward(pbf, p, ulim, llim, pos, vel, ga, gb, lanes=0):
    """One taped step, then its reverse pass with g_npos = ga[iid], g_nvel = gb[iid]
    (lanes: the reverse pass's lanes per particle, 0 for the default)."""
    import torch

    n = len(pos)
    d_pos = torch.from_numpy(pos.copy()).cuda()
    d_vel = torch.from_numpy(vel.copy()).cuda()
    iid = torch.arange(n, dtype=torch.int32, device="cuda")
    npos = torch.empty_like(d_pos)
    nvel = torch.empty_like(d_vel)
    with pbf.Simulator(p, ulim, llim, n) as sim:
        sim.set_tuning(bwd_lanes=lanes)
        sim.tape(True)
        sim.step(d_pos, npos, d_vel, nvel, iid, n)
        order = iid.long()
        g_npos = torch.from_numpy(ga).cuda()[order].contiguous()
        g_nvel = torch.from_numpy(gb).cuda()[order].contiguous()
        g_pos, g_vel, g_lim = sim.backward(g_npos, g_nvel)
        torch.cuda.synchronize()
        return g_pos.cpu().numpy(), g_vel.cpu().numpy(), g_lim.cpu().numpy(), iid.cpu().numpy()


@pytest.mark.parametrize("seed,n,lanes", [(0, (5, 5, 5), 0), (1, (10, 8, 6), 0), (2, (12, 12, 12), 0),
                                          (2, (12, 12, 12), 8), (1, (10, 8, 6), 16)])
def test_backward_matches_oracle(pbf, oracle, cuda, seed, n, lanes):
    _, pos, vel, p, a, b = setup(pbf, seed=seed, n=n)
    ulim, llim = (1.2, 1.2, 1.2), (0.0, 0.0, 0.0)
    g_pos, g_vel, g_lim, _ = gpu_step_backward(pbf, p, ulim, llim, pos, vel, a, b, lanes)
    iid = np.arange(len(pos), dtype=np.uint32)
    r = oracle.step(p, ulim, llim, pos.astype(np.float64), vel.astype(np.float64), iid, "f64")
    want = oracle.step_backward(p, ulim, llim, pos.astype(np.float64), vel.astype(np.float64), iid,
                                a[r["iid"]].astype(np.float64), b[r["iid"]].astype(np.float64), "f64")
    close(g_pos[:, :3], want["pos"][:, :3], "g_pos")
    close(g_vel[:, :3], want["vel"][:, :3], "g_vel")
    assert np.all(g_lim == 0)


def test_backward_wall_adjoint(pbf, oracle, cuda):
    """Particles driven into the x-max wall: the limits' adjoint is non-zero and
    matches the oracle's."""
    _, pos, vel, p, a, b = setup(pbf, seed=7, push_x=20.0)
    ulim, llim = (0.62, 1.2, 1.2), (0.0, 0.0, 0.0)
    g_pos, g_vel, g_lim, _ = gpu_step_backward(pbf, p, ulim, llim, pos, vel, a, b)
    iid = np.arange(len(pos), dtype=np.uint32)
    r = oracle.step(p, ulim, llim, pos.astype(np.float64), vel.astype(np.float64), iid, "f64")
    want = oracle.step_backward(p, ulim, llim, pos.astype(np.float64), vel.astype(np.float64), iid,
                                a[r["iid"]].astype(np.float64), b[r["iid"]].astype(np.float64), "f64")
    assert want["ulim"][0] != 0
    close(g_pos[:, :3], want["pos"][:, :3], "g_pos")
    close(g_vel[:, :3], want["vel"][:, :3], "g_vel")
    close(g_lim[:3], want["ulim"], "g_ulim")
    close(g_lim[3:], want["llim"], "g_llim")


def oracle_chain(oracle, p, lims, pos, vel, steps, a, b):
    iid = np.arange(len(pos), dtype=np.uint32)
    hist = []
    pos, vel = pos.astype(np.float64), vel.astype(np.float64)
    for k in range(steps):
        hist.append((pos, vel, iid))
        r = oracle.step(p, *lims(k), pos, vel, iid, "f64")
        pos, vel, iid = r["npos"], r["nvel"], r["iid"]
    gp, gv = a[iid].astype(np.float64), b[iid].astype(np.float64)
    g_lim = np.zeros((steps, 6))
    for k in range(steps - 1, -1, -1):
        pi, vi, ii = hist[k]
        g = oracle.step_backward(p, *lims(k), pi, vi, ii, gp, gv, "f64")
        gp, gv = g["pos"], g["vel"]
        g_lim[k, :3], g_lim[k, 3:] = g["ulim"], g["llim"]
    return gp, gv, g_lim


@pytest.mark.parametrize("every", [1, 2, 10])
def test_rollout_matches_oracle_chain(pbf, oracle, cuda, every):
    """Three steps with a moving x-max wall through the checkpointed rollout."""
    import torch

    steps = 3
    _, pos, vel, p, a, b = setup(pbf, seed=11, push_x=6.0)

    def lims(k):
        return (0.66 - 0.01 * k, 1.2, 1.2), (0.0, 0.0, 0.0)

    n = len(pos)
    with pbf.Simulator(p, *lims(0), n) as sim:
        ro = pbf.adjoint.Rollout(sim, every=every)
        fpos, fvel, fiid = ro.run(torch.from_numpy(pos).cuda(), torch.from_numpy(vel).cuda(),
                                  torch.arange(n, dtype=torch.int32, device="cuda"), steps, lims)
        order = fiid.long()
        g_pos, g_vel, g_lim = ro.backward(torch.from_numpy(a).cuda()[order].contiguous(),
                                          torch.from_numpy(b).cuda()[order].contiguous())
        torch.cuda.synchronize()
    gp, gv, gl = oracle_chain(oracle, p, lims, pos, vel, steps, a, b)
    assert np.abs(gl[:, 0]).max() > 0
    close(g_pos.cpu().numpy()[:, :3], gp[:, :3], "g_pos")
    close(g_vel.cpu().numpy()[:, :3], gv[:, :3], "g_vel")
    close(g_lim.cpu().numpy(), gl, "g_lim")


def test_autograd_step_matches_rollout(pbf, cuda):
    """Two steps through the torch.autograd binding equal the rollout's reverse sweep bitwise."""
    import torch

    _, pos, vel, p, a, b = setup(pbf, seed=5)
    n = len(pos)
    lims = ((1.2, 1.2, 1.2), (0.0, 0.0, 0.0))
    with pbf.Simulator(p, *lims, n) as sim:
        x = torch.from_numpy(pos).cuda().requires_grad_(True)
        v = torch.from_numpy(vel).cuda().requires_grad_(True)
        iid = torch.arange(n, dtype=torch.int32, device="cuda")
        x1, v1, i1 = pbf.adjoint.step(sim, x, v, iid, *lims)
        x2, v2, i2 = pbf.adjoint.step(sim, x1, v1, i1, *lims)
        ga = torch.from_numpy(a).cuda()[i2.long()]
        gb = torch.from_numpy(b).cuda()[i2.long()]
        loss = (ga * x2).sum() + (gb * v2).sum()
        gx, gv = torch.autograd.grad(loss, (x, v))
        ro = pbf.adjoint.Rollout(sim, every=10)
        _, _, fiid = ro.run(torch.from_numpy(pos).cuda(), torch.from_numpy(vel).cuda(),
                            torch.arange(n, dtype=torch.int32, device="cuda"), 2, lambda k: lims)
        assert torch.equal(fiid, i2)
        rx, rv, _ = ro.backward(ga.contiguous(), gb.contiguous())
        assert torch.equal(gx, rx) and torch.equal(gv, rv)


def test_density_grid_matches_oracle(pbf, oracle, cuda):
    import torch

    rng = np.random.default_rng(9)
    pos = pbf.scenes.lattice((25, 25, 25), (0.0, 0.0, 0.0), rng, spacing=0.04)
    lo, hi, dims, h = (0.0, 0.0, 0.0), (2.0, 1.0, 1.0), (32, 16, 16), 0.1
    d_pos = torch.from_numpy(pos).cuda()
    got = pbf.adjoint.density_grid(d_pos, lo, hi, dims, h)
    want = oracle.density_grid(pos, lo, hi, dims, h)
    assert np.abs(got.cpu().numpy() - want).max() <= 1e-5 * want.max()
    g_grid = rng.normal(size=dims).astype(np.float32)
    g = pbf.adjoint.density_grid_backward(d_pos, lo, hi, dims, h, torch.from_numpy(g_grid).cuda())
    gw = oracle.density_grid_backward(pos, lo, hi, dims, h, g_grid)
    close(g.cpu().numpy()[:, :3], gw[:, :3], "g_pos")


def test_backward_errors(pbf, cuda):
    import torch

    _, pos, vel, p, a, b = setup(pbf)
    n = len(pos)
    with pbf.Simulator(p, (1.2, 1.2, 1.2), (0.0, 0.0, 0.0), n) as sim:
        g = torch.zeros(n, 4, device="cuda")
        with pytest.raises(pbf.PbfError):
            sim.backward(g, g)  # nothing taped yet
        d_pos = torch.from_numpy(pos).cuda()
        d_vel = torch.from_numpy(vel).cuda()
        iid = torch.arange(n, dtype=torch.int32, device="cuda")
        npos, nvel = torch.empty_like(d_pos), torch.empty_like(d_vel)
        sim.step(d_pos, npos, d_vel, nvel, iid, n)
        with pytest.raises(pbf.PbfError):
            sim.backward(g, g)  # the step was not taped
        p2 = sim.saveParams()
        p2.k_boundaryDensity = 0.1
        sim.loadParams(p2)
        with pytest.raises(pbf.PbfError):
            sim.tape(True)


def test_backward_is_bitwise_reproducible(pbf, oracle, cuda):
    """Two reverse passes of the same taped step give bitwise equal adjoints,
    on a step where many pairs are one-sided (fast particles crossing cell
    boundaries during the iterations, so their terms are scattered rather than
    gathered: the scattered sums are exact integer sums, independent of the
    order the terms arrive in).  The result still matches the FP64 adjoint."""
    _, pos, vel, p, a, b = setup(pbf, seed=11, n=(12, 12, 12), speed=3.0)
    ulim, llim = (1.2, 1.2, 1.2), (0.0, 0.0, 0.0)
    runs = [gpu_step_backward(pbf, p, ulim, llim, pos, vel, a, b) for _ in range(3)]
    for other in runs[1:]:
        for x, y in zip(runs[0], other):
            assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))
    iid = np.arange(len(pos), dtype=np.uint32)
    r = oracle.step(p, ulim, llim, pos.astype(np.float64), vel.astype(np.float64), iid, "f64")
    want = oracle.step_backward(p, ulim, llim, pos.astype(np.float64), vel.astype(np.float64), iid,
                                a[r["iid"]].astype(np.float64), b[r["iid"]].astype(np.float64), "f64")
    g_pos, g_vel = runs[0][0], runs[0][1]
    close(g_pos[:, :3], want["pos"][:, :3], "g_pos")
    close(g_vel[:, :3], want["vel"][:, :3], "g_vel")


def test_backward_graph_replay_matches_eager(pbf, cuda):
    """The reverse pass as a CUDA graph -- captured on the first call, replayed
    from the solver's cache when the same tape slot is reversed into the same
    buffers again -- gives bitwise the adjoints of the same pass launched kernel
    by kernel (pbf_use_graphs(s, 0))."""
    import torch

    _, pos, vel, p, a, b = setup(pbf, seed=12, n=(12, 12, 12), speed=3.0)
    ulim, llim = (1.2, 1.2, 1.2), (0.0, 0.0, 0.0)
    n = len(pos)
    d_pos0 = torch.from_numpy(pos.copy()).cuda()
    d_vel0 = torch.from_numpy(vel.copy()).cuda()
    d_pos, d_vel = torch.empty_like(d_pos0), torch.empty_like(d_vel0)
    npos, nvel = torch.empty_like(d_pos0), torch.empty_like(d_vel0)
    iid = torch.empty(n, dtype=torch.int32, device="cuda")
    g_npos = torch.from_numpy(a).cuda()
    g_nvel = torch.from_numpy(b).cuda()
    g_pos, g_vel = torch.empty_like(g_npos), torch.empty_like(g_nvel)
    g_lim = torch.empty(6, dtype=torch.float32, device="cuda")
    L = pbf.lib()
    runs = []
    with pbf.Simulator(p, ulim, llim, n) as sim:
        sim.tape(True)
        for graphs in (True, True, False):
            sim.use_graphs(graphs)
            d_pos.copy_(d_pos0)
            d_vel.copy_(d_vel0)
            iid.copy_(torch.arange(n, dtype=torch.int32, device="cuda"))
            sim.step(d_pos, npos, d_vel, nvel, iid, n)
            pbf.check(L.pbf_backward(sim._h, g_npos.data_ptr(), g_nvel.data_ptr(), g_pos.data_ptr(),
                                     g_vel.data_ptr(), g_lim.data_ptr(), None), "pbf_backward")
            torch.cuda.synchronize()
            runs.append((g_pos.cpu().numpy().copy(), g_vel.cpu().numpy().copy(), g_lim.cpu().numpy().copy()))
    assert np.isfinite(runs[0][0]).all() and np.abs(runs[0][0]).max() > 0
    for other in runs[1:]:
        for x, y in zip(runs[0], other):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
