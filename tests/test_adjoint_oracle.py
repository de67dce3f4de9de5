"""CPU tests of the FP64 oracle's reverse step (the adjoint the CUDA backward is
checked against) against FP64 central finite differences.

The loss is a fixed linear functional of a step's outputs written in particle
id space, L = sum_p a[iid_p] . npos_p + b[iid_p] . nvel_p, so it does not
depend on the cell order the step leaves the particles in.  Small scenes with
the reference's parameters: the step is smooth around the tested states, so
the bar is 1e-5 relative (FP64 central differences, step 1e-6).
"""
from __future__ import annotations

import numpy as np
import pytest


def setup(pbf, seed=0, n=(5, 5, 5), niter=3, speed=0.2, push_x=0.0):
    rng = np.random.default_rng(seed)
    pos = pbf.scenes.lattice(n, (0.3, 0.3, 0.3), rng).astype(np.float64)
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0, speed, size=(len(pos), 3))
    vel[:, 0] += push_x
    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    p.niter = niter
    a = rng.normal(size=(len(pos), 4))
    b = rng.normal(size=(len(pos), 4))
    a[:, 3] = b[:, 3] = 0
    return rng, pos, vel, p, a, b


def rollout(oracle, p, ulim, llim, pos, vel, steps):
    """steps chained oracle steps (tic-toc), returning per-step inputs and the last outputs."""
    iid = np.arange(len(pos), dtype=np.uint32)
    hist = []
    for _ in range(steps):
        hist.append((pos, vel, iid))
        r = oracle.step(p, ulim, llim, pos, vel, iid, "f64")
        pos, vel, iid = r["npos"], r["nvel"], r["iid"]
    return hist, pos, vel, iid


def loss_of(oracle, p, ulim, llim, pos, vel, steps, a, b):
    _, npos, nvel, iid = rollout(oracle, p, ulim, llim, pos, vel, steps)
    return float((a[iid] * npos).sum() + (b[iid] * nvel).sum())


def backward(oracle, p, ulim, llim, pos, vel, steps, a, b):
    hist, _, _, iid = rollout(oracle, p, ulim, llim, pos, vel, steps)
    gp, gv = a[iid], b[iid]
    gu = np.zeros(3)
    gl = np.zeros(3)
    for (pi, vi, ii) in reversed(hist):
        g = oracle.step_backward(p, ulim, llim, pi, vi, ii, gp, gv, "f64")
        gp, gv = g["pos"], g["vel"]
        gu += g["ulim"]
        gl += g["llim"]
    return gp, gv, gu, gl


@pytest.mark.parametrize("steps", [1, 3])
def test_oracle_adjoint_matches_finite_differences(pbf, oracle, steps):
    rng, pos, vel, p, a, b = setup(pbf, seed=steps)
    box = ((0.8, 1.2, 1.2), (0.0, 0.0, 0.0))
    gp, gv, _, _ = backward(oracle, p, *box, pos, vel, steps, a, b)
    eps = 1e-6
    for t in range(16):
        k, ax = int(rng.integers(len(pos))), int(rng.integers(3))
        for arr, g in ((pos, gp), (vel, gv)):
            x0 = arr[k, ax]
            arr[k, ax] = x0 + eps
            lp = loss_of(oracle, p, *box, pos, vel, steps, a, b)
            arr[k, ax] = x0 - eps
            lm = loss_of(oracle, p, *box, pos, vel, steps, a, b)
            arr[k, ax] = x0
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[k, ax]) <= 1e-5 * max(abs(fd), 1.0), (t, fd, g[k, ax])


def test_oracle_wall_adjoint(pbf, oracle):
    """Particles driven into the x-max wall: d loss / d ulim.x is the summed
    adjoint of the clamped coordinates (the clamp bound is ulim - LIM_EPS)."""
    rng, pos, vel, p, a, b = setup(pbf, seed=7, push_x=20.0)
    llim = (0.0, 0.0, 0.0)
    ulim = (0.62, 1.2, 1.2)
    _, _, gu, gl = backward(oracle, p, ulim, llim, pos, vel, 1, a, b)
    assert gu[0] != 0.0
    # 23 particles end on the wall plane; FP64 roundoff in the loss swamps
    # central differences below a 1e-4 step, and a slower push leaves
    # particles on the clamp's kink, so this check uses 20 m/s, a 1e-4 step
    # and a 1e-3 bar
    eps = 1e-4
    for axis in range(3):
        up = list(ulim)
        up[axis] += eps
        lp = loss_of(oracle, p, tuple(up), llim, pos, vel, 1, a, b)
        up[axis] -= 2 * eps
        lm = loss_of(oracle, p, tuple(up), llim, pos, vel, 1, a, b)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - gu[axis]) <= 1e-3 * max(abs(fd), 1.0), (axis, fd, gu[axis])


def test_oracle_adjoint_rejects_boundary_density(pbf, oracle):
    _, pos, vel, p, a, b = setup(pbf)
    p.k_boundaryDensity = 0.1
    with pytest.raises(ValueError):
        oracle.step_backward(p, (1, 1, 1), (0, 0, 0), pos, vel, np.arange(len(pos), dtype=np.uint32), a, b)
