"""CPU test: the FP64 inverse problem (oracle/inverse.py: chained oracle steps,
density-grid loss, reverse sweep, wall-amplitude chain rule) against FP64
central finite differences.

A reduced problem: 216 particles, 6 steps, the x-max wall sweeping with a
0.2 s period into the fluid, the reference's default solver parameters.
Velocity coordinates use the 1e-4 finite-difference step.  The amplitude uses
3e-5: at 1e-4 the curvature of the wall contact (particles entering and
leaving the clamp) costs ~1.5e-3, and below ~1e-5 the float32 wall position
(the limits are float, as in the reference) quantises the difference.
"""
from __future__ import annotations

import numpy as np


def reduced_problem(pbf, oinv, steps=6):
    rng = np.random.default_rng(0)
    pos = pbf.scenes.lattice((6, 6, 6), (0.0, 0.0, 0.0), rng, spacing=0.05).astype(np.float64)
    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    pb = oinv.Problem(p, pos, (0.27, 0.3, 0.3), (6, 6, 6), steps, period=0.2)
    vt = np.random.default_rng(1).normal(0.0, 0.2, size=(len(pos), 3))
    _, pt, _, _ = oinv.rollout(pb, vt, 0.05)
    return pb, oinv.density(pb, pt)


def test_inverse_gradient_matches_finite_differences(pbf):
    from oracle import inverse as oinv

    pb, target = reduced_problem(pbf, oinv)
    v0 = np.zeros((len(pb.pos0), 3))
    amp = 0.02
    _, gv, ga = oinv.loss_and_grad(pb, v0, amp, target)
    assert ga != 0.0
    rng = np.random.default_rng(2)
    eps = 1e-4
    for _ in range(32):
        k, ax = int(rng.integers(len(v0))), int(rng.integers(3))
        v0[k, ax] += eps
        lp = oinv.loss(pb, v0, amp, target)
        v0[k, ax] -= 2 * eps
        lm = oinv.loss(pb, v0, amp, target)
        v0[k, ax] += eps
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - gv[k, ax]) <= 1e-3 * max(abs(fd), 1e-6 * np.abs(gv).max()), (k, ax, fd, gv[k, ax])
    eps_a = 3e-5
    fd = (oinv.loss(pb, v0, amp + eps_a, target) - oinv.loss(pb, v0, amp - eps_a, target)) / (2 * eps_a)
    assert abs(fd - ga) <= 1e-3 * abs(fd), (fd, ga)
