"""CPU test of the oracle's FP64 density grid (the inverse problem's loss) and
its adjoint against central finite differences."""
from __future__ import annotations

import numpy as np


def test_density_grid_adjoint_matches_finite_differences(pbf, oracle):
    rng = np.random.default_rng(4)
    pos = pbf.scenes.lattice((6, 5, 4), (0.2, 0.1, 0.1), rng).astype(np.float64)
    lo, hi, dims, h = (0.0, 0.0, 0.0), (1.0, 0.6, 0.6), (10, 6, 6), 0.1
    target = rng.uniform(0, 3000, size=dims)

    def loss(p):
        d = oracle.density_grid(p, lo, hi, dims, h)
        return float(((d - target) ** 2).sum())

    g_grid = 2.0 * (oracle.density_grid(pos, lo, hi, dims, h) - target)
    g = oracle.density_grid_backward(pos, lo, hi, dims, h, g_grid)
    assert np.abs(g).max() > 0
    eps = 1e-6
    for _ in range(24):
        k, ax = int(rng.integers(len(pos))), int(rng.integers(3))
        x0 = pos[k, ax]
        pos[k, ax] = x0 + eps
        lp = loss(pos)
        pos[k, ax] = x0 - eps
        lm = loss(pos)
        pos[k, ax] = x0
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k, ax]) <= 1e-5 * max(abs(fd), 1.0), (fd, g[k, ax])


def test_density_grid_of_lattice_is_near_rest_density(pbf, oracle):
    """Inside an unjittered lattice the node density is close to the lattice's rest density."""
    rng = np.random.default_rng(0)
    pos = pbf.scenes.lattice((20, 20, 20), (0.0, 0.0, 0.0), rng, jitter=0.0)
    d = oracle.density_grid(pos, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (10, 10, 10), 0.1)
    inner = d[3:7, 3:7, 3:7]
    rho0 = pbf.scenes.rest_density()
    assert np.all(np.abs(inner / rho0 - 1) < 0.1)
