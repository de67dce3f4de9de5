"""Statistical parity over long runs: 300 frames (600 steps) of the 8,000-particle
dam break (32 jitter seeds) and of the 32,768-particle double dam break (32
seeds with the reference's parameters, 8 with the dam-break ones), against the
reference's own kernels (tests/golden/stats_*.npz, made by
tests/golden/make_stats.py).

Trajectories diverge chaotically (FP32 rounding differences grow, and the
fluid settles into one of several layered packings), so runs are compared
through the per-step mean and max of the compression max(C_i, 0),
C_i = rho_i / rho0 - 1, averaged over the 600 steps and the seeds:
  * the reference's own parameters: both within 1% of the reference, or within
    three combined standard errors of the seed means where those exceed 1%
    (the per-step maximum over 32,768 particles varies by ~3.6% from seed to
    seed, so 32 seeds resolve a difference of ~1.9% at three standard errors);
  * the dam-break parameters (the fluid collapses into dense clusters and the
    reference's seeds alone spread by +-30%): within three combined standard
    errors of the seed means.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def run_ours(pbf, p, sc, steps):
    from make_stats import constraint_stats

    st = pbf.ParticleState(sc.pos, sc.vel)
    out = np.zeros((steps, 3))
    with pbf.Simulator(p, sc.ulim, sc.llim, sc.n) as sim:
        for k in range(steps):
            st.step(sim)
            out[k] = constraint_stats(sim.density(sc.n).cpu().numpy(), float(p.pho0))
    return out


@pytest.fixture(scope="module")
def golden_path():
    import sys

    sys.path.insert(0, str(GOLDEN))
    yield
    sys.path.remove(str(GOLDEN))


@pytest.mark.parametrize("name", ["dam8k_refparams", "dam8k_sceneparams", "ddam32k_refparams",
                                  "ddam32k_sceneparams"])
def test_constraint_statistics_match_reference(pbf, cuda, golden_path, name):
    from make_stats import cases

    z = np.load(GOLDEN / f"stats_{name}.npz")
    ref, seeds, steps = z["stats"], [int(s) for s in z["seeds"]], int(z["steps"])
    ours = np.stack([run_ours(pbf, *cases(pbf, s)[name], steps) for s in seeds])
    assert np.count_nonzero(ours[:, :, 2]) == np.count_nonzero(ref[:, :, 2])
    for col, what in ((0, "mean C+"), (1, "max C+")):
        r_seed, o_seed = ref[:, :, col].mean(1), ours[:, :, col].mean(1)
        r, o = r_seed.mean(), o_seed.mean()
        se = np.sqrt(r_seed.var(ddof=1) / len(seeds) + o_seed.var(ddof=1) / len(seeds))
        if name.endswith("_refparams"):
            assert abs(o / r - 1) <= max(0.01, 3 * se / r), (what, o, r, se)
        else:
            assert abs(o - r) <= 3 * se, (what, o, r, se)
