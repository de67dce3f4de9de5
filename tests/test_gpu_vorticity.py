"""GPU test of vorticity confinement (vorticity_eps > 0; the reference has
none, README.md:14): one step against the FP64 oracle's restatement of the
same formulas.  Positions are untouched by it; velocities within 1e-5 h / dt
+ 1e-5 |v|, except where |eta| is near zero and the normal's direction is
ill-conditioned: there the error may reach 3x the reference-order float
port's."""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import TOL_X, gpu_step, ref_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("eps", [1e-4, 1e-3])
def test_vorticity_matches_fp64(pbf, oracle, cuda, eps):
    sc = pbf.scenes.dam_break(seed=3)
    rng = np.random.default_rng(3)
    vel = np.zeros_like(sc.pos)
    vel[:, :3] = rng.normal(0, 0.3, size=(sc.n, 3))
    p = ref_params(pbf, 3)
    p.vorticity_eps = eps
    got = gpu_step(pbf, p, sc.ulim, sc.llim, sc.pos, vel)
    iid = np.arange(sc.n, dtype=np.uint32)
    r = oracle.step(p, sc.ulim, sc.llim, sc.pos.astype(np.float64), vel.astype(np.float64), iid, "f64")
    r32 = oracle.step(p, sc.ulim, sc.llim, sc.pos, vel, iid, "f32")
    np.testing.assert_array_equal(got["iid"], r["iid"])
    assert np.abs(got["npos"][:, :3] - r["npos"][:, :3]).max() <= TOL_X
    err = np.abs(got["nvel"][:, :3] - r["nvel"][:, :3])
    bar = TOL_X / p.dt + 1e-5 * np.abs(r["nvel"][:, :3]) + 3 * np.abs(r32["nvel"][:, :3] - r["nvel"][:, :3])
    assert np.all(err <= bar), (err.max(), int(np.sum(err > bar)))
    # the confinement does act
    p0 = ref_params(pbf, 3)
    plain = gpu_step(pbf, p0, sc.ulim, sc.llim, sc.pos, vel)
    assert np.abs(plain["nvel"] - got["nvel"]).max() > 1e-4


def test_vorticity_rejected_by_the_tape(pbf, cuda):
    sc = pbf.scenes.dam_break()
    p = ref_params(pbf, 2)
    p.vorticity_eps = 0.1
    with pbf.Simulator(p, sc.ulim, sc.llim, sc.n) as sim:
        with pytest.raises(pbf.PbfError):
            sim.tape(1)
