"""GPU test of the reference application's own scene (fluids/FluidSystem.cpp:34-61):
the DoubleDamSource state of 32,000 particles, bit for bit as the reference
builds it, stepped with the reference's default parameters (z up, dt 0.0083).

Its heavily overlapping start (jitter scaled by the start coordinate, up to 3.6
lattice spacings) makes one step ill-conditioned for any float arithmetic, so
the bar is the port-relative one: cell order bit-exact against the FP64
oracle; median, 99th percentile and maximum of the position and velocity
errors within 1e-5 h (1e-5 h / dt) + 3x those of the reference-order float
port."""
from __future__ import annotations

import pytest

from test_gpu_groups import check_fp64
from test_gpu_parity import gpu_step

pytestmark = pytest.mark.gpu


def test_reference_double_dam_one_step(pbf, oracle, cuda):
    sc = pbf.scenes.reference_double_dam()
    got = gpu_step(pbf, sc.params, sc.ulim, sc.llim, sc.pos, sc.vel)
    check_fp64(oracle, sc.params, sc.ulim, sc.llim, sc.pos, sc.vel, got, conditioned=False)
