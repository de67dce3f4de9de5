"""GPU tests of grouped cells: particles piled at bitwise-identical positions
in cells holding >= 512 particles, the state the dam-break parameters drive
large scenes into.  The dense kernels then visit each distinct position of
such a cell once, with its multiplicity (pbf_internal.cuh: group tables), so
results equal the reference's up to rounding.

Bars: one step against the FP64 oracle within 1e-5 h (positions), the
density within 1e-6 relative and velocities within 1e-5 h / dt + 1e-5 |v|
where the step is well conditioned (clusters alone); where clusters touch
other particles, error percentiles within 1e-5 h + 3x those of the
reference-order float port; two runs bitwise identical; a batch holding the
scene bitwise equal to the scene alone.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import TOL_X, gpu_step, ref_params

pytestmark = pytest.mark.gpu


def clustered(pbf, seed=0, counts=(1500, 700, 300), touching=True):
    """A jittered lattice plus clusters of particles at identical positions
    (one cell of h = 0.1 holds all clusters).  touching: the clusters lie
    inside the lattice and within h of each other; otherwise each cluster is
    alone, farther than h from every other particle."""
    rng = np.random.default_rng(seed)
    lat = pbf.scenes.lattice((10, 8, 8), (0.1, 0.1, 0.1), rng)
    if touching:
        centres = [(0.331, 0.352, 0.347), (0.362, 0.352, 0.347), (0.348, 0.371, 0.333)]
    else:
        centres = [(0.65, 0.65, 0.15), (0.65, 0.15, 0.65), (0.72, 0.72, 0.72)]
    parts = [lat]
    vparts = [np.zeros_like(lat)]
    vparts[0][:, :3] = rng.normal(0, 0.05, size=(len(lat), 3))
    for c, k in zip(centres, counts):
        blk = np.zeros((k, 4), np.float32)
        blk[:, :3] = c
        parts.append(blk)
        v = np.zeros((k, 4), np.float32)
        v[:, :3] = rng.normal(0, 0.05, size=3)  # a collapsed cluster moves as one
        vparts.append(v)
    order = rng.permutation(sum(len(q) for q in parts))
    return np.concatenate(parts)[order], np.concatenate(vparts)[order].astype(np.float32)


def check_fp64(oracle, p, ulim, llim, pos, vel, got, conditioned=True):
    """Against the FP64 oracle.  conditioned=False (clusters within h of other
    particles: the clusters' huge densities make delta_p a sum of large terms
    that nearly cancel, so any float arithmetic lands far from FP64): the
    median, 99th percentile and maximum of the position and velocity errors
    within 1e-5 h (1e-5 h / dt) + 3x those of the reference-order float port
    of the same step."""
    iid = np.arange(len(pos), dtype=np.uint32)
    r = oracle.step(p, ulim, llim, pos.astype(np.float64), vel.astype(np.float64), iid, "f64")
    np.testing.assert_array_equal(got["iid"], r["iid"])
    err = np.abs(got["npos"][:, :3] - r["npos"][:, :3]).max(1)
    if conditioned:
        assert err.max() <= TOL_X
        assert np.all(np.abs(got["nvel"][:, :3] - r["nvel"][:, :3]) <= TOL_X / p.dt + 1e-5 * np.abs(r["nvel"][:, :3]))
        assert np.abs(got["rho"] - r["rho"]).max() <= 1e-6 * np.abs(r["rho"]).max()
    else:
        r32 = oracle.step(p, ulim, llim, pos, vel, iid, "f32")
        for k, tol in (("npos", TOL_X), ("nvel", TOL_X / p.dt)):
            e_gpu = np.abs(got[k][:, :3] - r[k][:, :3]).ravel()
            e_port = np.abs(r32[k][:, :3] - r[k][:, :3]).ravel()
            for q in (50, 99, 100):
                a, b = np.percentile(e_gpu, q), np.percentile(e_port, q)
                assert a <= tol + 3 * b, (k, q, a, b)


@pytest.mark.parametrize("niter", [1, 3])
def test_isolated_grouped_cells_match_fp64(pbf, oracle, cuda, niter):
    pos, vel = clustered(pbf, touching=False)
    p = ref_params(pbf, niter)
    box = ((0.8, 0.8, 0.8), (0.0, 0.0, 0.0))
    got = gpu_step(pbf, p, *box, pos, vel)
    check_fp64(oracle, p, *box, pos, vel, got)


@pytest.mark.parametrize("niter", [1, 3])
def test_touching_grouped_cells_match_fp64(pbf, oracle, cuda, niter):
    pos, vel = clustered(pbf)
    p = ref_params(pbf, niter)
    box = ((0.8, 0.8, 0.8), (0.0, 0.0, 0.0))
    got = gpu_step(pbf, p, *box, pos, vel)
    check_fp64(oracle, p, *box, pos, vel, got, conditioned=False)


@pytest.mark.parametrize("niter", [2, 4])
def test_corner_cluster_with_distinct_velocities(pbf, oracle, cuda, niter):
    """5,000 particles driven into a box corner at different speeds: the wall
    clamps many of them onto one point, so XSPH groups those by (position,
    density) and sums their different velocities in fixed point.  The pile's
    density makes the step ill-conditioned: the port-relative bar."""
    rng = np.random.default_rng(5)
    lat = pbf.scenes.lattice((6, 6, 6), (0.1, 0.1, 0.1), rng)
    k = 5000
    blk = np.zeros((k, 4), np.float32)
    blk[:, :3] = (0.79, 0.79, 0.79)
    pos = np.concatenate([lat, blk])
    vel = np.zeros_like(pos)
    vel[: len(lat), :3] = rng.normal(0, 0.05, size=(len(lat), 3))
    vel[len(lat):, :3] = rng.uniform(0.5, 2.0, size=(k, 3))
    order = rng.permutation(len(pos))
    pos, vel = pos[order], vel[order].astype(np.float32)
    p = ref_params(pbf, niter)
    box = ((0.8, 0.8, 0.8), (0.0, 0.0, 0.0))
    got = gpu_step(pbf, p, *box, pos, vel)
    check_fp64(oracle, p, *box, pos, vel, got, conditioned=False)


@pytest.mark.parametrize("niter", [1, 3])
def test_grouped_cells_with_nonfinite_neighbours(pbf, oracle, cuda, niter):
    """Isolated clusters plus particles with NaN or infinite velocities next
    to them: the reference's NaN poisoning then reaches the clusters' windows
    and the exact rules run per group.  The non-finite entries of positions,
    velocities and densities match the FP64 oracle's exactly; finite
    positions within 1e-5 h + 3x the reference-order float port's error."""
    pos, vel = clustered(pbf, seed=6, touching=False)
    rng = np.random.default_rng(7)
    for c in [(0.65, 0.65, 0.15), (0.72, 0.72, 0.72)]:
        near = np.zeros((3, 4), np.float32)
        near[:, :3] = np.asarray(c) + rng.uniform(-0.05, 0.05, size=(3, 3))
        bad = np.zeros((3, 4), np.float32)
        bad[:, :3] = [[np.nan, 0.0, 0.0], [np.inf, 0.0, 0.0], [0.0, -np.inf, np.nan]]
        pos = np.concatenate([pos, near])
        vel = np.concatenate([vel, bad])
    p = ref_params(pbf, niter)
    box = ((0.8, 0.8, 0.8), (0.0, 0.0, 0.0))
    got = gpu_step(pbf, p, *box, pos, vel)
    iid = np.arange(len(pos), dtype=np.uint32)
    r = oracle.step(p, *box, pos.astype(np.float64), vel.astype(np.float64), iid, "f64")
    np.testing.assert_array_equal(got["iid"], r["iid"])
    for k in ("npos", "nvel"):
        np.testing.assert_array_equal(np.isfinite(got[k][:, :3]), np.isfinite(r[k][:, :3]), err_msg=k)
    np.testing.assert_array_equal(np.isfinite(got["rho"]), np.isfinite(r["rho"]))
    fin = np.isfinite(r["npos"][:, :3])
    r32 = oracle.step(p, *box, pos, vel, iid, "f32")
    port = np.abs(r32["npos"][:, :3][fin] - r["npos"][:, :3][fin]).max()
    assert np.abs(got["npos"][:, :3][fin] - r["npos"][:, :3][fin]).max() <= TOL_X + 3 * port


@pytest.mark.parametrize("distinct", [1000, 6000])
def test_grouped_cell_with_many_groups(pbf, oracle, cuda, distinct):
    """One cell holding `distinct` random positions, each taken by 1-3
    particles: groups ranked in shared memory (up to 4096 groups) or by the
    ordered block scan (more).  Error percentiles against FP64 as for
    touching clusters (the pile is ill-conditioned)."""
    rng = np.random.default_rng(distinct)
    base = rng.uniform(0.405, 0.495, size=(distinct, 3)).astype(np.float32)
    reps = rng.integers(1, 4, size=distinct)
    pts = np.repeat(base, reps, axis=0)
    pos = np.zeros((len(pts), 4), np.float32)
    pos[:, :3] = pts
    lat = pbf.scenes.lattice((6, 6, 6), (0.1, 0.1, 0.5), rng)
    pos = np.concatenate([pos, lat])
    vel = np.zeros_like(pos)
    pos = pos[rng.permutation(len(pos))]
    p = ref_params(pbf, 2)
    box = ((0.9, 0.9, 0.9), (0.0, 0.0, 0.0))
    got = gpu_step(pbf, p, *box, pos, vel)
    check_fp64(oracle, p, *box, pos, vel, got, conditioned=False)


def test_grouped_cells_deterministic(pbf, cuda):
    pos, vel = clustered(pbf, seed=2)
    p = ref_params(pbf, 4)
    box = ((0.8, 0.8, 0.8), (0.0, 0.0, 0.0))
    a = gpu_step(pbf, p, *box, pos, vel)
    b = gpu_step(pbf, p, *box, pos, vel)
    for k in ("npos", "nvel", "iid", "rho"):
        np.testing.assert_array_equal(a[k], b[k])


def test_grouped_cells_in_batch_equal_single(pbf, cuda):
    import torch

    pos, vel = clustered(pbf, seed=3)
    p = ref_params(pbf, 3)
    box = ((0.8, 0.8, 0.8), (0.0, 0.0, 0.0))
    single = gpu_step(pbf, p, *box, pos, vel)
    rng = np.random.default_rng(4)
    other = pbf.scenes.lattice((8, 8, 8), (0.0, 0.0, 0.0), rng)
    allpos = np.concatenate([other, pos])
    allvel = np.concatenate([np.zeros_like(other), vel])
    st = pbf.ParticleState(allpos, allvel)
    with pbf.Ensemble(p, [(0.8, 0.8, 0.8), box[0]], [(0.0, 0.0, 0.0), box[1]], [len(other), len(pos)]) as ens:
        st.step(ens)
        torch.cuda.synchronize()
        got = st.pos.cpu().numpy()[len(other):]
        iid = st.iid[: st.n].cpu().numpy()[len(other):] - len(other)
    np.testing.assert_array_equal(iid.astype(np.uint32), single["iid"])
    np.testing.assert_array_equal(got, single["npos"])
