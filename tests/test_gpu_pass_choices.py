"""GPU tests of the neighbour passes' tunable choices beyond the dense window
(pbf_tuning): shared-memory staging (stage_sparse / stage_dense: a block whose
particles share one column of cells copies the column runs of their windows
into shared memory with bulk asynchronous copies and reads candidate
positions there), the hit queues (queue_sparse / queue_dense) and the dense
kernel's warps per batch (dense_split).

Bars:
  * staging and the hit queues change nothing: on or off, in either kernel,
    bitwise the same states over many steps (the same candidates summed in
    the same order) -- on scenes that pile particles up (dam-break
    parameters) and on scenes at rest (the reference's parameters), single
    and batched;
  * no staging wait gives up (pbf_check_device);
  * a staged step, and a step at every dense split (which changes the order of
    window sums), match the FP64 oracle within 1e-5 h.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import TOL_X, ref_params

pytestmark = pytest.mark.gpu

OFF = {"stage_sparse": 0, "stage_dense": 0}
CHOICES = [{"stage_sparse": 1024, "stage_dense": 0}, {"stage_sparse": 0, "stage_dense": 1536},
           {"stage_sparse": 2048, "stage_dense": 4096}, {"queue_sparse": 16, "queue_dense": 8},
           {"queue_sparse": 4, "queue_dense": 2}]


def run_steps(pbf, scene, params, steps, tuning):
    import torch

    st = pbf.ParticleState(scene.pos, scene.vel)
    with pbf.Simulator(params, scene.ulim, scene.llim, scene.n) as sim:
        sim.set_tuning(**tuning)
        t = 0.0
        for _ in range(steps):
            ulim, llim = scene.limits_at(t)
            sim.setLim(ulim, llim)
            st.step(sim)
            t += params.dt
        torch.cuda.synchronize()
        sim.check_device()
        return st.pos.cpu().numpy(), st.vel.cpu().numpy(), st.iid[: st.n].cpu().numpy()


@pytest.mark.parametrize("dense_all", [1, 0])
@pytest.mark.parametrize("which", ["scene", "reference"])
def test_staging_is_bitwise_neutral(pbf, cuda, which, dense_all):
    """The 8,000-particle dam break over 40 steps: the dam-break parameters
    pile particles into cells of tens to hundreds (large windows, dense
    kernel), the reference's keep ~8 per cell; dense_all 0 sends windows under
    the dense window through the one-thread-per-particle kernel."""
    sc = pbf.scenes.dam_break(seed=3)
    p = sc.params if which == "scene" else ref_params(pbf)
    if which == "reference":
        p.dt = sc.params.dt
    base = run_steps(pbf, sc, p, 40, dict(OFF, dense_all=dense_all, dense_window=256))
    for ch in CHOICES:
        got = run_steps(pbf, sc, p, 40, dict(ch, dense_all=dense_all, dense_window=256))
        for a, b, name in zip(got, base, ("pos", "vel", "iid")):
            assert a.tobytes() == b.tobytes(), (which, dense_all, ch, name)


def test_staging_batch_is_bitwise_neutral(pbf, cuda):
    """Three scenes of uneven sizes in one batch: a staged block's particles
    share a scene as well as a column."""
    import torch

    scenes = [pbf.scenes.dam_break(seed=s) for s in range(2)] + [pbf.scenes.double_dam(seed=5)]
    p = scenes[0].params
    pos0 = np.concatenate([s.pos for s in scenes])

    def run(tuning):
        st = pbf.ParticleState(pos0, np.zeros_like(pos0))
        with pbf.Ensemble(p, [s.ulim for s in scenes], [s.llim for s in scenes], [s.n for s in scenes]) as ens:
            ens.set_tuning(**tuning)
            assert ens.tuning()["stage_dense"] == tuning["stage_dense"]
            for _ in range(20):
                st.step(ens)
            torch.cuda.synchronize()
            ens.check_device()
            return st.pos.cpu().numpy(), st.vel.cpu().numpy()

    base = run(dict(OFF, dense_all=0, dense_window=256))
    got = run({"stage_sparse": 1024, "stage_dense": 3072, "dense_all": 0, "dense_window": 256})
    for a, b in zip(got, base):
        assert a.tobytes() == b.tobytes()


def test_staged_step_matches_fp64(pbf, oracle, cuda):
    import torch

    sc = pbf.scenes.double_dam(seed=2)
    p = ref_params(pbf)
    n = sc.n
    pos = torch.from_numpy(sc.pos).cuda()
    vel = torch.zeros_like(pos)
    iid = torch.arange(n, dtype=torch.int32, device="cuda")
    npos, nvel = torch.empty_like(pos), torch.empty_like(vel)
    with pbf.Simulator(p, sc.ulim, sc.llim, n) as sim:
        sim.set_tuning(stage_sparse=2048, stage_dense=3072, dense_all=0, dense_window=128)
        sim.step(pos, npos, vel, nvel, iid, n)
        torch.cuda.synchronize()
        sim.check_device()
    r = oracle.step(p, sc.ulim, sc.llim, sc.pos.astype(np.float64), np.zeros((n, 4)), np.arange(n, dtype=np.uint32),
                    "f64")
    np.testing.assert_array_equal(iid.cpu().numpy().astype(np.uint32), r["iid"])
    assert np.abs(npos.cpu().numpy()[:, :3] - r["npos"][:, :3]).max() <= TOL_X


@pytest.mark.parametrize("split, interleave", [(1, 0), (2, 0), (4, 0), (8, 0), (2, 1), (8, 1)])
def test_dense_split_step_matches_fp64(pbf, oracle, cuda, split, interleave):
    import torch

    sc = pbf.scenes.dam_break(seed=7)
    p = ref_params(pbf)
    n = sc.n
    pos = torch.from_numpy(sc.pos).cuda()
    vel = torch.zeros_like(pos)
    iid = torch.arange(n, dtype=torch.int32, device="cuda")
    npos, nvel = torch.empty_like(pos), torch.empty_like(vel)
    with pbf.Simulator(p, sc.ulim, sc.llim, n) as sim:
        sim.set_tuning(dense_all=1, dense_split=split, dense_interleave=interleave)
        assert sim.tuning()["dense_split"] == split and sim.tuning()["dense_interleave"] == interleave
        sim.step(pos, npos, vel, nvel, iid, n)
        torch.cuda.synchronize()
    r = oracle.step(p, sc.ulim, sc.llim, sc.pos.astype(np.float64), np.zeros((n, 4)), np.arange(n, dtype=np.uint32),
                    "f64")
    np.testing.assert_array_equal(iid.cpu().numpy().astype(np.uint32), r["iid"])
    assert np.abs(npos.cpu().numpy()[:, :3] - r["npos"][:, :3]).max() <= TOL_X
