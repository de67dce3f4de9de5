"""GPU tests of pbf_autotune / pbf_batch_autotune: the caller's state is left
untouched, the choice is one of the candidates, and steps after tuning still
match the FP64 oracle (the choices change only the order of window sums)."""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_parity import TOL_X, ref_params

pytestmark = pytest.mark.gpu

# the library's defaults of the tuning fields beyond window, dense-for-all, order and lanes
STAGE_DEFAULT = {"stage_sparse": 0, "stage_dense": 0, "queue_sparse": 1, "queue_dense": 1, "dense_split": 8,
                 "dense_interleave": 0}


def test_autotune_single(pbf, oracle, cuda):
    import torch

    sc = pbf.scenes.dam_break(seed=4)
    p = ref_params(pbf, 3)
    n = sc.n
    pos = torch.from_numpy(sc.pos).cuda()
    vel = torch.zeros_like(pos)
    iid = torch.arange(n, dtype=torch.int32, device="cuda")
    keep = (pos.clone(), vel.clone(), iid.clone())
    with pbf.Simulator(p, sc.ulim, sc.llim, n) as sim:
        t = sim.autotune(pos, vel, iid, steps=2)
        torch.cuda.synchronize()
        assert t["dense_window"] in (64, 128, 256, 512, 1024, 2048) and t["dense_all"] in (0, 1)
        assert t["order"] in (0, 1)
        assert t["ms_per_step"] > 0 and t["ms_default"] > 0 and t["ms_per_step"] <= t["ms_default"]
        for a, b in zip((pos, vel, iid), keep):
            assert torch.equal(a, b)
        npos, nvel = torch.empty_like(pos), torch.empty_like(vel)
        sim.step(pos, npos, vel, nvel, iid, n)
        torch.cuda.synchronize()
    r = oracle.step(p, sc.ulim, sc.llim, sc.pos.astype(np.float64), np.zeros((n, 4)), np.arange(n, dtype=np.uint32),
                    "f64")
    np.testing.assert_array_equal(iid.cpu().numpy().astype(np.uint32), r["iid"])
    assert np.abs(npos.cpu().numpy()[:, :3] - r["npos"][:, :3]).max() <= TOL_X


def test_autotune_batch(pbf, oracle, cuda):
    import torch

    rng = np.random.default_rng(2)
    scenes = []
    for s in range(4):
        a, b, c = (int(x) for x in rng.integers(6, 12, size=3))
        scenes.append((pbf.scenes.lattice((a, b, c), (0.0, 0.0, 0.0), rng), (2 * a * 0.05, 2 * b * 0.05, 2 * c * 0.05)))
    p = ref_params(pbf, 3)
    pos = np.concatenate([s[0] for s in scenes])
    st = pbf.ParticleState(pos, np.zeros_like(pos))
    counts = [len(s[0]) for s in scenes]
    with pbf.Ensemble(p, [s[1] for s in scenes], [(0.0, 0.0, 0.0)] * len(scenes), counts) as ens:
        t = ens.autotune(st.pos, st.vel, st.iid, steps=2)
        assert t["dense_window"] in (64, 128, 256, 512, 1024, 2048) and t["dense_all"] in (0, 1)
        st.step(ens)
        torch.cuda.synchronize()
        got = st.pos.cpu().numpy()
        iid = st.iid[: st.n].cpu().numpy()
    off = 0
    for (sp, ext), k in zip(scenes, counts):
        r = oracle.step(p, ext, (0.0, 0.0, 0.0), sp.astype(np.float64), np.zeros((k, 4)), np.arange(k, dtype=np.uint32),
                        "f64")
        np.testing.assert_array_equal(iid[off:off + k] - off, r["iid"])
        assert np.abs(got[off:off + k, :3] - r["npos"][:, :3]).max() <= TOL_X
        off += k


def test_set_tuning_round_trip(pbf, oracle, cuda):
    """pbf_set_tuning / pbf_get_tuning: the choice reads back, 0 / -1 restore the
    defaults, out-of-range values are refused, and a step at a set window still
    matches the FP64 oracle."""
    import torch

    sc = pbf.scenes.dam_break(seed=6)
    p = ref_params(pbf, 3)
    n = sc.n
    pos = torch.from_numpy(sc.pos).cuda()
    vel = torch.zeros_like(pos)
    iid = torch.arange(n, dtype=torch.int32, device="cuda")
    with pbf.Simulator(p, sc.ulim, sc.llim, n) as sim:
        assert sim.tuning() == {"dense_window": 512, "dense_all": -1, "order": 1, "bwd_lanes": 32, **STAGE_DEFAULT}
        sim.set_tuning(128, 0, 0)
        assert sim.tuning() == {"dense_window": 128, "dense_all": 0, "order": 0, "bwd_lanes": 32, **STAGE_DEFAULT}
        for bad in ((16, 0), (256, 2), (256, -2), (0, -1, 2), (0, -1, -2), (0, -1, 1, 4), (0, -1, 1, 0, 4097),
                    (0, -1, 1, 0, -2), (0, -1, 1, 0, 0, 4097), (0, -1, 1, 0, -1, -1, 17),
                    (0, -1, 1, 0, -1, -1, 0, 9), (0, -1, 1, 0, -1, -1, 0, 0, 3),
                    (0, -1, 1, 0, -1, -1, 0, 0, 0, 2)):
            with pytest.raises(pbf.PbfError):
                sim.set_tuning(*bad)
        assert sim.tuning() == {"dense_window": 128, "dense_all": 0, "order": 0, "bwd_lanes": 32, **STAGE_DEFAULT}
        npos, nvel = torch.empty_like(pos), torch.empty_like(vel)
        sim.step(pos, npos, vel, nvel, iid, n)
        torch.cuda.synchronize()
        sim.set_tuning(0, -1)
        assert sim.tuning() == {"dense_window": 512, "dense_all": -1, "order": 1, "bwd_lanes": 32, **STAGE_DEFAULT}
    r = oracle.step(p, sc.ulim, sc.llim, sc.pos.astype(np.float64), np.zeros((n, 4)), np.arange(n, dtype=np.uint32),
                    "f64")
    np.testing.assert_array_equal(iid.cpu().numpy().astype(np.uint32), r["iid"])
    assert np.abs(npos.cpu().numpy()[:, :3] - r["npos"][:, :3]).max() <= TOL_X
