"""GPU tests of the batched ensemble (pbf_batch_*): every scene of a batch
matches the same scene stepped alone (bit-exact order, positions within
1e-5 h; bitwise when no window is dense) and the FP64 oracle."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_X = 1e-5 * 0.1


def small_scenes(pbf, count=5, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        a, b, c = (int(x) for x in rng.integers(6, 14, size=3))
        pos = pbf.scenes.lattice((a, b, c), (0.0, 0.0, 0.0), rng)
        ext = (2 * a * 0.05, 2 * b * 0.05, 2 * c * 0.05)
        out.append((pos, ext))
    return out


def ref_params(pbf, niter=3):
    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    p.niter = niter
    return p


def run_batch(pbf, p, scenes, steps, walls=None):
    import torch

    pos = np.concatenate([s[0] for s in scenes])
    st = pbf.ParticleState(pos, np.zeros_like(pos))
    with pbf.Ensemble(p, [s[1] for s in scenes], [(0.0, 0.0, 0.0)] * len(scenes), [len(s[0]) for s in scenes]) as ens:
        for k in range(steps):
            if walls:
                for sc, fn in walls.items():
                    u = list(scenes[sc][1])
                    u[0] = fn(k)
                    ens.setLim(sc, u, (0.0, 0.0, 0.0))
            st.step(ens)
        rho = ens.density()
        torch.cuda.synchronize()
        return st.pos.cpu().numpy(), st.vel.cpu().numpy(), st.iid[: st.n].cpu().numpy(), rho.cpu().numpy()


def run_single(pbf, p, pos, ext, steps, wall=None):
    import torch

    st = pbf.ParticleState(pos, np.zeros_like(pos))
    with pbf.Simulator(p, ext, (0.0, 0.0, 0.0), len(pos)) as sim:
        for k in range(steps):
            if wall:
                u = list(ext)
                u[0] = wall(k)
                sim.setLim(u, (0.0, 0.0, 0.0))
            st.step(sim)
        rho = sim.density(len(pos))
        torch.cuda.synchronize()
        return st.pos.cpu().numpy(), st.vel.cpu().numpy(), st.iid[: st.n].cpu().numpy(), rho.cpu().numpy()


def test_batch_matches_single_scenes(pbf, cuda):
    p = ref_params(pbf)
    scenes = small_scenes(pbf)
    walls = {1: lambda k, e=scenes[1][1][0]: e - 0.03 * k}
    bpos, bvel, biid, brho = run_batch(pbf, p, scenes, 4, walls)
    off = 0
    for s, (pos, ext) in enumerate(scenes):
        n = len(pos)
        spos, svel, siid, srho = run_single(pbf, p, pos, ext, 4, walls.get(s))
        np.testing.assert_array_equal(biid[off:off + n] - off, siid)  # batch iids are global
        np.testing.assert_array_equal(bpos[off:off + n], spos)
        np.testing.assert_array_equal(bvel[off:off + n], svel)
        np.testing.assert_array_equal(brho[off:off + n], srho)
        off += n


def test_batch_scenes_match_fp64(pbf, oracle, cuda):
    p = ref_params(pbf, 4)
    scenes = small_scenes(pbf, count=4, seed=9)
    bpos, _, biid, _ = run_batch(pbf, p, scenes, 1)
    off = 0
    for pos, ext in scenes:
        n = len(pos)
        ref = oracle.step(p, ext, (0.0, 0.0, 0.0), pos, np.zeros_like(pos), np.arange(n, dtype=np.uint32), prec="f64")
        np.testing.assert_array_equal(biid[off:off + n] - off, ref["iid"])
        assert np.abs(bpos[off:off + n, :3] - ref["npos"][:, :3]).max() <= TOL_X
        off += n


def test_batch_with_dense_scene(pbf, cuda):
    """A dense scene (dense kernels) next to sparse ones: each scene still
    matches its single-scene run within 1e-5 h, order bit-exact."""
    rng = np.random.default_rng(5)
    dense = pbf.scenes.lattice((12, 12, 12), (0.3, 0.3, 0.3), rng, spacing=0.02, jitter=0.002)
    scenes = [small_scenes(pbf, 1, seed=1)[0], (dense, (1.0, 1.0, 1.0)), small_scenes(pbf, 1, seed=2)[0]]
    p = ref_params(pbf, 2)
    p.pho0 = pbf.scenes.rest_density(0.1, 0.02)
    bpos, _, biid, _ = run_batch(pbf, p, scenes, 1)
    off = 0
    for pos, ext in scenes:
        n = len(pos)
        spos, _, siid, _ = run_single(pbf, p, pos, ext, 1)
        np.testing.assert_array_equal(biid[off:off + n] - off, siid)
        assert np.abs(bpos[off:off + n, :3] - spos[:, :3]).max() <= TOL_X
        off += n


def test_batch_errors(pbf, cuda):
    p = ref_params(pbf)
    with pytest.raises(pbf.PbfError):
        pbf.Ensemble(p, [(1.0, 1.0, 1.0)], [(0.0, 0.0, 0.0)], [-1])
    with pbf.Ensemble(p, [(1.0, 1.0, 1.0), (0.5, 0.5, 0.5)], [(0.0, 0.0, 0.0)] * 2, [10, 5]) as ens:
        with pytest.raises(pbf.PbfError) as e:
            ens.setLim(2, (1.0, 1.0, 1.0), (0.0, 0.0, 0.0))
        assert e.value.status == pbf.PBF_ERR_INVALID_ARG
        with pytest.raises(pbf.PbfError) as e:
            ens.setLim(0, (30.0, 30.0, 30.0), (0.0, 0.0, 0.0))
        assert e.value.status == pbf.PBF_ERR_CAPACITY
        with pytest.raises(pbf.PbfError) as e:
            ens.density()
        assert e.value.status == pbf.PBF_ERR_NOT_READY
