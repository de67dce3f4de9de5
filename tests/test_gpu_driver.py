"""GPU test of the headless scene driver (FluidSystem::stepSimulate's loop):
frames of substeps with a reference-style sinusoidal sweep, per-frame state
files, and the same states as stepping the simulator by hand."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_driver_matches_manual_steps_and_dumps(pbf, cuda, tmp_path):
    import torch

    sc = pbf.scenes.dam_break(seed=5)
    sweep = pbf.driver.Sweep((-0.3, 0.0, 0.0), (0.0, 0.0, 0.0), w=0.2)
    with pbf.driver.SceneDriver(sc, substeps=2, sweep=sweep, dump_dir=tmp_path) as drv:
        drv.run(3)
        torch.cuda.synchronize()
        got = drv.state.pos.cpu().numpy()
    files = sorted(tmp_path.glob("frame_*.bin"))
    assert [f.name for f in files] == ["frame_000001.bin", "frame_000002.bin", "frame_000003.bin"]
    pos3, _, iid3 = pbf.scenes.load_state(files[-1])
    np.testing.assert_array_equal(pos3, got)
    st = pbf.ParticleState(sc.pos, sc.vel)
    with pbf.Simulator(sc.params, sc.ulim, sc.llim, sc.n) as sim:
        for frame in range(3):
            u, l = sweep.limits(sc.ulim, sc.llim, frame)
            for _ in range(2):
                sim.setLim(u, l)
                st.step(sim)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(st.pos.cpu().numpy(), got)
        np.testing.assert_array_equal(st.iid[: st.n].cpu().numpy().astype(np.uint32), iid3)


def test_driver_renders_frames(pbf, oracle, cuda, tmp_path):
    """One SSF image per frame; the last one equals the oracle's splat of the
    same state bit for bit (no smoothing, so the raw depth reaches shading)."""
    import torch

    sc = pbf.scenes.dam_break(seed=1)
    p = pbf.ssf_default_params(160, 120)
    pbf.ssf.look_at(p, (2.6, -3.2, 1.8), (0.5, -0.5, 0.5))
    p.smooth_niter = 0
    r = pbf.SSFRenderer(p)
    with pbf.driver.SceneDriver(sc, substeps=2, render_dir=tmp_path, renderer=r) as drv:
        drv.run(2)
        torch.cuda.synchronize()
        state = drv.state.pos.cpu().numpy()
        depth = r.images()["depth"].cpu().numpy()
    files = sorted(tmp_path.glob("frame_*.ppm"))
    assert [f.name for f in files] == ["frame_000001.ppm", "frame_000002.ppm"]
    assert files[-1].read_bytes().startswith(b"P6 160 120 255\n")
    zup = np.stack([state[:, 0], -state[:, 2], state[:, 1], state[:, 3]], 1).astype(np.float32)
    o = oracle.ssf_render(p, zup, prec="f32")
    np.testing.assert_array_equal(depth.view(np.uint32), o["depth_raw"].view(np.uint32))


def test_fluid_system_is_the_reference_application_loop(pbf, cuda):
    """driver.fluid_system(moving=True): the reference's DoubleDamSource scene
    with its default parameters, one step per frame, and its sweep
    ulim.x + 2 sin(0.05 frame) (fluids/FluidSystem.cpp:34-61, 99-120) -- the
    same states as stepping that scene by hand."""
    import math

    import torch

    with pbf.driver.fluid_system(moving=True) as drv:
        assert drv.scene.n == 32000 and drv.substeps == 1 and not drv.y_up
        drv.run(3)
        torch.cuda.synchronize()
        got = drv.state.pos.cpu().numpy()
        got_iid = drv.state.iid[: drv.state.n].cpu().numpy()
    sc = pbf.scenes.reference_double_dam()
    st = pbf.ParticleState(sc.pos, sc.vel)
    with pbf.Simulator(sc.params, sc.ulim, sc.llim, sc.n) as sim:
        for frame in range(3):
            phi = math.sin(0.05 * frame)
            sim.setLim((sc.ulim[0] + 2.0 * phi, sc.ulim[1], sc.ulim[2]), sc.llim)
            st.step(sim)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(st.pos.cpu().numpy(), got)
        np.testing.assert_array_equal(st.iid[: st.n].cpu().numpy(), got_iid)
