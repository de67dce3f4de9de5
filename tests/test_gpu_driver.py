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
