"""CPU tests of the headless scene sources and their parameters."""
from __future__ import annotations

import math

import numpy as np
import pytest


def test_rest_density_is_the_lattice_poly6_sum(pbf):
    rho = pbf.scenes.rest_density()
    h, d = 0.1, 0.05
    coef = 315.0 / (64.0 * math.pi * h ** 9)
    # 27 sites with r < h in a cubic lattice of spacing h/2: 1 + 6 + 12 + 8
    want = coef * (h * h) ** 3 + 6 * coef * (h * h - d * d) ** 3 + 12 * coef * (h * h - 2 * d * d) ** 3 \
        + 8 * coef * (h * h - 3 * d * d) ** 3
    assert abs(rho - want) < 1e-3
    assert abs(rho - 8078.20) < 0.01


def test_scene_sizes_and_boxes(pbf):
    s = pbf.scenes
    assert s.inverse_scene().n == 15625
    for scene, n in ((s.dam_break(), 8000), (s.double_dam(), 32768)):
        assert scene.n == n
        assert scene.pos.dtype == np.float32 and scene.pos.shape == (n, 4)
        assert np.all(scene.pos[:, :3] > np.array(scene.llim)) and np.all(scene.pos[:, :3] < np.array(scene.ulim))
        assert np.all(scene.vel == 0)
    big = s.large_sweep()
    assert big.n == 1 << 20
    assert big.ulim == (12.8, 6.4, 6.4)


def test_lattice_jitter_is_seeded_and_bounded(pbf):
    s = pbf.scenes
    a, b = s.dam_break(seed=7), s.dam_break(seed=7)
    np.testing.assert_array_equal(a.pos, b.pos)
    assert not np.array_equal(a.pos, s.dam_break(seed=8).pos)
    ii = np.arange(20)
    grid = 0.025 + 0.05 * ii
    dev = a.pos[:, 0].reshape(20, 400) - grid[:, None]
    assert np.abs(dev).max() <= 0.005 + 1e-6


def test_double_dam_against_opposite_walls(pbf):
    sc = pbf.scenes.double_dam()
    left, right = sc.pos[:16384], sc.pos[16384:]
    assert left[:, 0].max() < 0.81 and right[:, 0].min() > 3.2 - 0.81


def test_sweep_wall(pbf):
    s = pbf.scenes
    assert s.sweep_wall_x(0.0) == 12.8
    assert abs(s.sweep_wall_x(2.0) - 9.6) < 1e-12
    assert abs(s.sweep_wall_x(4.0) - 12.8) < 1e-12
    u, l = s.large_sweep().limits_at(1.0)
    assert abs(u[0] - 11.2) < 1e-12 and l == (0.0, 0.0, 0.0)


def test_ensemble(pbf):
    scenes = pbf.scenes.ensemble(seed=0)
    assert len(scenes) == 256
    ns = np.array([sc.n for sc in scenes])
    assert ns.min() >= 12 ** 3 and ns.max() <= 40 ** 3
    assert 3.5e6 < ns.sum() < 5.5e6
    for sc in scenes[:8]:
        assert np.all(sc.pos[:, :3] < np.array(sc.ulim))


def test_scene_params(pbf):
    p = pbf.scenes.scene_params()
    assert p.niter == 4 and abs(p.pho0 - 8078.2) < 0.01
    assert p.lambda_eps == 100.0 and abs(p.delta_q - 0.02) < 1e-7 and abs(p.k_corr - 0.1) < 1e-7
    assert p.n_corr == 4.0 and abs(p.c_XSPH - 0.01) < 1e-9
    assert list(p.up) == [0.0, 1.0, 0.0]
    assert abs(p.dt - 1.0 / 120.0) < 1e-9


def test_state_file_round_trip(pbf, tmp_path):
    s = pbf.scenes
    sc = s.dam_break(seed=2)
    rng = np.random.default_rng(0)
    vel = rng.normal(size=(sc.n, 3)).astype(np.float32)
    iid = rng.permutation(sc.n).astype(np.uint32)
    path = tmp_path / "state.bin"
    s.save_state(path, sc.pos, vel, iid)
    assert path.stat().st_size == 16 + sc.n * 36
    pos2, vel2, iid2 = s.load_state(path)
    np.testing.assert_array_equal(pos2, sc.pos)
    np.testing.assert_array_equal(vel2[:, :3], vel)
    assert np.all(vel2[:, 3] == 0)
    np.testing.assert_array_equal(iid2, iid)
    path.write_bytes(path.read_bytes()[:-4])
    with pytest.raises(ValueError):
        s.load_state(path)


def test_msvc_rand_known_answers(pbf):
    """The Microsoft C runtime's rand(): the first values after the default seed 1."""
    r = pbf.scenes.MsvcRand(1)
    assert [r.rand() for _ in range(10)] == [41, 18467, 6334, 26500, 19169, 15724, 11478, 29358, 26962, 24464]


def test_reference_double_dam_layout(pbf):
    """fluids/FluidSystem.cpp:55-61, fluids/DoubleDamSource.cpp:5-31: 2 x 20 x 20 x 40
    particles, the first at (llim + d/2) + 0.1 (s r1, s r2, s r3) with the first
    three draws after srand(27), the cubes' x steps negative (ulim.x < llim.x
    for the first cube, as the reference writes it), all inside the box."""
    sc = pbf.scenes.reference_double_dam()
    assert sc.n == 32000 and sc.ulim == (2.0, 2.0, 4.0) and sc.llim == (-2.0, -2.0, 0.0)
    assert list(sc.params.up) == [0.0, 0.0, 1.0] and sc.params.niter == 4
    f = np.float32
    r = pbf.scenes.MsvcRand(27)
    r1, r2, r3 = (f(1.0) * f(r.rand()) / f(32767) for _ in range(3))
    d = (f(-1.8) - (f(-1.8) + f(1.0) / f(20) * f(20))) / f(20)
    sx = (f(-1.8) + f(1.0) / f(20) * f(20)) + d / f(2)
    assert sc.pos[0, 0] == sx + f(0.1) * (sx * r1)
    assert np.all(sc.pos[:, :3] > np.array(sc.llim, np.float32)) and np.all(sc.pos[:, :3] < np.array(sc.ulim, np.float32))
    # first cube in x < 0, y > 0; second in x > 0, y < 0
    assert np.all(sc.pos[:16000, 0] < 0) and np.all(sc.pos[:16000, 1] > 0)
    assert np.all(sc.pos[16000:, 0] > 0) and np.all(sc.pos[16000:, 1] < 0)
    # the reference's jitter quirk: scaled by the start coordinate, up to 0.1 * sz = 0.1825 in z
    assert sc.pos[:, 2].max() > 3.9
    fc = pbf.scenes.reference_fixed_cube()
    assert fc.n == 27000 and np.all(fc.pos[:, :3] < np.array(fc.ulim, np.float32) + 0.2)


def test_reference_double_dam_oracle_step(pbf, oracle):
    """One step of the reference's own scene with its own parameters: the float
    port and the FP64 oracle give the same cell order; the heavily overlapping
    start (jitter up to 3.6 spacings in z) makes the step ill-conditioned, so
    positions agree to ~1e-3 h, not 1e-5 h."""
    sc = pbf.scenes.reference_double_dam()
    iid = np.arange(sc.n, dtype=np.uint32)
    r32 = oracle.step(sc.params, sc.ulim, sc.llim, sc.pos, sc.vel, iid, "f32")
    r64 = oracle.step(sc.params, sc.ulim, sc.llim, sc.pos.astype(np.float64), sc.vel.astype(np.float64), iid, "f64")
    np.testing.assert_array_equal(r32["iid"], r64["iid"])
    assert np.abs(r32["npos"][:, :3] - r64["npos"][:, :3]).max() < 1e-3


def test_reference_params_match_the_library_defaults(pbf):
    """scenes.reference_params (no library) and pbf_params_default agree bit for bit."""
    import ctypes

    a, b = pbf.scenes.reference_params(), pbf.default_params()
    assert ctypes.string_at(ctypes.addressof(a), ctypes.sizeof(a)) == \
        ctypes.string_at(ctypes.addressof(b), ctypes.sizeof(b))
