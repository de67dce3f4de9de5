"""Headless scene sources: the particle lattices the solver is tested and
measured on, and their solver parameters.

The reference fills its buffers from ParticleSource subclasses
(fluids/ParticleSource.h:4-17; FixedCubeSource / DoubleDamSource generate
jittered lattices with srand(27), fluids/DoubleDamSource.cpp:5-21).  These
sources keep that interface idea (a source produces positions, velocities and
iids for a box) with seeded numpy jitter and y up:

  dam_break     8,000 particles: 20x20x20 lattice in a 2.0 x 1.0 x 1.0 box
  double_dam    32,768 particles: two 16x32x32 lattices at opposite x walls of
                a 3.2 x 1.6 x 1.6 box
  large_sweep   1,048,576 particles: 128x64x128 lattice in a 12.8 x 6.4 x 6.4
                box whose x-max wall moves as x_w(t) = 12.8 - 1.6 (1 - cos(2 pi t / 4 s))
  ensemble      256 independent a x b x c lattices, a, b, c uniform in [12, 40],
                each in its own (2a d, 2b d, 2c d) box
  inverse       15,625 particles: 25x25x25 lattice (spacing 0.04) in a 2.0 x 1.0 x 1.0 box
  clustered     1,048,576 particles: a 64^3 lattice plus six collapsed clusters
                in the large sweep's box (the grouped-cell profiling case)
  reference_double_dam / reference_fixed_cube
                the reference application's own sources, bit for bit: the same
                C-runtime generator seeded 27, the same float arithmetic and
                jitter quirk, z up, the reference's default parameters

Lattice spacing d = 0.05, jitter uniform +-0.005 per coordinate, velocities 0.
save_state / load_state keep a particle state (float4 positions, float4
velocities, uint32 iids) in one raw binary file for fixtures and restarts.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Tuple

import numpy as np

from ._abi import PbfParams

SPACING = 0.05
JITTER = 0.005
H = 0.1
FRAME_DT = 1.0 / 60.0
SUBSTEPS = 2


def rest_density(h: float = H, spacing: float = SPACING) -> float:
    """Poly6 density (mass 1) of a particle in an unjittered cubic lattice,
    summed in float64 over every lattice site with r < h, self included."""
    m = int(math.ceil(h / spacing)) + 1
    coef = 315.0 / (64.0 * math.pi * h ** 9)
    rho = 0.0
    for a in range(-m, m + 1):
        for b in range(-m, m + 1):
            for c in range(-m, m + 1):
                r2 = (a * a + b * b + c * c) * spacing * spacing
                if r2 < h * h * (1 - 1e-12):
                    rho += coef * (h * h - r2) ** 3
    return float(np.float32(rho))


def reference_params() -> PbfParams:
    """The reference's solver defaults (fluids/FluidSystem.cpp:15-25; LIM_EPS,
    KERNAL_EPS and MAX_DP from fluids/helper.h:5-9), z up as the reference's
    advect_kernel has it: the values pbf_params_default fills in, set here
    without the library so that building a scene (the CPU reference arm of
    bench.py does) loads no CUDA code.  tests/test_scenes.py checks the two
    agree field for field."""
    p = PbfParams()
    p.niter = 4
    p.pho0 = 8000.0
    p.g = 9.8
    p.h = 0.1
    p.dt = 0.0083
    p.lambda_eps = 1000.0
    p.delta_q = 0.3 * float(np.float32(0.1))  # (float)(0.3 * h), h the float 0.1
    p.k_corr = 0.001
    p.n_corr = 4.0
    p.k_boundaryDensity = 0.0
    p.c_XSPH = 0.5
    p.up[0], p.up[1], p.up[2] = 0.0, 0.0, 1.0
    p.lim_eps = 1e-3
    p.kernel_eps = 1e-4
    p.max_dp = 0.1
    p.vorticity_eps = 0.0
    return p


def scene_params(niter: int = 4) -> PbfParams:
    """Solver parameters of the dam-break scenes: h = 0.1, pho0 = lattice
    density, epsilon = 100, s_corr k = 0.1 n = 4 dq = 0.2 h, XSPH c = 0.01,
    gravity 9.8 along -y, dt = 1/120 s (a 1/60 s frame in 2 steps)."""
    p = reference_params()
    p.niter = niter
    p.h = H
    p.pho0 = rest_density()
    p.lambda_eps = 100.0
    p.delta_q = 0.2 * H
    p.k_corr = 0.1
    p.n_corr = 4.0
    p.k_boundaryDensity = 0.0
    p.c_XSPH = 0.01
    p.g = 9.8
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    p.dt = FRAME_DT / SUBSTEPS
    return p


def lattice(counts: Tuple[int, int, int], origin, rng: np.random.Generator,
            spacing: float = SPACING, jitter: float = JITTER) -> np.ndarray:
    """(a*b*c, 4) float32 positions: origin + d/2 + index * d + U(-jitter, jitter),
    x slowest, z fastest (the reference's loop order, fluids/FixedCubeSource.cpp:12-20)."""
    a, b, c = counts
    ii, jj, kk = np.meshgrid(np.arange(a), np.arange(b), np.arange(c), indexing="ij")
    base = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], 1).astype(np.float64)
    p = np.asarray(origin, np.float64) + spacing / 2 + base * spacing
    p += rng.uniform(-jitter, jitter, size=p.shape)
    out = np.zeros((p.shape[0], 4), np.float32)
    out[:, :3] = p
    return out


@dataclass
class Scene:
    name: str
    pos: np.ndarray                      # (n, 4) float32
    vel: np.ndarray                      # (n, 4) float32
    ulim: Tuple[float, float, float]
    llim: Tuple[float, float, float]
    wall: Optional[Callable[[float], Tuple[Tuple[float, ...], Tuple[float, ...]]]] = None
    params: PbfParams = field(default_factory=scene_params)

    @property
    def n(self) -> int:
        return self.pos.shape[0]

    def limits_at(self, t: float):
        """(ulim, llim) at time t (the moving wall; static boxes ignore t)."""
        if self.wall is None:
            return self.ulim, self.llim
        return self.wall(t)


def _zeros_like(p):
    return np.zeros_like(p)


def dam_break(seed: int = 0, niter: int = 4) -> Scene:
    rng = np.random.default_rng(seed)
    pos = lattice((20, 20, 20), (0.0, 0.0, 0.0), rng)
    return Scene("dam_break_8k", pos, _zeros_like(pos), (2.0, 1.0, 1.0), (0.0, 0.0, 0.0),
                 params=scene_params(niter))


def double_dam(seed: int = 0, niter: int = 4) -> Scene:
    rng = np.random.default_rng(seed)
    a = lattice((16, 32, 32), (0.0, 0.0, 0.0), rng)
    b = lattice((16, 32, 32), (3.2 - 16 * SPACING, 0.0, 0.0), rng)
    pos = np.concatenate([a, b])
    return Scene("double_dam_32k", pos, _zeros_like(pos), (3.2, 1.6, 1.6), (0.0, 0.0, 0.0),
                 params=scene_params(niter))


# ---- the reference application's own sources -------------------------------------------


class MsvcRand:
    """The C runtime rand() the reference application draws its jitter from
    (a Windows / Visual Studio build, fluids/fluids.vcxproj): the published
    linear congruential generator of the Microsoft C runtime, state = state *
    214013 + 2531011 (mod 2^32), rand() = bits 16..30 of the state, RAND_MAX =
    32767; srand(seed) sets the state."""

    RAND_MAX = 32767

    def __init__(self, seed: int = 1):
        self.state = seed & 0xFFFFFFFF

    def rand(self) -> int:
        self.state = (self.state * 214013 + 2531011) & 0xFFFFFFFF
        return (self.state >> 16) & 0x7FFF


def _reference_cube(llim, d, ns, rng: MsvcRand, out: list) -> None:
    """generate_cube / FixedCubeSource::initialize (fluids/DoubleDamSource.cpp:5-21,
    fluids/FixedCubeSource.cpp:6-26) in float32 and the same order: x, y, z start
    at llim + d / 2 and step by d (accumulated), x slowest; each particle gets
    0.1 (sx r1, sy r2, sz r3) added, r = 1.f * rand() / RAND_MAX, the jitter
    scaled by the start coordinate s (the reference's quirk)."""
    f = np.float32
    sx, sy, sz = (f(llim[a]) + f(d[a]) / f(2) for a in range(3))
    x = sx
    for _ in range(ns[0]):
        y = sy
        for _ in range(ns[1]):
            z = sz
            for _ in range(ns[2]):
                r1 = f(1.0) * f(rng.rand()) / f(MsvcRand.RAND_MAX)
                r2 = f(1.0) * f(rng.rand()) / f(MsvcRand.RAND_MAX)
                r3 = f(1.0) * f(rng.rand()) / f(MsvcRand.RAND_MAX)
                out.append((x + f(0.1) * (sx * r1), y + f(0.1) * (sy * r2), z + f(0.1) * (sz * r3)))
                z = z + f(d[2])
            y = y + f(d[1])
        x = x + f(d[0])


def _reference_spacing(ulim, llim, ns):
    """m_d = (ulim - llim) / ns per axis in float32 (fluids/DoubleDamSource.h:11-21)."""
    f = np.float32
    return [(f(ulim[a]) - f(llim[a])) / f(ns[a]) for a in range(3)]


def reference_double_dam() -> Scene:
    """The reference application's default scene (fluids/FluidSystem.cpp:34-61):
    DoubleDamSource of two 20 x 20 x 40 cubes (32,000 particles, srand(27)) in the
    box [-2, 2] x [-2, 2] x [0, 4], z up, the reference's default solver
    parameters (dt 0.0083, one step per frame).  Its second cube is generated
    with the first cube's ulim (fluids/DoubleDamSource.cpp:31), which
    generate_cube does not use.  The reference's boundary sweep, when switched
    on, is driver.Sweep((2, 0, 0), (0, 0, 0), w=0.05) (fluids/FluidSystem.cpp:36-38)."""
    f = np.float32
    dd = f(1.0) / f(20)
    d1, d2, d3 = dd * f(20), dd * f(20), dd * f(40)
    ulim1 = (f(-1.8), f(1.8), f(3.8))
    llim1 = (f(-1.8) + d1, f(1.8) - d2, f(3.8) - d3)
    ulim2 = (f(1.8) - d1, f(-1.8) + d2, f(3.8))
    llim2 = (f(1.8), f(-1.8), f(3.8) - d3)
    ns = (20, 20, 40)
    rng = MsvcRand(27)
    pts: list = []
    _reference_cube(llim1, _reference_spacing(ulim1, llim1, ns), ns, rng, pts)
    _reference_cube(llim2, _reference_spacing(ulim2, llim2, ns), ns, rng, pts)
    pos = np.zeros((len(pts), 4), np.float32)
    pos[:, :3] = np.asarray(pts, np.float32)
    return Scene("reference_double_dam_32k", pos, _zeros_like(pos), (2.0, 2.0, 4.0), (-2.0, -2.0, 0.0),
                 params=reference_params())


def reference_fixed_cube() -> Scene:
    """The reference's single-cube alternative (commented out in
    fluids/FluidSystem.cpp:47-52): FixedCubeSource of 30 x 30 x 30 particles
    below (1.8, 1.8, 3.8), srand(27), the same box and parameters as
    reference_double_dam."""
    f = np.float32
    dd = f(1.0) / f(20)
    d1 = d2 = d3 = dd * f(30)
    ulim = (f(1.8), f(1.8), f(3.8))
    llim = (f(1.8) - d1, f(1.8) - d2, f(3.8) - d3)
    ns = (30, 30, 30)
    pts: list = []
    _reference_cube(llim, _reference_spacing(ulim, llim, ns), ns, MsvcRand(27), pts)
    pos = np.zeros((len(pts), 4), np.float32)
    pos[:, :3] = np.asarray(pts, np.float32)
    return Scene("reference_fixed_cube_27k", pos, _zeros_like(pos), (2.0, 2.0, 4.0), (-2.0, -2.0, 0.0),
                 params=reference_params())


def sweep_wall_x(t: float) -> float:
    """x-max wall of the large sweep: 12.8 - 1.6 (1 - cos(2 pi t / 4 s))."""
    return 12.8 - 1.6 * (1.0 - math.cos(2.0 * math.pi * t / 4.0))


def large_sweep(seed: int = 0, niter: int = 4) -> Scene:
    rng = np.random.default_rng(seed)
    pos = lattice((128, 64, 128), (0.0, 0.0, 0.0), rng)

    def wall(t: float):
        return (sweep_wall_x(t), 6.4, 6.4), (0.0, 0.0, 0.0)

    return Scene("large_sweep_1m", pos, _zeros_like(pos), (12.8, 6.4, 6.4), (0.0, 0.0, 0.0), wall=wall,
                 params=scene_params(niter))


def clustered(seed: int = 0, niter: int = 4) -> Scene:
    """1,048,576 particles in the 12.8 x 6.4 x 6.4 box in the state the
    dam-break parameters drive large scenes into: a 64^3 lattice of fluid
    plus 786,432 particles collapsed onto six points (cells of 131,072
    particles at one position: three box corners, two wall points, one point
    in the fluid), each cluster moving as one.  The profiling case of the
    grouped-cell path."""
    rng = np.random.default_rng(seed)
    lat = lattice((64, 64, 64), (0.0, 0.0, 0.0), rng)
    pts = [(12.799, 0.001, 0.001), (12.799, 0.001, 6.399), (0.001, 0.001, 6.399),
           (6.4, 0.001, 3.2), (12.799, 3.2, 3.2), (1.6, 1.2, 1.6)]
    k = 131072
    parts, vparts = [lat], [np.zeros_like(lat)]
    for c in pts:
        blk = np.zeros((k, 4), np.float32)
        blk[:, :3] = c
        parts.append(blk)
        v = np.zeros((k, 4), np.float32)
        v[:, :3] = rng.normal(0.0, 0.1, size=3)
        vparts.append(v)
    order = rng.permutation(sum(len(q) for q in parts))
    pos = np.concatenate(parts)[order]
    vel = np.concatenate(vparts)[order]
    return Scene("clustered_1m", pos, vel, (12.8, 6.4, 6.4), (0.0, 0.0, 0.0), params=scene_params(niter))


INVERSE_SPACING = 0.04


def inverse_scene(seed: int = 0, niter: int = 4) -> Scene:
    """15,625 particles (25^3 lattice) in a 2 x 1 x 1 box with the dam-break
    parameters.  The lattice spacing is 0.04, not 0.05: 25 particles at 0.05
    span 1.25, more than the box's 1.0 height and depth, while at 0.04 they
    fill it exactly (the fluid starts ~1.95x denser than rest and spreads
    into the free half of the box)."""
    rng = np.random.default_rng(seed)
    pos = lattice((25, 25, 25), (0.0, 0.0, 0.0), rng, spacing=INVERSE_SPACING)
    return Scene("inverse_15k", pos, _zeros_like(pos), (2.0, 1.0, 1.0), (0.0, 0.0, 0.0),
                 params=scene_params(niter))


def ensemble(seed: int = 0, count: int = 256, niter: int = 4) -> List[Scene]:
    rng = np.random.default_rng(seed)
    dims = rng.integers(12, 41, size=(count, 3))
    out = []
    for s, (a, b, c) in enumerate(dims):
        pos = lattice((int(a), int(b), int(c)), (0.0, 0.0, 0.0), rng)
        ext = (2 * a * SPACING, 2 * b * SPACING, 2 * c * SPACING)
        out.append(Scene(f"ensemble_{s}", pos, _zeros_like(pos), tuple(float(e) for e in ext),
                         (0.0, 0.0, 0.0), params=scene_params(niter)))
    return out


SCENES = {
    "dam_break": dam_break,
    "double_dam": double_dam,
    "large_sweep": large_sweep,
    "clustered": clustered,
    "inverse": inverse_scene,
}


# ---- particle state files ---------------------------------------------------------------

_STATE_MAGIC = b"PBFSTATE"


def save_state(path, pos, vel, iid) -> None:
    """Write n particles to `path`: the 8-byte magic, n (uint64, little
    endian), then pos (n x 4 float32), vel (n x 4 float32), iid (n uint32),
    all little endian.  Accepts numpy arrays or CUDA tensors (copied to the
    host); (n, 3) arrays get w = 0."""
    def host(a, dtype, cols):
        a = a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)
        a = np.asarray(a, dtype=dtype)
        if cols and a.shape[1] == 3:
            a = np.concatenate([a, np.zeros((a.shape[0], 1), dtype)], 1)
        return np.ascontiguousarray(a)
    p = host(pos, "<f4", 4)
    v = host(vel, "<f4", 4)
    i = host(iid, "<u4", 0).reshape(-1)
    n = p.shape[0]
    if v.shape != (n, 4) or i.shape != (n,):
        raise ValueError("pos, vel and iid must hold the same number of particles")
    with open(path, "wb") as f:
        f.write(_STATE_MAGIC)
        f.write(np.uint64(n).astype("<u8").tobytes())
        f.write(p.tobytes())
        f.write(v.tobytes())
        f.write(i.tobytes())


def load_state(path):
    """Read a file written by save_state: (pos (n, 4) float32, vel (n, 4)
    float32, iid (n,) uint32)."""
    with open(path, "rb") as f:
        if f.read(8) != _STATE_MAGIC:
            raise ValueError(f"{path}: not a particle state file")
        n = int(np.frombuffer(f.read(8), "<u8")[0])
        body = f.read()
    need = n * (16 + 16 + 4)
    if len(body) != need:
        raise ValueError(f"{path}: {len(body)} bytes of particle data, expected {need}")
    pos = np.frombuffer(body, "<f4", n * 4, 0).reshape(n, 4).astype(np.float32)
    vel = np.frombuffer(body, "<f4", n * 4, n * 16).reshape(n, 4).astype(np.float32)
    iid = np.frombuffer(body, "<u4", n, n * 32).astype(np.uint32)
    return pos, vel, iid
