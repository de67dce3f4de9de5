"""The differentiable inverse problem on the GPU (no counterpart in the reference).

Parameters: a per-particle initial velocity (n x 3, float32) and a scalar
amplitude A of the x-max wall sweep, x_w(t) = X - A (1 - cos(2 pi t / T)) with
X the box's x extent, T = 4 s and t = k dt at step k.  The loss is the squared
L2 error between the poly6 density of the final positions on a lattice of
cell centres (32 x 16 x 16 over the 2 x 1 x 1 box) and a target density grid.

``InverseProblem.loss_and_grad`` runs the forward rollout with checkpoints
every ``every`` frames (adjoint.Rollout), the density grid and its adjoint,
and the reverse sweep; the amplitude's gradient is the chain rule through the
wall position of every step, sum_k (d loss / d ulim_x(k)) (d x_w(t_k) / d A).
"""
from __future__ import annotations

import math
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import scenes
from .adjoint import Rollout, density_grid, density_grid_backward
from .simulator import Simulator

STEPS_PER_FRAME = 2
GRID_DIMS = (32, 16, 16)


class InverseProblem:
    """One scene, one simulator, the rollout and the loss.

    ``scene``: a scenes.Scene (default scenes.inverse_scene()); ``frames``:
    frames of STEPS_PER_FRAME steps (``steps``: a step count instead);
    ``every``: checkpoint interval in frames; ``period``: the wall sweep's
    period in seconds; ``keep``: trailing checkpoint segments the forward
    tapes (adjoint.Rollout).
    """

    def __init__(self, scene: Optional[scenes.Scene] = None, frames: int = 60, every: int = 10,
                 dims: Sequence[int] = GRID_DIMS, period: float = 4.0, device: str = "cuda", keep: int = 1,
                 steps: Optional[int] = None):
        self.scene = scene if scene is not None else scenes.inverse_scene()
        self.params = self.scene.params
        self.box = tuple(float(x) for x in self.scene.ulim)
        self.dims = tuple(int(d) for d in dims)
        self.steps = int(frames) * STEPS_PER_FRAME if steps is None else int(steps)
        self.period = float(period)
        self.device = torch.device(device)
        self.n = self.scene.n
        self.dt = float(np.float32(self.params.dt))
        self.h = float(np.float32(self.params.h))
        self.sim = Simulator(self.params, self.box, (0.0, 0.0, 0.0), self.n)
        self.rollout = Rollout(self.sim, every=int(every) * STEPS_PER_FRAME, keep=keep)
        self.pos0 = torch.from_numpy(np.ascontiguousarray(self.scene.pos, np.float32)).to(self.device)
        self.target: Optional[torch.Tensor] = None

    # -- the wall --------------------------------------------------------------------

    def wall_x(self, amp: float, k: int) -> float:
        t = k * self.dt
        return self.box[0] - amp * (1.0 - math.cos(2.0 * math.pi * t / self.period))

    def dwall_damp(self, k: int) -> float:
        t = k * self.dt
        return -(1.0 - math.cos(2.0 * math.pi * t / self.period))

    def limits(self, amp: float):
        def at(k: int) -> Tuple[Tuple[float, float, float], Tuple[float, float, float]]:
            return (float(np.float32(self.wall_x(amp, k))), self.box[1], self.box[2]), (0.0, 0.0, 0.0)
        return at

    # -- forward / loss / gradient ----------------------------------------------------

    def _vel4(self, vel0: torch.Tensor) -> torch.Tensor:
        v = torch.zeros((self.n, 4), dtype=torch.float32, device=self.device)
        v[:, :3] = vel0.to(self.device, torch.float32).reshape(self.n, 3)
        return v

    def forward(self, vel0: torch.Tensor, amp: float):
        """Final (pos, vel, iid) after ``steps`` steps from pos0 with velocities vel0."""
        iid = torch.arange(self.n, dtype=torch.int32, device=self.device)
        return self.rollout.run(self.pos0, self._vel4(vel0), iid, self.steps, self.limits(amp))

    def density(self, pos: torch.Tensor) -> torch.Tensor:
        return density_grid(pos, (0.0, 0.0, 0.0), self.box, self.dims, self.h)

    def make_target(self, seed: int = 1, sigma: float = 0.2, amp: float = 0.3) -> torch.Tensor:
        """The target grid: the density after a forward run from seeded
        N(0, sigma^2) initial velocities and amplitude ``amp``."""
        rng = np.random.default_rng(seed)
        v = torch.from_numpy(rng.normal(0.0, sigma, size=(self.n, 3)).astype(np.float32))
        pos, _, _ = self.forward(v, amp)
        self.target = self.density(pos).clone()
        return self.target

    def loss(self, vel0: torch.Tensor, amp: float) -> float:
        pos, _, _ = self.forward(vel0, amp)
        r = self.density(pos) - self.target
        return float((r.double() ** 2).sum())

    def loss_and_grad(self, vel0: torch.Tensor, amp: float):
        """(loss, d loss / d vel0 as (n, 3) in the initial order, d loss / d amp)."""
        if self.target is None:
            raise RuntimeError("no target: call make_target() or set .target first")
        pos, _, _ = self.forward(vel0, amp)
        r = self.density(pos) - self.target
        g_pos = density_grid_backward(pos, (0.0, 0.0, 0.0), self.box, self.dims, self.h, 2.0 * r)
        g_pos0, g_vel0, g_lim = self.rollout.backward(g_pos, torch.zeros_like(g_pos))
        dw = torch.tensor([self.dwall_damp(k) for k in range(self.steps)], dtype=torch.float64)
        g_amp = float((g_lim[:, 0].double().cpu() * dw).sum())
        return float((r.double() ** 2).sum()), g_vel0[:, :3], g_amp

    def autotune_backward(self, vel0: torch.Tensor, amp: float, lanes=(8, 16, 32)) -> dict:
        """Times one gradient evaluation per choice of the reverse pass's lanes
        per particle (pbf_tuning.bwd_lanes) at (vel0, amp) and keeps the fastest
        for the following evaluations; returns the choice and the times (ms).
        The choice changes the order of the reverse pass's window sums only."""
        times = {}
        tune = self.sim.tuning()
        for lane_count in lanes:
            self.sim.set_tuning(**{**tune, "bwd_lanes": int(lane_count)})
            self.loss_and_grad(vel0, amp)  # untimed: the first evaluation of a setting
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            self.loss_and_grad(vel0, amp)
            e1.record()
            torch.cuda.synchronize()
            times[int(lane_count)] = e0.elapsed_time(e1)
        best = min(times, key=times.get)
        self.sim.set_tuning(**{**tune, "bwd_lanes": best})
        return {"bwd_lanes": best, "ms": times}

    def optimise(self, iters: int = 10, lr_vel: float = 1e-9, lr_amp: float = 1e-10,
                 vel0: Optional[torch.Tensor] = None, amp: float = 0.0):
        """Plain gradient descent on (vel0, amp); returns (vel0, amp, losses)."""
        v = torch.zeros((self.n, 3), dtype=torch.float32, device=self.device) if vel0 is None else vel0.clone()
        losses = []
        for _ in range(iters):
            L, gv, ga = self.loss_and_grad(v, amp)
            losses.append(L)
            v = v - lr_vel * gv
            amp = amp - lr_amp * ga
        return v, amp, losses

    def close(self) -> None:
        self.sim.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
