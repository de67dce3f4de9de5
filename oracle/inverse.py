"""FP64 restatement of the differentiable inverse problem (test infrastructure).

TEST INFRASTRUCTURE, NOT PRODUCT CODE: imported only by tests/ as the checker
of the GPU inverse problem.  The reference has no adjoint; this module chains
the FP64 oracle's step and its exact transpose (oracle.step /
oracle.step_backward) with the FP64 density grid (oracle.density_grid /
density_grid_backward):

  parameters: initial velocities v0 (n x 3) and a wall-sweep amplitude A;
  the x-max wall at step k is x_w(t_k) = X - A (1 - cos(2 pi t_k / T)),
  t_k = k dt;  loss = sum over nodes of (density_grid(x_final) - target)^2.

Everything here is float64, so tests check it against central finite
differences.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Tuple

import numpy as np

from . import oracle


@dataclass
class Problem:
    params: object                      # pbf_params-like (fields of include/pbf.h)
    pos0: np.ndarray                    # (n, 4) initial positions
    box: Tuple[float, float, float]     # ulim at rest; llim is the origin
    dims: Tuple[int, int, int]          # density grid nodes
    steps: int
    period: float = 4.0

    def wall_x(self, amp: float, k: int) -> float:
        t = k * float(np.float32(self.params.dt))
        return self.box[0] - amp * (1.0 - math.cos(2.0 * math.pi * t / self.period))

    def dwall_damp(self, k: int) -> float:
        t = k * float(np.float32(self.params.dt))
        return -(1.0 - math.cos(2.0 * math.pi * t / self.period))

    def limits(self, amp: float, k: int):
        return (float(np.float32(self.wall_x(amp, k))), self.box[1], self.box[2]), (0.0, 0.0, 0.0)


def rollout(pb: Problem, vel0: np.ndarray, amp: float, prec: str = "f64"):
    """Chained steps (FP64, or "f32": the reference-order float port); returns
    the per-step inputs and the final state."""
    dt = np.float64 if prec == "f64" else np.float32
    pos = np.asarray(pb.pos0, dt).copy()
    vel = np.zeros_like(pos)
    vel[:, :3] = vel0
    iid = np.arange(len(pos), dtype=np.uint32)
    hist = []
    for k in range(pb.steps):
        hist.append((pos, vel, iid))
        r = oracle.step(pb.params, *pb.limits(amp, k), pos, vel, iid, prec)
        pos, vel, iid = r["npos"], r["nvel"], r["iid"]
    return hist, pos, vel, iid


def density(pb: Problem, pos: np.ndarray) -> np.ndarray:
    return oracle.density_grid(pos, (0.0, 0.0, 0.0), pb.box, pb.dims, float(np.float32(pb.params.h)))


def loss(pb: Problem, vel0: np.ndarray, amp: float, target: np.ndarray) -> float:
    _, pos, _, _ = rollout(pb, vel0, amp)
    r = density(pb, pos) - target
    return float((r * r).sum())


def loss_and_grad(pb: Problem, vel0: np.ndarray, amp: float, target: np.ndarray, prec: str = "f64"):
    """(loss, d loss / d v0 (n x 3, initial order), d loss / d A)."""
    hist, pos, _, _ = rollout(pb, vel0, amp, prec)
    r = density(pb, pos) - target
    h = float(np.float32(pb.params.h))
    gp = oracle.density_grid_backward(pos, (0.0, 0.0, 0.0), pb.box, pb.dims, h, 2.0 * r)
    gv = np.zeros_like(gp)
    g_amp = 0.0
    for k in range(pb.steps - 1, -1, -1):
        pi, vi, ii = hist[k]
        g = oracle.step_backward(pb.params, *pb.limits(amp, k), pi, vi, ii, gp, gv, prec)
        gp, gv = g["pos"], g["vel"]
        g_amp += g["ulim"][0] * pb.dwall_damp(k)
    return float((r * r).sum()), gv[:, :3], g_amp
