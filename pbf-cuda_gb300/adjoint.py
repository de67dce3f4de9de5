"""Differentiable rollouts of the PBF step (no counterpart in the reference).

Building blocks, all on the GPU through the C ABI:

* ``Simulator.tape()`` / ``Simulator.backward()`` — the reverse pass of one
  step (pbf_tape_enable / pbf_backward): adjoints of the step's outputs
  (npos, nvel, in its output order) -> adjoints of its inputs (pos, vel, in
  its input order) and of the six box limits.
* ``density_grid`` / ``density_grid_backward`` — the poly6 density of the
  particles at the centres of a lattice of cells, and its adjoint
  (pbf_density_grid / pbf_density_grid_backward).

On top of them:

* ``Rollout`` — T chained steps with checkpoints every K steps.  The last
  ``keep`` segments are taped as the forward runs them; the reverse sweep pops
  their reverse passes directly, then re-runs each earlier K-step segment from
  its checkpoint with the tape on (a stack of K taped steps) and pops its
  reverse passes, last step first.  A step of a re-run segment runs twice
  forward and once backward; memory: T/K checkpoints + max(keep, 1) K tape
  records.
* ``step`` — one step as a ``torch.autograd.Function`` (its backward re-runs
  the step from saved copies of its inputs with the tape on).
* ``DensityGrid`` — the density grid as a ``torch.autograd.Function``.

The reverse pass holds the step's neighbour sets and clamp states fixed
(their derivatives are zero almost everywhere) and needs
``k_boundaryDensity == 0``.
"""
from __future__ import annotations

import ctypes
from typing import Callable, List, Optional, Sequence, Tuple

import torch

from ._abi import check, lib
from .simulator import Simulator, _check_state, _stream_handle

Limits = Tuple[Sequence[float], Sequence[float]]


def _f3(v: Sequence[float]) -> ctypes.Array:
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def density_grid(pos: torch.Tensor, lo: Sequence[float], hi: Sequence[float], dims: Sequence[int], h: float,
                 n: Optional[int] = None, stream=None) -> torch.Tensor:
    """Poly6 density (mass 1, radius h) at the centres of the dims[0] x dims[1] x
    dims[2] cells spanning [lo, hi]: a float32 tensor of shape dims (x slowest)."""
    n = pos.shape[0] if n is None else int(n)
    _check_state(pos, "pos", n, 4)
    grid = torch.empty(tuple(int(d) for d in dims), dtype=torch.float32, device=pos.device)
    d = (ctypes.c_int * 3)(*[int(x) for x in dims])
    check(lib().pbf_density_grid(pos.data_ptr(), n, _f3(lo), _f3(hi), d, float(h), grid.data_ptr(),
                                 _stream_handle(stream)), "pbf_density_grid")
    return grid


def density_grid_backward(pos: torch.Tensor, lo: Sequence[float], hi: Sequence[float], dims: Sequence[int],
                          h: float, g_grid: torch.Tensor, n: Optional[int] = None, stream=None) -> torch.Tensor:
    """Adjoint of ``density_grid`` w.r.t. the positions: (n, 4) float32."""
    n = pos.shape[0] if n is None else int(n)
    _check_state(pos, "pos", n, 4)
    g_grid = g_grid.contiguous().to(torch.float32)
    if g_grid.numel() != int(dims[0]) * int(dims[1]) * int(dims[2]) or not g_grid.is_cuda:
        raise ValueError("g_grid must be a CUDA tensor with one value per node")
    g_pos = torch.empty((max(n, 1), 4), dtype=torch.float32, device=pos.device)
    d = (ctypes.c_int * 3)(*[int(x) for x in dims])
    check(lib().pbf_density_grid_backward(pos.data_ptr(), n, _f3(lo), _f3(hi), d, float(h), g_grid.data_ptr(),
                                          g_pos.data_ptr(), _stream_handle(stream)), "pbf_density_grid_backward")
    return g_pos[:n]


class DensityGrid(torch.autograd.Function):
    """``DensityGrid.apply(pos, lo, hi, dims, h)``: differentiable in pos."""

    @staticmethod
    def forward(ctx, pos, lo, hi, dims, h):
        pos = pos.contiguous()
        ctx.save_for_backward(pos)
        ctx.cfg = (tuple(lo), tuple(hi), tuple(dims), float(h))
        return density_grid(pos, lo, hi, dims, h)

    @staticmethod
    def backward(ctx, g_grid):
        (pos,) = ctx.saved_tensors
        lo, hi, dims, h = ctx.cfg
        return density_grid_backward(pos, lo, hi, dims, h, g_grid), None, None, None, None


class _Step(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sim, pos, vel, iid, ulim, llim):
        n = pos.shape[0]
        lims = ([float(x) for x in ulim], [float(x) for x in llim])
        ctx.sim, ctx.lims = sim, lims
        ctx.save_for_backward(pos.detach().clone(), vel.detach().clone(), iid.clone())
        p, v, i = pos.detach().clone(), vel.detach().clone(), iid.clone()
        npos = torch.empty_like(p)
        nvel = torch.empty_like(v)
        sim.tape(0)
        sim.setLim(*lims)
        sim.step(p, npos, v, nvel, i, n)
        ctx.mark_non_differentiable(i)
        return npos, nvel, i

    @staticmethod
    def backward(ctx, g_npos, g_nvel, _g_iid):
        sim = ctx.sim
        pos, vel, iid = (t.clone() for t in ctx.saved_tensors)
        n = pos.shape[0]
        g_npos = torch.zeros_like(pos) if g_npos is None else g_npos.contiguous()
        g_nvel = torch.zeros_like(vel) if g_nvel is None else g_nvel.contiguous()
        npos = torch.empty_like(pos)
        nvel = torch.empty_like(vel)
        sim.tape(1)
        sim.setLim(*ctx.lims)
        sim.step(pos, npos, vel, nvel, iid, n)
        g_pos, g_vel, g_lim = sim.backward(g_npos, g_nvel)
        sim.tape(0)
        return None, g_pos, g_vel, None, g_lim[:3].cpu(), g_lim[3:].cpu()


def step(sim: Simulator, pos: torch.Tensor, vel: torch.Tensor, iid: torch.Tensor,
         ulim: Sequence[float], llim: Sequence[float]):
    """One differentiable step: returns (npos, nvel, iid_out).  ``pos`` and
    ``vel`` are not modified; ``ulim``/``llim`` may be tensors that require
    grad (3 floats each, read on the host)."""
    ulim_t = ulim if isinstance(ulim, torch.Tensor) else torch.tensor([float(x) for x in ulim])
    llim_t = llim if isinstance(llim, torch.Tensor) else torch.tensor([float(x) for x in llim])
    return _Step.apply(sim, pos, vel, iid, ulim_t, llim_t)


class Rollout:
    """T chained steps of one Simulator with checkpoints every ``every`` steps.

    ``run`` advances (pos, vel, iid) by ``steps`` steps, the box of step k given
    by ``limits(k)`` (None: the simulator's current box), and returns the final
    state.  ``backward(g_pos, g_vel)`` takes the adjoints of that final state
    (in its order) and returns the adjoints of the initial pos and vel (in
    their order) and a (steps, 6) tensor of the limits' adjoints per step
    (ulim xyz, llim xyz).  The forward tapes its last ``keep`` segments
    (``keep`` = 0: none; a large value: the whole rollout, no re-runs); the
    reverse sweep pops those, then re-runs each earlier segment from its
    checkpoint with a tape of ``every`` steps and pops their reverse passes.
    """

    def __init__(self, sim: Simulator, every: int = 10, keep: int = 1):
        if every < 1:
            raise ValueError("every must be >= 1")
        if keep < 0:
            raise ValueError("keep must be >= 0")
        self.sim = sim
        self.every = int(every)
        self.keep = int(keep)
        self._first_taped = 0
        self._ckpt: List[Tuple[torch.Tensor, torch.Tensor, torch.Tensor]] = []
        self._steps = 0
        self._limits: Optional[Callable[[int], Limits]] = None
        self._n = 0

    def _advance(self, pos, vel, iid, k):
        """One step from (pos, vel, iid), which it leaves permuted; returns the new state."""
        if self._limits is not None:
            self.sim.setLim(*self._limits(k))
        npos = torch.empty_like(pos)
        nvel = torch.empty_like(vel)
        self.sim.step(pos, npos, vel, nvel, iid, self._n)
        return npos, nvel, iid

    def run(self, pos: torch.Tensor, vel: torch.Tensor, iid: torch.Tensor, steps: int,
            limits: Optional[Callable[[int], Limits]] = None):
        self._n = pos.shape[0]
        self._steps = int(steps)
        self._limits = limits
        self._ckpt = []
        self.sim.tape(0)
        nseg = (self._steps + self.every - 1) // self.every
        self._first_taped = nseg - min(self.keep, nseg)
        pos, vel, iid = pos.clone(), vel.clone(), iid.clone()
        for k in range(self._steps):
            if k % self.every == 0:
                self._ckpt.append((pos.clone(), vel.clone(), iid.clone()))
                if k // self.every == self._first_taped:  # tape from here to the end
                    self.sim.tape(self._steps - k)
            pos, vel, iid = self._advance(pos, vel, iid, k)
        return pos, vel, iid

    def backward(self, g_pos: torch.Tensor, g_vel: torch.Tensor):
        g_pos = g_pos.contiguous().clone()
        g_vel = g_vel.contiguous().clone()
        g_lim = torch.zeros((self._steps, 6), dtype=torch.float32, device=g_pos.device)
        for seg in range(len(self._ckpt) - 1, -1, -1):
            start = seg * self.every
            end = min(start + self.every, self._steps)
            if seg < self._first_taped:  # not taped by the forward: re-run it taped
                if seg == self._first_taped - 1:
                    self.sim.tape(self.every)
                pos, vel, iid = (t.clone() for t in self._ckpt[seg])
                for k in range(start, end):
                    pos, vel, iid = self._advance(pos, vel, iid, k)
            for k in range(end - 1, start - 1, -1):
                g_pos, g_vel, gl = self.sim.backward(g_pos, g_vel)
                g_lim[k] = gl
        self.sim.tape(0)
        return g_pos, g_vel, g_lim
