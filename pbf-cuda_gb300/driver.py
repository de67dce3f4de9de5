"""Headless scene driver: the per-frame loop of the reference's FluidSystem.

FluidSystem::stepSimulate (fluids/FluidSystem.cpp:99-120) reloads the solver
parameters, optionally sweeps the box limits sinusoidally
(ulim + A_ulim sin(w t), llim + A_llim sin(w t), t = w (frame - start frame)),
and calls Simulator::step once with the tic-toc buffer roles.  SceneDriver
does the same without a window: `substeps` steps per frame (the scenes here
use dt = 1/120 s, two per 1/60 s frame), the limits from the scene's own wall
function or from a reference-style sweep, and optionally one particle state
file per frame (scenes.save_state) for offline comparison and one rendered
image per frame (the SSF surface, ssf.SSFRenderer, as Renderer::render draws
after each simulated frame, fluids/FluidSystem.cpp:119).
"""
from __future__ import annotations

import math
from pathlib import Path
from typing import Optional, Sequence, Tuple

import torch

from . import scenes as _scenes
from . import ssf as _ssf
from .simulator import ParticleState, Simulator


class Sweep:
    """The reference's sinusoidal boundary sweep: limits = base + A sin(w (frame - start))."""

    def __init__(self, a_ulim: Sequence[float], a_llim: Sequence[float], w: float, start_frame: int = 0):
        self.a_ulim = tuple(float(x) for x in a_ulim)
        self.a_llim = tuple(float(x) for x in a_llim)
        self.w = float(w)
        self.start = int(start_frame)

    def limits(self, ulim, llim, frame: int):
        phi = math.sin(self.w * (frame - self.start))
        return (tuple(u + a * phi for u, a in zip(ulim, self.a_ulim)),
                tuple(l + a * phi for l, a in zip(llim, self.a_llim)))


class SceneDriver:
    """Runs a scenes.Scene frame by frame on the GPU."""

    def __init__(self, scene: _scenes.Scene, substeps: int = _scenes.SUBSTEPS, sweep: Optional[Sweep] = None,
                 dump_dir=None, dump_every: int = 1, render_dir=None,
                 renderer: Optional["_ssf.SSFRenderer"] = None, y_up: bool = True):
        self.scene = scene
        self.substeps = int(substeps)
        self.sweep = sweep
        self.dump_dir = Path(dump_dir) if dump_dir is not None else None
        self.dump_every = max(1, int(dump_every))
        self.sim = Simulator(scene.params, scene.ulim, scene.llim, scene.n)
        self.state = ParticleState(scene.pos, scene.vel)
        self.frame = 0
        self.t = 0.0
        if self.dump_dir is not None:
            self.dump_dir.mkdir(parents=True, exist_ok=True)
        # rendered frames: renderer (its camera and settings) or the reference's defaults
        self.render_dir = Path(render_dir) if render_dir is not None else None
        self.renderer = renderer
        self.y_up = bool(y_up)
        self.last_image = None
        if self.render_dir is not None:
            self.render_dir.mkdir(parents=True, exist_ok=True)
            if self.renderer is None:
                self.renderer = _ssf.SSFRenderer()

    def limits(self) -> Tuple[Tuple[float, ...], Tuple[float, ...]]:
        if self.sweep is not None:
            return self.sweep.limits(self.scene.ulim, self.scene.llim, self.frame)
        return self.scene.limits_at(self.t)

    def step_frame(self) -> None:
        dt = float(self.scene.params.dt)
        for _ in range(self.substeps):
            self.sim.setLim(*self.limits())
            self.state.step(self.sim)
            self.t += dt
        self.frame += 1
        if self.dump_dir is not None and self.frame % self.dump_every == 0:
            self.dump(self.dump_dir / f"frame_{self.frame:06d}.bin")
        if self.render_dir is not None and self.frame % self.dump_every == 0:
            _ssf.write_ppm(self.render_dir / f"frame_{self.frame:06d}.ppm", self.render())

    def render(self) -> torch.Tensor:
        """The SSF image of the current state (positions turned z-up when the scene is y-up)."""
        pos = self.state.pos
        self.last_image = self.renderer.render(_ssf.z_up(pos) if self.y_up else pos.contiguous())
        return self.last_image

    def run(self, frames: int) -> None:
        for _ in range(int(frames)):
            self.step_frame()

    def dump(self, path) -> None:
        """The current state (positions, velocities, iids in cell order) to a state file."""
        torch.cuda.synchronize()
        _scenes.save_state(path, self.state.pos, self.state.vel, self.state.iid[: self.state.n])

    def close(self) -> None:
        self.sim.close()
        if self.renderer is not None:
            self.renderer.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def fluid_system(moving: bool = False, dump_dir=None, render_dir=None, renderer=None) -> SceneDriver:
    """FluidSystem() (fluids/FluidSystem.cpp:8-85) without a window: the
    reference's DoubleDamSource scene with its default parameters, one step
    per frame (stepSimulate calls Simulator::step once, dt = 0.0083), and,
    when `moving`, its boundary sweep ulim + (2, 0, 0) sin(0.05 frame)
    (fluids/FluidSystem.cpp:36-38, 104-110).  The scene is z up, the
    renderer's world, so rendered frames need no axis change."""
    sweep = Sweep((2.0, 0.0, 0.0), (0.0, 0.0, 0.0), w=0.05) if moving else None
    return SceneDriver(_scenes.reference_double_dam(), substeps=1, sweep=sweep, dump_dir=dump_dir,
                       render_dir=render_dir, renderer=renderer, y_up=False)
