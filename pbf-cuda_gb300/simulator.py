"""Host-side mirror of naeioi/PBF-CUDA's ``Simulator`` (fluids/Simulator.h:7-61).

Same method names and argument meaning as the reference; buffers are CUDA
tensors (float32 (n, 4) for positions/velocities, int32 (n,) for iid) instead
of OpenGL buffer names.  Every call goes through the C ABI of libpbf.so; a
non-OK status raises PbfError (the reference exits the process instead,
common/cuda_inc/helper_cuda.h:1000-1014).
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import torch

from ._abi import PBF_ERR_NOT_READY, PbfParams, PbfStepProfile, PbfTuning, check, lib


def _vec3(v: Sequence[float]) -> ctypes.Array:
    if len(v) != 3:
        raise ValueError("expected 3 components")
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def _stream_handle(stream) -> Optional[int]:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


def _check_state(t: torch.Tensor, name: str, n: int, cols: Optional[int]) -> None:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if cols is None:
        if t.dtype not in (torch.int32, torch.uint32) or t.dim() != 1 or t.shape[0] < n:
            raise ValueError(f"{name} must be int32 of shape (>= {n},)")
    elif t.dtype != torch.float32 or t.dim() != 2 or t.shape[1] != cols or t.shape[0] < n:
        raise ValueError(f"{name} must be float32 of shape (>= {n}, {cols})")


def _tuning(dense_window, dense_all, order, bwd_lanes, stage_sparse, stage_dense, queue_sparse, queue_dense,
            dense_split, dense_interleave) -> PbfTuning:
    t = PbfTuning()
    t.dense_window, t.dense_all, t.order, t.bwd_lanes = int(dense_window), int(dense_all), int(order), int(bwd_lanes)
    t.stage_sparse, t.stage_dense = int(stage_sparse), int(stage_dense)
    t.queue_sparse, t.queue_dense, t.dense_split = int(queue_sparse), int(queue_dense), int(dense_split)
    t.dense_interleave = int(dense_interleave)
    return t


def _tuning_dict(t: PbfTuning) -> dict:
    return {k: getattr(t, k) for k in ("dense_window", "dense_all", "order", "bwd_lanes", "stage_sparse",
                                       "stage_dense", "queue_sparse", "queue_dense", "dense_split",
                                       "dense_interleave")}


class Simulator:
    """One PBF solver instance: ``Simulator(params, ulim, llim)`` + ``step``.

    ``max_particles`` bounds ``nparticle`` (the reference's MAX_PARTICLE_NUM,
    fluids/helper.h:10, is a compile-time 130000; here it is per instance).
    Construct with the target CUDA device current.
    """

    def __init__(self, params: PbfParams, ulim: Sequence[float], llim: Sequence[float],
                 max_particles: int):
        self._L = lib()
        self._h = ctypes.c_void_p()
        check(self._L.pbf_create(ctypes.byref(params), _vec3(ulim), _vec3(llim), int(max_particles),
                                 ctypes.byref(self._h)), "pbf_create")
        self.max_particles = int(max_particles)

    # -- reference interface -------------------------------------------------------

    def step(self, pos: torch.Tensor, npos: torch.Tensor, vel: torch.Tensor, nvel: torch.Tensor,
             iid: torch.Tensor, nparticle: Optional[int] = None, stream=None) -> None:
        """Simulator::step (fluids/Simulator.cpp:10-99): advance one dt.

        pos/vel/iid are permuted in place into cell order; npos/nvel receive
        the new state; vel receives (npos - pos) / dt.  Asynchronous on
        ``stream`` (default: torch's current stream).
        """
        n = pos.shape[0] if nparticle is None else int(nparticle)
        for t, name, cols in ((pos, "pos", 4), (npos, "npos", 4), (vel, "vel", 4), (nvel, "nvel", 4),
                              (iid, "iid", None)):
            _check_state(t, name, n, cols)
        check(self._L.pbf_step(self._h, pos.data_ptr(), npos.data_ptr(), vel.data_ptr(), nvel.data_ptr(),
                               iid.data_ptr(), n, _stream_handle(stream)), "pbf_step")

    def loadParams(self, params: PbfParams) -> None:
        """Simulator::loadParams (fluids/Simulator.cpp:101-115); the reference
        reads the GUIParams singleton, here the caller passes the struct."""
        check(self._L.pbf_set_params(self._h, ctypes.byref(params)), "pbf_set_params")

    def saveParams(self) -> PbfParams:
        """Simulator::saveParams (fluids/Simulator.cpp:117-130)."""
        p = PbfParams()
        check(self._L.pbf_get_params(self._h, ctypes.byref(p)), "pbf_get_params")
        return p

    def setLim(self, ulim: Sequence[float], llim: Sequence[float]) -> None:
        """Simulator::setLim (fluids/Simulator.cpp:132-136)."""
        check(self._L.pbf_set_limits(self._h, _vec3(ulim), _vec3(llim)), "pbf_set_limits")

    # -- additions -------------------------------------------------------------------

    def getLim(self):
        u = (ctypes.c_float * 3)()
        l = (ctypes.c_float * 3)()
        check(self._L.pbf_get_limits(self._h, u, l), "pbf_get_limits")
        return list(u), list(l)

    def density(self, n: int, stream=None) -> torch.Tensor:
        """rho of the last step's final lambda pass, in that step's cell order."""
        out = torch.empty(max(n, 1), dtype=torch.float32, device="cuda")
        check(self._L.pbf_get_density(self._h, out.data_ptr(), int(n), _stream_handle(stream)),
              "pbf_get_density")
        return out[:n]

    def grid_dims(self):
        dims = (ctypes.c_int * 3)()
        check(self._L.pbf_build_grid(self._h, None, 0, None, None, None, None, dims, None), "pbf_build_grid")
        return tuple(int(d) for d in dims)

    def build_grid(self, xstar: torch.Tensor, stream=None) -> dict:
        """The reference's neighbour grid (fluids/Simulator.cu:178-211) of the
        predicted positions ``xstar``: keys, stable perm, start/end, dims."""
        n = xstar.shape[0]
        _check_state(xstar, "xstar", n, 4)
        dims = self.grid_dims()
        cells = dims[0] * dims[1] * dims[2]
        dev = xstar.device
        keys = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        perm = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        start = torch.empty(cells, dtype=torch.int32, device=dev)
        end = torch.empty(cells, dtype=torch.int32, device=dev)
        d = (ctypes.c_int * 3)()
        check(self._L.pbf_build_grid(self._h, xstar.data_ptr(), n, keys.data_ptr(), perm.data_ptr(),
                                     start.data_ptr(), end.data_ptr(), d, _stream_handle(stream)),
              "pbf_build_grid")
        return {"keys": keys[:n], "perm": perm[:n], "start": start, "end": end, "dims": dims}

    def use_graphs(self, on: bool = True) -> None:
        """Run each step as a CUDA graph (default) or as individual launches."""
        check(self._L.pbf_use_graphs(self._h, int(bool(on))), "pbf_use_graphs")

    def tape(self, depth=1) -> None:
        """Record the following steps for their reverse passes: a stack of up
        to ``depth`` taped steps (True: 1; 0 / False: tape off), emptied here.
        ``backward`` pops the most recent one."""
        check(self._L.pbf_tape_enable(self._h, int(depth)), "pbf_tape_enable")

    def backward(self, g_npos: torch.Tensor, g_nvel: torch.Tensor, stream=None):
        """Reverse pass of the most recent taped step (popped from the tape):
        adjoints of its outputs npos, nvel (its output order) -> adjoints of its
        inputs pos, vel (its input order) and of the limits (6 floats: ulim
        xyz, llim xyz)."""
        n = g_npos.shape[0]
        for t, name in ((g_npos, "g_npos"), (g_nvel, "g_nvel")):
            _check_state(t, name, n, 4)
        g_pos = torch.zeros_like(g_npos)
        g_vel = torch.zeros_like(g_nvel)
        g_lim = torch.zeros(6, dtype=torch.float32, device=g_npos.device)
        check(self._L.pbf_backward(self._h, g_npos.data_ptr(), g_nvel.data_ptr(), g_pos.data_ptr(),
                                   g_vel.data_ptr(), g_lim.data_ptr(), _stream_handle(stream)), "pbf_backward")
        return g_pos, g_vel, g_lim

    def set_tuning(self, dense_window: int = 0, dense_all: int = -1, order: int = -1, bwd_lanes: int = 0,
                   stage_sparse: int = -1, stage_dense: int = -1, queue_sparse: int = 0, queue_dense: int = 0,
                   dense_split: int = 0, dense_interleave: int = -1) -> None:
        """The neighbour passes' choices for the following steps (dense window,
        dense-for-all, particle order, shared-memory stages, hit queues, dense
        split) and the reverse pass's lanes per particle (pbf_set_tuning); 0 /
        -1: the defaults (stage_*: 0 turns staging off)."""
        check(self._L.pbf_set_tuning(self._h, ctypes.byref(_tuning(
            dense_window, dense_all, order, bwd_lanes, stage_sparse, stage_dense, queue_sparse, queue_dense,
            dense_split, dense_interleave))), "pbf_set_tuning")

    def tuning(self) -> dict:
        t = PbfTuning()
        check(self._L.pbf_get_tuning(self._h, ctypes.byref(t)), "pbf_get_tuning")
        return _tuning_dict(t)

    def check_device(self, stream=None) -> None:
        """Raise PbfError (PBF_ERR_TIMEOUT) if a bounded device-side wait of the
        steps since the last check gave up (pbf_check_device)."""
        check(self._L.pbf_check_device(self._h, _stream_handle(stream)), "pbf_check_device")

    def autotune(self, pos: torch.Tensor, vel: torch.Tensor, iid: torch.Tensor, nparticle: Optional[int] = None,
                 steps: int = 3, stream=None) -> dict:
        """Time the dense-kernel choices on copies of this state (pbf_autotune)
        and keep the fastest; returns the choice and its time per step."""
        n = pos.shape[0] if nparticle is None else int(nparticle)
        for t, name, cols in ((pos, "pos", 4), (vel, "vel", 4), (iid, "iid", None)):
            _check_state(t, name, n, cols)
        out = PbfTuning()
        check(self._L.pbf_autotune(self._h, pos.data_ptr(), vel.data_ptr(), iid.data_ptr(), n, int(steps),
                                   ctypes.byref(out), _stream_handle(stream)), "pbf_autotune")
        return out.as_dict()

    def profile(self, on: bool = True) -> None:
        """Record CUDA events between the phases of every following step."""
        check(self._L.pbf_profile_enable(self._h, int(bool(on))), "pbf_profile_enable")

    def last_profile(self) -> dict:
        """Phase times (ms) and kernel launch counts of the last step.  Without
        profiling only the launch counts are filled in."""
        prof = PbfStepProfile()
        st = self._L.pbf_profile_read(self._h, ctypes.byref(prof))
        if st not in (0, PBF_ERR_NOT_READY):
            check(st, "pbf_profile_read")
        return prof.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            check(self._L.pbf_destroy(self._h), "pbf_destroy")
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ParticleState:
    """Device-resident particle buffers with the reference's tic-toc roles
    (fluids/FluidSystem.cpp:112-117): after each step the new state is
    (npos, nvel) and the next step writes into the old (pos, vel)."""

    def __init__(self, pos, vel, iid=None, device="cuda", capacity: Optional[int] = None):
        pos = torch.as_tensor(pos, dtype=torch.float32)
        vel = torch.as_tensor(vel, dtype=torch.float32)
        n = pos.shape[0]
        cap = n if capacity is None else int(capacity)
        if pos.shape[1] == 3:
            pos = torch.cat([pos, torch.zeros(n, 1)], 1)
        if vel.shape[1] == 3:
            vel = torch.cat([vel, torch.zeros(n, 1)], 1)
        self.n = n
        self.a_pos = torch.zeros(cap, 4, dtype=torch.float32, device=device)
        self.a_vel = torch.zeros(cap, 4, dtype=torch.float32, device=device)
        self.b_pos = torch.zeros(cap, 4, dtype=torch.float32, device=device)
        self.b_vel = torch.zeros(cap, 4, dtype=torch.float32, device=device)
        self.iid = torch.zeros(cap, dtype=torch.int32, device=device)
        self.a_pos[:n] = pos.to(device)
        self.a_vel[:n] = vel.to(device)
        if iid is None:
            self.iid[:n] = torch.arange(n, dtype=torch.int32, device=device)
        else:
            self.iid[:n] = torch.as_tensor(iid, dtype=torch.int32).to(device)
        self.tictoc = False

    @property
    def pos(self) -> torch.Tensor:
        return (self.b_pos if self.tictoc else self.a_pos)[: self.n]

    @property
    def vel(self) -> torch.Tensor:
        return (self.b_vel if self.tictoc else self.a_vel)[: self.n]

    def step(self, sim, stream=None) -> None:
        """One step with a Simulator, or with an Ensemble over all its scenes."""
        if not self.tictoc:
            src = (self.a_pos, self.b_pos, self.a_vel, self.b_vel)
        else:
            src = (self.b_pos, self.a_pos, self.b_vel, self.a_vel)
        if isinstance(sim, Ensemble):
            sim.step(src[0], src[1], src[2], src[3], self.iid, stream)
        else:
            sim.step(src[0], src[1], src[2], src[3], self.iid, self.n, stream)
        self.tictoc = not self.tictoc


class Ensemble:
    """Many independent scenes advanced together (pbf_batch_* of the C ABI).

    Scene s owns particle slots [offsets[s], offsets[s] + counts[s]) of every
    buffer; each scene follows Simulator.step's contract inside its range.
    """

    def __init__(self, params: PbfParams, ulims, llims, counts):
        self._L = lib()
        self.nscenes = len(counts)
        u = (ctypes.c_float * (3 * self.nscenes))(*[float(x) for v in ulims for x in v])
        l = (ctypes.c_float * (3 * self.nscenes))(*[float(x) for v in llims for x in v])
        cnt = (ctypes.c_int * self.nscenes)(*[int(c) for c in counts])
        self._h = ctypes.c_void_p()
        check(self._L.pbf_batch_create(ctypes.byref(params), self.nscenes, u, l, cnt, ctypes.byref(self._h)),
              "pbf_batch_create")
        self.counts = [int(c) for c in counts]
        self.n = sum(self.counts)
        self.offsets = [sum(self.counts[:k]) for k in range(self.nscenes)]

    def step(self, pos, npos, vel, nvel, iid, stream=None) -> None:
        for t, name, cols in ((pos, "pos", 4), (npos, "npos", 4), (vel, "vel", 4), (nvel, "nvel", 4),
                              (iid, "iid", None)):
            _check_state(t, name, self.n, cols)
        check(self._L.pbf_batch_step(self._h, pos.data_ptr(), npos.data_ptr(), vel.data_ptr(), nvel.data_ptr(),
                                     iid.data_ptr(), _stream_handle(stream)), "pbf_batch_step")

    def setLim(self, scene: int, ulim: Sequence[float], llim: Sequence[float]) -> None:
        check(self._L.pbf_batch_set_limits(self._h, int(scene), _vec3(ulim), _vec3(llim)), "pbf_batch_set_limits")

    def set_tuning(self, dense_window: int = 0, dense_all: int = -1, order: int = -1, stage_sparse: int = -1,
                   stage_dense: int = -1, queue_sparse: int = 0, queue_dense: int = 0, dense_split: int = 0,
                   dense_interleave: int = -1) -> None:
        """The neighbour passes' choices for the following steps (pbf_batch_set_tuning)."""
        check(self._L.pbf_batch_set_tuning(self._h, ctypes.byref(_tuning(
            dense_window, dense_all, order, 0, stage_sparse, stage_dense, queue_sparse, queue_dense,
            dense_split, dense_interleave))), "pbf_batch_set_tuning")

    def tuning(self) -> dict:
        t = PbfTuning()
        check(self._L.pbf_batch_get_tuning(self._h, ctypes.byref(t)), "pbf_batch_get_tuning")
        d = _tuning_dict(t)
        del d["bwd_lanes"]
        return d

    def check_device(self, stream=None) -> None:
        """Raise PbfError (PBF_ERR_TIMEOUT) if a bounded device-side wait of the
        steps since the last check gave up (pbf_batch_check_device)."""
        check(self._L.pbf_batch_check_device(self._h, _stream_handle(stream)), "pbf_batch_check_device")

    def density(self, stream=None) -> torch.Tensor:
        out = torch.empty(max(self.n, 1), dtype=torch.float32, device="cuda")
        check(self._L.pbf_batch_get_density(self._h, out.data_ptr(), _stream_handle(stream)),
              "pbf_batch_get_density")
        return out[: self.n]

    def autotune(self, pos: torch.Tensor, vel: torch.Tensor, iid: torch.Tensor, steps: int = 3,
                 stream=None) -> dict:
        """pbf_batch_autotune on copies of this state; returns the choice."""
        out = PbfTuning()
        check(self._L.pbf_batch_autotune(self._h, pos.data_ptr(), vel.data_ptr(), iid.data_ptr(), int(steps),
                                         ctypes.byref(out), _stream_handle(stream)), "pbf_batch_autotune")
        return out.as_dict()

    def use_graphs(self, on: bool = True) -> None:
        check(self._L.pbf_batch_use_graphs(self._h, int(bool(on))), "pbf_batch_use_graphs")

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            check(self._L.pbf_batch_destroy(self._h), "pbf_batch_destroy")
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
