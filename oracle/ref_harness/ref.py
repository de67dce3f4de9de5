"""ctypes binding of the reference harness (test infrastructure, part of the
oracle): the reference's own kernels, compiled from its sources, run on a GPU
with Simulator::step's host sequencing.  Used only to generate golden vectors
(tests/golden/make_golden.py) and as an optional GPU baseline in bench.py."""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import build_ref
from ..oracle import OracleParams, to_oracle_params

_lock = threading.Lock()
_lib = None


def available() -> bool:
    return build_ref.CUBIN.exists()


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not available():
                raise RuntimeError("reference cubin missing (built where the reference sources are)")
            L = ctypes.CDLL(str(build_ref.build_launcher()))
            P = ctypes.POINTER
            f = P(ctypes.c_float)
            u = P(ctypes.c_uint32)
            L.pbfref_last_error.restype = ctypes.c_char_p
            L.pbfref_init.argtypes = [ctypes.c_char_p]
            L.pbfref_step.argtypes = [P(OracleParams), f, f, f, f, f, f, u, ctypes.c_int, f, f, u, u, u,
                                      P(ctypes.c_int)]
            L.pbfref_bench.argtypes = [P(OracleParams), f, f, f, f, ctypes.c_int, ctypes.c_int, ctypes.c_int, f,
                                       ctypes.c_int, P(ctypes.c_double)]
            rc = L.pbfref_init(str(build_ref.CUBIN).encode())
            if rc != 0:
                raise RuntimeError(f"pbfref_init: {L.pbfref_last_error().decode()}")
            _lib = L
    return _lib


def _f3(a) -> np.ndarray:
    a = np.asarray(a, np.float32)
    return np.ascontiguousarray(a[:, :3])


def _lim(v):
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def _p(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def step(params, ulim, llim, pos, vel, iid) -> dict:
    """One reference step (host arrays (n, 3|4) float32, iid uint32).  Returns
    float3 arrays pos/vel/npos/nvel, iid, rho, lambda, sorted cell ids,
    start/end and dims, as the reference leaves them."""
    L = lib()
    pos3, vel3 = _f3(pos).copy(), _f3(vel).copy()
    n = pos3.shape[0]
    iid = np.ascontiguousarray(iid, np.uint32).copy()
    npos3 = np.zeros_like(pos3)
    nvel3 = np.zeros_like(vel3)
    rho = np.zeros(n, np.float32)
    lam = np.zeros(n, np.float32)
    ids = np.zeros(n, np.uint32)
    dims = (ctypes.c_int * 3)()
    h = float(params.h)
    cells = 1
    for a in range(3):
        cells *= int(np.ceil(np.float32(np.float32(ulim[a]) - np.float32(llim[a])) / np.float32(h)))
    start = np.zeros(cells, np.uint32)
    end = np.zeros(cells, np.uint32)
    op = to_oracle_params(params)
    fl = ctypes.c_float
    rc = L.pbfref_step(ctypes.byref(op), _lim(ulim), _lim(llim), _p(pos3, fl), _p(vel3, fl), _p(npos3, fl),
                       _p(nvel3, fl), _p(iid, ctypes.c_uint32), n, _p(rho, fl), _p(lam, fl),
                       _p(ids, ctypes.c_uint32), _p(start, ctypes.c_uint32), _p(end, ctypes.c_uint32), dims)
    if rc != 0:
        raise RuntimeError(f"pbfref_step: {L.pbfref_last_error().decode()}")
    return {"pos": pos3, "vel": vel3, "npos": npos3, "nvel": nvel3, "iid": iid, "rho": rho, "lambda": lam,
            "ids": ids, "start": start, "end": end, "dims": tuple(dims)}


def bench(params, ulim, llim, pos, vel, warmup: int, steps: int, ulim_x=None, sync: bool = True) -> float:
    """Milliseconds of `steps` reference steps on device-resident state, after
    `warmup` untimed ones; ulim_x: the x-max wall of every step (warm-up
    first); sync: keep the reference's per-phase cudaDeviceSynchronize."""
    L = lib()
    pos3, vel3 = _f3(pos), _f3(vel)
    ux = None if ulim_x is None else np.ascontiguousarray(ulim_x, np.float32)
    ms = ctypes.c_double()
    op = to_oracle_params(params)
    fl = ctypes.c_float
    rc = L.pbfref_bench(ctypes.byref(op), _lim(ulim), _lim(llim), _p(pos3, fl), _p(vel3, fl), pos3.shape[0],
                        int(warmup), int(steps), None if ux is None else _p(ux, fl), int(bool(sync)),
                        ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError(f"pbfref_bench: {L.pbfref_last_error().decode()}")
    return ms.value
