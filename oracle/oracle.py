"""ctypes binding of the CPU oracle (oracle/pbf_oracle.c).

TEST INFRASTRUCTURE, NOT PRODUCT CODE: imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker or the
timed CPU baseline.

The oracle is a CPU restatement of naeioi/PBF-CUDA's Simulator::step
(fluids/Simulator.cpp:10-99, fluids/Simulator.cu:165-273,
fluids/Simulator_kernel.cuh:7-239) in two arithmetics: ``"f32"`` (float, in
the reference's operation order, OpenMP-parallel: the CPU port) and ``"f64"``
(double: the FP64 oracle).  It defines its own mirror of ``pbf_params`` from
include/pbf.h so that it depends on nothing in the product package.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import build_oracle

_lock = threading.Lock()
_lib = None


class OracleParams(ctypes.Structure):
    """Field-for-field mirror of ``pbf_params`` (include/pbf.h)."""

    _fields_ = [
        ("niter", ctypes.c_int),
        ("pho0", ctypes.c_float),
        ("g", ctypes.c_float),
        ("h", ctypes.c_float),
        ("dt", ctypes.c_float),
        ("lambda_eps", ctypes.c_float),
        ("delta_q", ctypes.c_float),
        ("k_corr", ctypes.c_float),
        ("n_corr", ctypes.c_float),
        ("k_boundaryDensity", ctypes.c_float),
        ("c_XSPH", ctypes.c_float),
        ("up", ctypes.c_float * 3),
        ("lim_eps", ctypes.c_float),
        ("kernel_eps", ctypes.c_float),
        ("max_dp", ctypes.c_float),
        ("vorticity_eps", ctypes.c_float),
    ]


def to_oracle_params(p) -> OracleParams:
    """Copy any object with pbf_params' field names into an OracleParams."""
    out = OracleParams()
    for name, _ in OracleParams._fields_:
        v = getattr(p, name)
        if name == "up":
            for a in range(3):
                out.up[a] = float(v[a])
        else:
            setattr(out, name, v)
    return out


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = build_oracle.build()
            L = ctypes.CDLL(str(path))
            f3 = ctypes.POINTER(ctypes.c_float)
            u32 = ctypes.POINTER(ctypes.c_uint32)
            i32 = ctypes.POINTER(ctypes.c_int)
            for tag, rp in (("f32", ctypes.POINTER(ctypes.c_float)), ("f64", ctypes.POINTER(ctypes.c_double))):
                fn = getattr(L, f"oracle_step_{tag}")
                fn.argtypes = [ctypes.POINTER(OracleParams), f3, f3, rp, rp, rp, rp, u32, ctypes.c_int, rp, rp]
                fn.restype = ctypes.c_int
                fn = getattr(L, f"oracle_grid_{tag}")
                fn.argtypes = [ctypes.POINTER(OracleParams), f3, f3, rp, ctypes.c_int, u32, u32, u32, u32, i32]
                fn.restype = ctypes.c_int
                fn = getattr(L, f"oracle_predict_{tag}")
                fn.argtypes = [ctypes.POINTER(OracleParams), rp, rp, ctypes.c_int, rp]
                fn.restype = ctypes.c_int
                fn = getattr(L, f"oracle_step_backward_{tag}")
                fn.argtypes = [ctypes.POINTER(OracleParams), f3, f3, rp, rp, u32, ctypes.c_int, rp, rp, rp, rp, rp, rp]
                fn.restype = ctypes.c_int
                fn = getattr(L, f"oracle_threads_{tag}")
                fn.argtypes = []
                fn.restype = ctypes.c_int
            _lib = L
    return _lib


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _dtype(prec: str):
    if prec == "f32":
        return np.float32, ctypes.c_float
    if prec == "f64":
        return np.float64, ctypes.c_double
    raise ValueError(f"precision must be 'f32' or 'f64', not {prec!r}")


def _lim(v) -> ctypes.Array:
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def threads() -> int:
    return int(lib().oracle_threads_f32())


def step(params, ulim, llim, pos, vel, iid, prec: str = "f32"):
    """One reference step on host arrays.

    pos, vel: (n, 4) arrays (converted to the precision's dtype), iid: (n,) uint32.
    Returns a dict with the reference's outputs: pos, vel, iid (permuted into
    cell order; vel = (npos - pos) / dt), npos, nvel, rho and lambda of the last
    lambda pass.  Inputs are not modified.
    """
    dt, ct = _dtype(prec)
    pos = np.ascontiguousarray(pos, dtype=dt).copy()
    vel = np.ascontiguousarray(vel, dtype=dt).copy()
    iid = np.ascontiguousarray(iid, dtype=np.uint32).copy()
    n = pos.shape[0]
    assert pos.shape == (n, 4) and vel.shape == (n, 4) and iid.shape == (n,)
    npos = np.zeros_like(pos)
    nvel = np.zeros_like(vel)
    rho = np.zeros(n, dtype=dt)
    lam = np.zeros(n, dtype=dt)
    op = to_oracle_params(params)
    fn = getattr(lib(), f"oracle_step_{prec}")
    rc = fn(ctypes.byref(op), _lim(ulim), _lim(llim), _ptr(pos, ct), _ptr(npos, ct), _ptr(vel, ct),
            _ptr(nvel, ct), _ptr(iid, ctypes.c_uint32), n, _ptr(rho, ct), _ptr(lam, ct))
    if rc != 0:
        raise ValueError(f"oracle_step_{prec} rejected its arguments (rc={rc})")
    return {"pos": pos, "vel": vel, "iid": iid, "npos": npos, "nvel": nvel, "rho": rho, "lambda": lam}


def grid(params, ulim, llim, xstar, prec: str = "f32"):
    """The reference's neighbour grid for predicted positions xstar ((n, 4)).

    Returns keys (input order), perm (input index per sorted slot), start/end
    per cell (0/0 for empty cells) and dims.
    """
    dt, ct = _dtype(prec)
    xs = np.ascontiguousarray(xstar, dtype=dt)
    n = xs.shape[0]
    op = to_oracle_params(params)
    dims = np.zeros(3, dtype=np.int32)
    fn = getattr(lib(), f"oracle_grid_{prec}")
    keys = np.zeros(max(n, 1), dtype=np.uint32)
    perm = np.zeros(max(n, 1), dtype=np.uint32)
    # first call: dims only
    null = ctypes.POINTER(ctypes.c_uint32)()
    fn(ctypes.byref(op), _lim(ulim), _lim(llim), _ptr(xs, ct), 0, null, null, null, null,
       _ptr(dims, ctypes.c_int))
    cells = int(np.prod(dims.astype(np.int64)))
    start = np.zeros(cells, dtype=np.uint32)
    end = np.zeros(cells, dtype=np.uint32)
    rc = fn(ctypes.byref(op), _lim(ulim), _lim(llim), _ptr(xs, ct), n, _ptr(keys, ctypes.c_uint32),
            _ptr(perm, ctypes.c_uint32), _ptr(start, ctypes.c_uint32), _ptr(end, ctypes.c_uint32),
            _ptr(dims, ctypes.c_int))
    if rc != 0:
        raise ValueError(f"oracle_grid_{prec} rejected its arguments (rc={rc})")
    return {"keys": keys[:n], "perm": perm[:n], "start": start, "end": end, "dims": tuple(int(d) for d in dims)}


def predict(params, pos, vel, prec: str = "f32"):
    """advect_kernel's predicted positions (fluids/Simulator_kernel.cuh:14-15),
    with the fused multiply-adds nvcc emits: v' = fma(dt, g, v), x* = fma(dt, v', x)."""
    dt, ct = _dtype(prec)
    pos = np.ascontiguousarray(pos, dtype=dt)
    vel = np.ascontiguousarray(vel, dtype=dt)
    out = np.zeros_like(pos)
    op = to_oracle_params(params)
    rc = getattr(lib(), f"oracle_predict_{prec}")(ctypes.byref(op), _ptr(pos, ct), _ptr(vel, ct), pos.shape[0],
                                                  _ptr(out, ct))
    if rc != 0:
        raise ValueError("oracle_predict rejected its arguments")
    return out


def step_backward(params, ulim, llim, pos, vel, iid, g_npos, g_nvel, prec: str = "f64"):
    """Reverse pass of one step: the exact transpose of oracle step (neighbour
    sets and clamp states fixed).  g_npos/g_nvel: adjoints of the step's
    outputs, in its output (cell) order.  Returns adjoints of the inputs pos
    and vel (input order) and of the limits ulim, llim."""
    dt, ct = _dtype(prec)
    pos = np.ascontiguousarray(pos, dtype=dt)
    vel = np.ascontiguousarray(vel, dtype=dt)
    iid = np.ascontiguousarray(iid, dtype=np.uint32)
    gn = np.ascontiguousarray(g_npos, dtype=dt)
    gv = np.ascontiguousarray(g_nvel, dtype=dt)
    n = pos.shape[0]
    g_pos = np.zeros_like(pos)
    g_vel = np.zeros_like(vel)
    gu = np.zeros(3, dtype=dt)
    gl = np.zeros(3, dtype=dt)
    op = to_oracle_params(params)
    fn = getattr(lib(), f"oracle_step_backward_{prec}")
    rc = fn(ctypes.byref(op), _lim(ulim), _lim(llim), _ptr(pos, ct), _ptr(vel, ct), _ptr(iid, ctypes.c_uint32), n,
            _ptr(gn, ct), _ptr(gv, ct), _ptr(g_pos, ct), _ptr(g_vel, ct), _ptr(gu, ct), _ptr(gl, ct))
    if rc != 0:
        raise ValueError(f"oracle_step_backward_{prec} rejected its arguments (rc={rc})")
    return {"pos": g_pos, "vel": g_vel, "ulim": gu, "llim": gl}


def _nodes(lo, hi, dims):
    lo = np.asarray(lo, np.float64)
    step = (np.asarray(hi, np.float64) - lo) / np.asarray(dims, np.float64)
    axes = [lo[a] + (np.arange(dims[a]) + 0.5) * step[a] for a in range(3)]
    gx, gy, gz = np.meshgrid(*axes, indexing="ij")
    return np.stack([gx.ravel(), gy.ravel(), gz.ravel()], 1)


def _node_pairs(x, lo, hi, dims, h):
    """Every (particle, node) pair closer than h: particle indices, flat node
    indices and r = x - node.  A node within h of a particle lies within
    h / step of its lattice coordinate u, so within ceil(h / step + 0.5) of
    rint(u): those nodes are tested."""
    lo = np.asarray(lo, np.float64)
    dims = np.asarray(dims, np.int64)
    step = (np.asarray(hi, np.float64) - lo) / dims
    u = (x - lo) / step - 0.5  # lattice coordinate of the particle (node k sits at k)
    base = np.rint(u).astype(np.int64)
    reach = [int(np.ceil(h / step[a] + 0.5)) for a in range(3)]
    offs = np.stack(np.meshgrid(*[np.arange(-r, r + 1) for r in reach], indexing="ij"), -1).reshape(-1, 3)
    k = base[:, None, :] + offs[None, :, :]                      # (n, m, 3) node indices
    inside = np.all((k >= 0) & (k < dims), -1)
    node = lo + (k + 0.5) * step
    r = x[:, None, :] - node
    q = (r * r).sum(-1)
    hit = inside & (q < h * h)
    pi, mi = np.nonzero(hit)
    kk = k[pi, mi]
    flat = (kk[:, 0] * dims[1] + kk[:, 1]) * dims[2] + kk[:, 2]
    return pi, flat, r[pi, mi], q[pi, mi]


def density_grid(pos, lo, hi, dims, h):
    """FP64 poly6 density (mass 1, radius h) at the centres of the dims cells
    spanning [lo, hi] (x slowest).  The inverse problem's loss term; the
    reference has none, so this restatement is checked against finite
    differences instead."""
    x = np.asarray(pos, np.float64)[:, :3]
    coef = 315.0 / (64.0 * np.pi * h ** 9)
    pi, flat, _, q = _node_pairs(x, lo, hi, dims, h)
    out = np.bincount(flat, weights=coef * (h * h - q) ** 3, minlength=int(np.prod(dims)))
    return out.reshape(tuple(dims))


def density_grid_backward(pos, lo, hi, dims, h, g_grid):
    """Adjoint of ``density_grid`` w.r.t. the positions, (n, 4) FP64."""
    x = np.asarray(pos, np.float64)[:, :3]
    g = np.asarray(g_grid, np.float64).ravel()
    coef = 315.0 / (64.0 * np.pi * h ** 9)
    out = np.zeros((len(x), 4))
    pi, flat, r, q = _node_pairs(x, lo, hi, dims, h)
    w = h * h - q
    dq = g[flat] * (-3.0 * coef * w * w) * 2.0
    for a in range(3):
        out[:, a] = np.bincount(pi, weights=dq * r[:, a], minlength=len(x))
    return out


# ---- screen-space fluid renderer (oracle/ssf_oracle.c) ------------------------------------

class OracleSsfParams(ctypes.Structure):
    """Field-for-field mirror of ``pbf_ssf_params`` (include/pbf_ssf.h)."""

    _fields_ = [
        ("width", ctypes.c_int), ("height", ctypes.c_int),
        ("view", ctypes.c_float * 16), ("proj", ctypes.c_float * 16),
        ("p_n", ctypes.c_float), ("p_f", ctypes.c_float), ("p_t", ctypes.c_float), ("p_r", ctypes.c_float),
        ("radius", ctypes.c_float),
        ("smooth_niter", ctypes.c_int), ("kernel_r", ctypes.c_int),
        ("sigma_r", ctypes.c_float), ("sigma_z", ctypes.c_float),
        ("keep_edge", ctypes.c_int), ("blur_option", ctypes.c_int), ("shading_option", ctypes.c_int),
        ("r0", ctypes.c_float), ("sky", ctypes.c_float * 3),
    ]


def to_oracle_ssf_params(p) -> OracleSsfParams:
    """Copy any object with pbf_ssf_params' field names into an OracleSsfParams."""
    out = OracleSsfParams()
    for name, ctype in OracleSsfParams._fields_:
        v = getattr(p, name)
        if hasattr(ctype, "_length_"):
            arr = getattr(out, name)
            for k in range(ctype._length_):
                arr[k] = float(v[k])
        else:
            setattr(out, name, v)
    return out


def ssf_render(params, pos, sky=None, color=None, prec: str = "f32"):
    """The reference's SSF render (fluids/SSFRenderer.cpp:113-146) on host arrays.

    pos: (n, 4) float32 positions; sky: optional (6, S, S, 3) float32 cube map;
    color: optional (H, W, 4) float32 image the shading writes into (a copy is
    returned).  Returns a dict of (H, W[, 4]) float32 images depth_raw, depth,
    thick, normal_D, color, and the fragment count."""
    L = lib()
    fn = getattr(L, f"oracle_ssf_render_{prec}")
    f32p = ctypes.POINTER(ctypes.c_float)
    fn.argtypes = [ctypes.POINTER(OracleSsfParams), f32p, ctypes.c_int, f32p, ctypes.c_int, f32p, f32p, f32p, f32p,
                   f32p]
    fn.restype = ctypes.c_longlong
    op = to_oracle_ssf_params(params)
    W, H = op.width, op.height
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    n = pos.shape[0]
    if n:
        assert pos.shape == (n, 4)
    out = {k: np.zeros((H, W), np.float32) for k in ("depth_raw", "depth", "thick")}
    out["normal_D"] = np.zeros((H, W, 4), np.float32)
    out["color"] = (np.zeros((H, W, 4), np.float32) if color is None
                    else np.ascontiguousarray(color, dtype=np.float32).copy())
    if sky is not None:
        sky = np.ascontiguousarray(sky, dtype=np.float32)
        assert sky.ndim == 4 and sky.shape[0] == 6 and sky.shape[1] == sky.shape[2] and sky.shape[3] == 3
    null = f32p()
    frags = fn(ctypes.byref(op), _ptr(pos, ctypes.c_float) if n else null, n,
               _ptr(sky, ctypes.c_float) if sky is not None else null, 0 if sky is None else sky.shape[1],
               _ptr(out["depth_raw"], ctypes.c_float), _ptr(out["depth"], ctypes.c_float),
               _ptr(out["thick"], ctypes.c_float), _ptr(out["normal_D"], ctypes.c_float),
               _ptr(out["color"], ctypes.c_float))
    if frags < 0:
        raise ValueError(f"oracle_ssf_render_{prec} rejected its arguments")
    out["fragments"] = int(frags)
    return out


def ssf_smooth(params, raw, prec: str = "f32"):
    """smooth_niter smoothing passes from a splatted depth image (H, W)."""
    f32p = ctypes.POINTER(ctypes.c_float)
    fn = getattr(lib(), f"oracle_ssf_smooth_{prec}")
    fn.argtypes = [ctypes.POINTER(OracleSsfParams), f32p, f32p]
    fn.restype = ctypes.c_int
    raw = np.ascontiguousarray(raw, dtype=np.float32)
    out = np.zeros_like(raw)
    if fn(ctypes.byref(to_oracle_ssf_params(params)), _ptr(raw, ctypes.c_float), _ptr(out, ctypes.c_float)) != 0:
        raise ValueError("oracle_ssf_smooth rejected its arguments")
    return out


def ssf_normals(params, depth, prec: str = "f32"):
    """Normal restoration of a depth image (H, W) -> (H, W, 4)."""
    f32p = ctypes.POINTER(ctypes.c_float)
    fn = getattr(lib(), f"oracle_ssf_normals_{prec}")
    fn.argtypes = [ctypes.POINTER(OracleSsfParams), f32p, f32p]
    fn.restype = ctypes.c_int
    depth = np.ascontiguousarray(depth, dtype=np.float32)
    out = np.zeros(depth.shape + (4,), np.float32)
    if fn(ctypes.byref(to_oracle_ssf_params(params)), _ptr(depth, ctypes.c_float), _ptr(out, ctypes.c_float)) != 0:
        raise ValueError("oracle_ssf_normals rejected its arguments")
    return out


def ssf_shade(params, depth, normal_D, thick, color, sky=None, prec: str = "f32"):
    """Shading of given images; returns a shaded copy of color (H, W, 4)."""
    f32p = ctypes.POINTER(ctypes.c_float)
    fn = getattr(lib(), f"oracle_ssf_shade_{prec}")
    fn.argtypes = [ctypes.POINTER(OracleSsfParams), f32p, f32p, f32p, f32p, ctypes.c_int, f32p]
    fn.restype = ctypes.c_int
    depth = np.ascontiguousarray(depth, dtype=np.float32)
    nd = np.ascontiguousarray(normal_D, dtype=np.float32)
    th = np.ascontiguousarray(thick, dtype=np.float32)
    out = np.ascontiguousarray(color, dtype=np.float32).copy()
    sk = None if sky is None else np.ascontiguousarray(sky, dtype=np.float32)
    rc = fn(ctypes.byref(to_oracle_ssf_params(params)), _ptr(depth, ctypes.c_float), _ptr(nd, ctypes.c_float),
            _ptr(th, ctypes.c_float), _ptr(sk, ctypes.c_float) if sk is not None else f32p(),
            0 if sk is None else sk.shape[1], _ptr(out, ctypes.c_float))
    if rc != 0:
        raise ValueError("oracle_ssf_shade rejected its arguments")
    return out


# ---- the reference's own SSF shaders on the CPU (oracle/ref_harness/ssf_ref.cpp) ----------

_ssf_ref = None


def ssf_ref_available() -> bool:
    """Whether the reference's shaders can be built here (its sources are present)."""
    from .ref_harness import build_ref

    return build_ref.ssf_shaders_present() or build_ref.ssf_ref_path().exists()


def _ssf_ref_lib():
    global _ssf_ref
    with _lock:
        if _ssf_ref is None:
            from .ref_harness import build_ref

            path = build_ref.build_ssf_ref() if build_ref.ssf_shaders_present() else build_ref.ssf_ref_path()
            L = ctypes.CDLL(str(path))
            f32p = ctypes.POINTER(ctypes.c_float)
            P = ctypes.POINTER(OracleSsfParams)
            L.ssf_ref_splat.argtypes = [P, f32p, ctypes.c_int, f32p, f32p]
            L.ssf_ref_splat.restype = ctypes.c_longlong
            L.ssf_ref_smooth.argtypes = [P, f32p, f32p]
            L.ssf_ref_normals.argtypes = [P, f32p, f32p]
            L.ssf_ref_shade.argtypes = [P, f32p, f32p, f32p, f32p, ctypes.c_int, f32p]
            for fn in (L.ssf_ref_smooth, L.ssf_ref_normals, L.ssf_ref_shade):
                fn.restype = ctypes.c_int
            _ssf_ref = L
    return _ssf_ref


def ssf_ref_splat(params, pos):
    """renderDepth + renderThick run through the reference's shaders: (depth,
    thick, fragments)."""
    op = to_oracle_ssf_params(params)
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    depth = np.zeros((op.height, op.width), np.float32)
    thick = np.zeros_like(depth)
    n = pos.shape[0]
    f = _ssf_ref_lib().ssf_ref_splat(ctypes.byref(op), _ptr(pos, ctypes.c_float) if n else None, n,
                                     _ptr(depth, ctypes.c_float), _ptr(thick, ctypes.c_float))
    return depth, thick, int(f)


def ssf_ref_smooth(params, raw):
    op = to_oracle_ssf_params(params)
    raw = np.ascontiguousarray(raw, dtype=np.float32)
    out = np.zeros_like(raw)
    _ssf_ref_lib().ssf_ref_smooth(ctypes.byref(op), _ptr(raw, ctypes.c_float), _ptr(out, ctypes.c_float))
    return out


def ssf_ref_normals(params, depth):
    op = to_oracle_ssf_params(params)
    depth = np.ascontiguousarray(depth, dtype=np.float32)
    out = np.zeros(depth.shape + (4,), np.float32)
    _ssf_ref_lib().ssf_ref_normals(ctypes.byref(op), _ptr(depth, ctypes.c_float), _ptr(out, ctypes.c_float))
    return out


def ssf_ref_shade(params, depth, normal_D, thick, color, sky=None):
    op = to_oracle_ssf_params(params)
    depth = np.ascontiguousarray(depth, dtype=np.float32)
    nd = np.ascontiguousarray(normal_D, dtype=np.float32)
    th = np.ascontiguousarray(thick, dtype=np.float32)
    out = np.ascontiguousarray(color, dtype=np.float32).copy()
    sk = None if sky is None else np.ascontiguousarray(sky, dtype=np.float32)
    rc = _ssf_ref_lib().ssf_ref_shade(ctypes.byref(op), _ptr(depth, ctypes.c_float), _ptr(nd, ctypes.c_float),
                                      _ptr(th, ctypes.c_float), _ptr(sk, ctypes.c_float) if sk is not None else None,
                                      0 if sk is None else sk.shape[1], _ptr(out, ctypes.c_float))
    if rc != 0:
        raise ValueError("ssf_ref_shade rejected its arguments")
    return out
