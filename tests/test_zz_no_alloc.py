"""pbf_step_noalloc, the step for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc: a host application whose device memory is
owned by its own memory manager (a fixed arena a plug-in must not grow), or a
real-time loop that cannot take the device-wide synchronisation an allocation
may cause.  pbf_step_noalloc serves them with scratch in a fixed array inside
the library, so it is limited to 32768 particles.  This test calls it through
the C ABI and checks it against pbf_step on the same inputs, for two calls in a
row (the second call starts from the first call's outputs and reuses the
array, which still holds the first call's contents): both run the same kernels
in the same order, so the results must be bitwise equal (a tolerance would hide
a stale-scratch bug that moves a value by one ulp).  One call is also checked
against the FP64 oracle at the parity tests' one-step bar.  It lives in its own
file, named to be collected last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_X = 1e-5 * 0.1  # 1e-5 h, the one-step bar of the parity tests


def _vec(v):
    return (ctypes.c_float * 3)(*v)


def test_noalloc_matches_pbf_step_twice(pbf, cuda):
    import torch

    sc = pbf.scenes.double_dam(seed=2)  # 32,768 particles: the array's limit
    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    n = sc.n
    L = pbf.lib()

    def bufs():
        d = {k: torch.zeros(n, 4, device="cuda") for k in ("pos", "vel", "npos", "nvel")}
        d["pos"].copy_(torch.from_numpy(sc.pos))
        d["vel"].copy_(torch.from_numpy(sc.vel))
        d["iid"] = torch.arange(n, dtype=torch.int32, device="cuda")
        return d

    a, b = bufs(), bufs()
    stream = torch.cuda.current_stream().cuda_stream
    with pbf.Simulator(p, sc.ulim, sc.llim, n) as sim:
        for call in range(2):
            src_a = ("pos", "npos", "vel", "nvel") if call == 0 else ("npos", "pos", "nvel", "vel")
            sim.step(a[src_a[0]], a[src_a[1]], a[src_a[2]], a[src_a[3]], a["iid"], n)
            st = L.pbf_step_noalloc(ctypes.byref(p), _vec(sc.ulim), _vec(sc.llim), b[src_a[0]].data_ptr(),
                                    b[src_a[1]].data_ptr(), b[src_a[2]].data_ptr(), b[src_a[3]].data_ptr(),
                                    b["iid"].data_ptr(), n, stream)
            pbf.check(st, "pbf_step_noalloc")
            torch.cuda.synchronize()
            # every output bitwise equal: new state, velocities, permuted inputs, cell order
            for k in ("pos", "vel", "npos", "nvel", "iid"):
                assert torch.equal(a[k].view(torch.int32), b[k].view(torch.int32)), (call, k)


def test_noalloc_matches_fp64_oracle(pbf, oracle, cuda):
    import torch

    sc = pbf.scenes.double_dam(seed=3)
    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    n = sc.n
    d = {k: torch.zeros(n, 4, device="cuda") for k in ("pos", "vel", "npos", "nvel")}
    d["pos"].copy_(torch.from_numpy(sc.pos))
    d["vel"].copy_(torch.from_numpy(sc.vel))
    d["iid"] = torch.arange(n, dtype=torch.int32, device="cuda")
    st = pbf.lib().pbf_step_noalloc(ctypes.byref(p), _vec(sc.ulim), _vec(sc.llim), d["pos"].data_ptr(),
                                    d["npos"].data_ptr(), d["vel"].data_ptr(), d["nvel"].data_ptr(),
                                    d["iid"].data_ptr(), n, torch.cuda.current_stream().cuda_stream)
    pbf.check(st, "pbf_step_noalloc")
    torch.cuda.synchronize()
    r = oracle.step(p, sc.ulim, sc.llim, sc.pos.astype(np.float64), sc.vel.astype(np.float64),
                    np.arange(n, dtype=np.uint32), "f64")
    np.testing.assert_array_equal(d["iid"].cpu().numpy().astype(np.uint32), r["iid"])
    assert np.abs(d["npos"].cpu().numpy()[:, :3] - r["npos"][:, :3]).max() <= TOL_X


def test_noalloc_rejects_sizes_beyond_its_limit(pbf, cuda):
    import torch

    L = pbf.lib()
    p = pbf.default_params()
    t = [torch.zeros(32769, 4, device="cuda") for _ in range(4)]
    iid = torch.zeros(32769, dtype=torch.int32, device="cuda")
    st = L.pbf_step_noalloc(ctypes.byref(p), _vec((1.0, 1.0, 1.0)), _vec((0.0, 0.0, 0.0)), t[0].data_ptr(),
                            t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), iid.data_ptr(), 32769, None)
    assert st == pbf.PBF_ERR_CAPACITY
    assert b"32768" in L.pbf_last_error()
    # a box of more than 131072 cells at h = 0.1
    st = L.pbf_step_noalloc(ctypes.byref(p), _vec((10.0, 10.0, 10.0)), _vec((0.0, 0.0, 0.0)), t[0].data_ptr(),
                            t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), iid.data_ptr(), 100, None)
    assert st == pbf.PBF_ERR_CAPACITY
