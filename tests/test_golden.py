"""Golden vectors: outputs of the reference's own kernels.

tests/golden/ref_*.npz were produced by tests/golden/make_golden.py, which runs
fluids/Simulator.cu + fluids/Simulator_kernel.cuh compiled unmodified for
sm_103a with Simulator::step's host sequencing (oracle/ref_harness).  The
CPU tests pin the oracle to them; the GPU tests hold the CUDA path to the same
bars:
  * cell order (iid), permuted positions, sorted cell ids, start/end: bit-exact;
  * positions within 1e-5 h, velocities within 1e-5 h / dt + 1e-5 |v|,
    density within 1e-5 relative, for every case except the chaotic one (dam-break parameters
    at 4 iterations, where FP32 rounding alone moves particles by ~1e-2): there
    the integer outputs, the set of particles left without density, and the
    set of non-finite velocities must match, and the CUDA path's floats are
    held to the reference's own float arithmetic as closely as the float port
    of the reference's kernels is: the median, 90th and 99th percentile of
    |CUDA - reference kernels| in positions, velocities and densities within
    1e-5 h (1e-5 h / dt, 1e-5 of the largest density) + 3x the same
    percentile of |float port - reference kernels| of the same step; the
    maximum (one worst particle of 1,728) within the floor + 3x the larger of
    the float port's and the FP64 oracle's maximum (the FP64 restatement is
    itself 6x farther than the port from the reference's float results there).
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("ref_*.npz"))
CHAOTIC = {"ref_dam1728_sceneparams_niter4"}
H = 0.1
TOL_X = 1e-5 * H


def load_case(pbf, name):
    z = np.load(GOLDEN / f"{name}.npz")
    p = pbf.PbfParams()
    for k, v in json.loads(str(z["params"])).items():
        if k == "up":
            for a in range(3):
                p.up[a] = v[a]
        else:
            setattr(p, k, v)
    return z, p


def as4(a3):
    out = np.zeros((a3.shape[0], 4), np.float32)
    out[:, :3] = a3
    return out


def steps_of(z):
    """(step index, input pos, input vel, input iid) per recorded step; step k+1
    starts from the reference's own outputs of step k."""
    pos, vel, iid = z["in_pos"], z["in_vel"], z["in_iid"]
    for s in range(int(z["steps"])):
        yield s, as4(pos), as4(vel), iid
        pos, vel, iid = z[f"s{s}_npos"], z[f"s{s}_nvel"], z[f"s{s}_iid"]


def check_against(z, s, got, name, p, what):
    np.testing.assert_array_equal(got["iid"], z[f"s{s}_iid"], err_msg=f"{what}: iid")
    np.testing.assert_array_equal(got["pos"][:, :3], z[f"s{s}_pos"], err_msg=f"{what}: permuted pos")
    if name in CHAOTIC:
        np.testing.assert_array_equal(got["rho"] == 0, z[f"s{s}_rho"] == 0, err_msg=f"{what}: rho == 0 set")
        np.testing.assert_array_equal(~np.isfinite(got["nvel"][:, :3]).all(1), ~np.isfinite(z[f"s{s}_nvel"]).all(1),
                                      err_msg=f"{what}: non-finite nvel set")
        return
    assert np.abs(got["npos"][:, :3] - z[f"s{s}_npos"]).max() <= TOL_X, what
    for k in ("vel", "nvel"):  # the position bar over dt, plus 1e-5 relative for fast particles
        ref = z[f"s{s}_{k}"]
        assert np.all(np.abs(got[k][:, :3] - ref) <= TOL_X / p.dt + 1e-5 * np.abs(ref)), (what, k)
    rho = z[f"s{s}_rho"]
    assert np.abs(got["rho"] - rho).max() <= 1e-5 * rho.max(), what


def test_golden_cases_present():
    assert len(CASES) >= 5


@pytest.mark.parametrize("name", CASES)
def test_oracle_grid_matches_reference(pbf, oracle, name):
    z, p = load_case(pbf, name)
    for s, pos, vel, iid in steps_of(z):
        xs = oracle.predict(p, pos, vel)
        g = oracle.grid(p, z["ulim"], z["llim"], xs)
        assert g["dims"] == tuple(int(d) for d in z["dims"])
        np.testing.assert_array_equal(g["keys"][g["perm"]], z[f"s{s}_ids"])
        np.testing.assert_array_equal(iid[g["perm"]], z[f"s{s}_iid"])
        np.testing.assert_array_equal(g["start"], z[f"s{s}_start"])
        np.testing.assert_array_equal(g["end"], z[f"s{s}_end"])


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("name", CASES)
def test_oracle_step_matches_reference(pbf, oracle, name, prec):
    z, p = load_case(pbf, name)
    for s, pos, vel, iid in steps_of(z):
        r = oracle.step(p, z["ulim"], z["llim"], pos, vel, iid, prec=prec)
        check_against(z, s, r, name, p, f"oracle {prec} {name} step {s}")


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_cuda_step_matches_reference(pbf, oracle, cuda, name):
    import torch

    z, p = load_case(pbf, name)
    for s, pos, vel, iid in steps_of(z):
        n = pos.shape[0]
        d = {k: torch.from_numpy(v.copy()).cuda() for k, v in (("pos", pos), ("vel", vel))}
        d["npos"] = torch.zeros(n, 4, device="cuda")
        d["nvel"] = torch.zeros(n, 4, device="cuda")
        d["iid"] = torch.from_numpy(iid.astype(np.int32)).cuda()
        with pbf.Simulator(p, tuple(z["ulim"]), tuple(z["llim"]), n) as sim:
            sim.step(d["pos"], d["npos"], d["vel"], d["nvel"], d["iid"], n)
            rho = sim.density(n)
            torch.cuda.synchronize()
        got = {k: v.cpu().numpy() for k, v in d.items()}
        got["iid"] = got["iid"].astype(np.uint32)
        got["rho"] = rho.cpu().numpy()
        check_against(z, s, got, name, p, f"cuda {name} step {s}")
        if name in CHAOTIC:
            port = oracle.step(p, z["ulim"], z["llim"], pos, vel, iid, prec="f32")
            fp64 = oracle.step(p, z["ulim"], z["llim"], pos, vel, iid, prec="f64")
            check_port_relative(z, s, got, port, fp64, p, f"cuda {name} step {s}")


def check_port_relative(z, s, got, port, fp64, p, what):
    """Error percentiles of the CUDA path against the reference's kernels
    within a floor + 3x those of the float port of the same step (the
    maximum: 3x the larger of the port's and the FP64 oracle's)."""
    rho_ref = z[f"s{s}_rho"]
    for k, ref, floor in (("npos", z[f"s{s}_npos"], TOL_X), ("nvel", z[f"s{s}_nvel"], TOL_X / p.dt),
                          ("rho", rho_ref, 1e-5 * float(rho_ref.max()))):
        def cols(a):
            return a[:, :3] if k != "rho" else np.asarray(a)[:, None]

        g, q, f, r = cols(got[k]), cols(port[k]), cols(fp64[k]), cols(ref)
        fin = np.isfinite(r).all(1)
        np.testing.assert_array_equal(np.isfinite(g).all(1), fin, err_msg=f"{what}: {k} non-finite set")
        e_gpu = np.abs(g[fin] - r[fin]).ravel()
        e_port = np.abs(q[fin] - r[fin]).ravel()
        for pct in (50, 90, 99):
            a, b = float(np.percentile(e_gpu, pct)), float(np.percentile(e_port, pct))
            assert a <= floor + 3 * b, (what, k, pct, a, b)
        worst = max(float(e_port.max()), float(np.abs(f[fin] - r[fin]).max()))
        assert float(e_gpu.max()) <= floor + 3 * worst, (what, k, "max", float(e_gpu.max()), worst)
