"""Generate the golden vectors in tests/golden/ by running the reference's own
kernels on a GPU.

The reference (naeioi/PBF-CUDA) ships no tests or fixtures.  These vectors are
outputs of its kernels — fluids/Simulator.cu and fluids/Simulator_kernel.cuh,
compiled unmodified for sm_103a by oracle/ref_harness/build_ref.py — driven
with Simulator::step's host sequencing by oracle/ref_harness/ref_launch.cu.
Needs a GPU and oracle/_ref/ref_kernels.cubin (built where the reference
sources are).  Usage:

    python tests/golden/make_golden.py [out_dir]

Each case is an .npz with the inputs (pos, vel, iid, limits, parameters) and,
per step, everything the reference step leaves behind.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def params_dict(p) -> dict:
    return {name: ([float(x) for x in getattr(p, name)] if name == "up" else getattr(p, name))
            for name, _ in p._fields_}


def run_case(ref, name, p, ulim, llim, pos, vel, iid, steps, out_dir):
    rec = {"params": np.array(json.dumps(params_dict(p))), "ulim": np.array(ulim, np.float32),
           "llim": np.array(llim, np.float32), "in_pos": pos[:, :3].astype(np.float32),
           "in_vel": vel[:, :3].astype(np.float32), "in_iid": iid.astype(np.uint32), "steps": np.array(steps)}
    cur_pos, cur_vel, cur_iid = pos[:, :3].astype(np.float32), vel[:, :3].astype(np.float32), iid.astype(np.uint32)
    for s in range(steps):
        r = ref.step(p, ulim, llim, cur_pos, cur_vel, cur_iid)
        for k in ("pos", "vel", "npos", "nvel", "iid", "rho", "lambda", "ids", "start", "end"):
            rec[f"s{s}_{k}"] = r[k]
        rec["dims"] = np.array(r["dims"], np.int32)
        cur_pos, cur_vel, cur_iid = r["npos"], r["nvel"], r["iid"]
    out = Path(out_dir) / f"ref_{name}.npz"
    np.savez_compressed(out, **rec)
    print(f"{out}: n={pos.shape[0]} steps={steps} {out.stat().st_size} B")


def main():
    import __graft_entry__
    from oracle.ref_harness import ref

    pbf = __graft_entry__.load()
    sc = pbf.scenes
    out_dir = sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).resolve().parent)
    Path(out_dir).mkdir(parents=True, exist_ok=True)

    ref_p = pbf.default_params()           # the reference's own parameters, y up
    ref_p.up[0], ref_p.up[1], ref_p.up[2] = 0.0, 1.0, 0.0
    box_u, box_l = (1.2, 1.0, 0.8), (0.0, 0.0, 0.0)
    rng = np.random.default_rng(101)
    lat = sc.lattice((12, 12, 12), (0.0, 0.0, 0.0), rng)
    zero = np.zeros_like(lat)
    ids = np.arange(lat.shape[0], dtype=np.uint32)

    run_case(ref, "dam1728_refparams", ref_p, box_u, box_l, lat, zero, ids, 2, out_dir)

    scene_p = sc.scene_params(niter=1)
    run_case(ref, "dam1728_sceneparams_niter1", scene_p, box_u, box_l, lat, zero, ids, 1, out_dir)
    run_case(ref, "dam1728_sceneparams_niter4", sc.scene_params(niter=4), box_u, box_l, lat, zero, ids, 1, out_dir)

    # shuffled order, random velocities, boundary density term, a narrower box
    p = pbf.default_params()
    p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
    p.niter = 2
    p.k_boundaryDensity = 0.05
    order = rng.permutation(lat.shape[0])
    vel = np.zeros_like(lat)
    vel[:, :3] = rng.normal(0, 0.3, size=(lat.shape[0], 3))
    run_case(ref, "moving1728", p, (0.9, 1.0, 0.8), box_l, lat[order], vel, order.astype(np.uint32), 1, out_dir)

    # the grid alone: x* = x (no gravity, no velocity), positions in and out of the box
    p = pbf.default_params()
    p.g = 0.0
    p.niter = 1
    pos = np.zeros((3000, 4), np.float32)
    pos[:, :3] = rng.uniform((-0.2, -0.2, -0.2), (1.4, 1.2, 1.0), size=(3000, 3))
    run_case(ref, "grid3000", p, box_u, box_l, pos, np.zeros_like(pos), np.arange(3000, dtype=np.uint32), 1,
             out_dir)


if __name__ == "__main__":
    main()
