"""Generate tests/golden/stats_*.npz: density-constraint statistics of long
runs of the reference's own kernels (300 frames = 600 steps), for the
statistical parity test (tests/test_gpu_stats.py).

Trajectories of this solver diverge chaotically from run to run of different
FP32 code, so long runs are compared through statistics: per step, over the
particles, the mean and the max of the compression part max(C_i, 0) of the
constraint C_i = rho_i / rho0 - 1, with rho_i from the step's last lambda
pass.  Needs a GPU and oracle/_ref/ref_kernels.cubin (built where the
reference sources are; see oracle/ref_harness).  Cases: the 8,000-particle
dam break and the 32,768-particle double dam break, each with the dam-break
parameters and with the reference's own defaults.  Usage:

    python tests/golden/make_stats.py [out_dir [case ...]]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

STEPS = 600


def constraint_stats(rho: np.ndarray, rho0: float):
    """(mean, max) of max(C, 0) over the particles with finite rho, and the
    count of non-finite rho."""
    fin = np.isfinite(rho)
    c = np.maximum(rho[fin].astype(np.float64) / rho0 - 1.0, 0.0)
    return (float(c.mean()) if c.size else 0.0, float(c.max()) if c.size else 0.0, int((~fin).sum()))


SEEDS = tuple(range(32))
# seeds of each case (lattice jitter); the 32K double dam runs fewer
CASE_SEEDS = {"dam8k_sceneparams": SEEDS, "dam8k_refparams": SEEDS,
              "ddam32k_sceneparams": tuple(range(8)), "ddam32k_refparams": SEEDS}


def cases(pbf, seed=0):
    """The 8,000-particle dam break and the 32,768-particle double dam break
    (lattice jitter from ``seed``), each with the dam-break parameters and with
    the reference's own defaults (y up)."""
    ref_p = pbf.scenes.reference_params()
    ref_p.up[0], ref_p.up[1], ref_p.up[2] = 0.0, 1.0, 0.0
    dam = pbf.scenes.dam_break(seed=seed)
    ddam = pbf.scenes.double_dam(seed=seed)
    return {
        "dam8k_sceneparams": (dam.params, dam),
        "dam8k_refparams": (ref_p, dam),
        "ddam32k_sceneparams": (ddam.params, ddam),
        "ddam32k_refparams": (ref_p, ddam),
    }


def run_reference(ref, p, sc, steps=STEPS):
    pos, vel = sc.pos[:, :3].astype(np.float32), sc.vel[:, :3].astype(np.float32)
    iid = np.arange(sc.n, dtype=np.uint32)
    out = np.zeros((steps, 3))
    for k in range(steps):
        r = ref.step(p, sc.ulim, sc.llim, pos, vel, iid)
        out[k] = constraint_stats(r["rho"], float(p.pho0))
        pos, vel, iid = r["npos"], r["nvel"], r["iid"]
    return out


def main():
    import __graft_entry__
    from oracle.ref_harness import ref

    pbf = __graft_entry__.load()
    out_dir = Path(sys.argv[1] if len(sys.argv) > 1 else Path(__file__).resolve().parent)
    out_dir.mkdir(parents=True, exist_ok=True)
    names = sys.argv[2:] or list(cases(pbf))
    for name in names:
        runs = []
        seeds = CASE_SEEDS[name]
        for seed in seeds:
            p, sc = cases(pbf, seed)[name]
            runs.append(run_reference(ref, p, sc))
        runs = np.stack(runs)  # (seeds, steps, [mean C+, max C+, non-finite rho])
        out = out_dir / f"stats_{name}.npz"
        np.savez_compressed(out, stats=runs, seeds=np.array(seeds), steps=np.array(STEPS))
        for k, seed in enumerate(seeds):
            print(f"{out.name} seed {seed}: time-mean of mean C+ {runs[k, :, 0].mean():.6g}, "
                  f"of max C+ {runs[k, :, 1].mean():.6g}, steps with non-finite rho "
                  f"{int(np.count_nonzero(runs[k, :, 2]))}")


if __name__ == "__main__":
    main()
