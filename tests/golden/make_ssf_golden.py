"""Golden outputs of the reference's own SSF shaders (fluids/shader/SSF*.glsl),
run on the CPU by oracle/ref_harness (ssf_ref.cpp with the shaders compiled as
C++), for tests/test_ssf_ref.py.

Needs the reference sources, so it runs where they are:

    python tests/golden/make_ssf_golden.py

Writes tests/golden/ssf_ref_<case>.npz: the particles, the renderer parameters
(pbf_ssf_params fields), the sky cube map when used, and each stage's output
fed with the previous stage's reference output: splat depth and thickness,
smoothed depth, normal_D, and the colour of every shading option.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def cases(pbf):
    """(name, params, positions (n, 4) float32, sky or None)."""
    out = []
    rng = np.random.default_rng(11)
    # a jittered block in front of the reference's default camera
    pos = np.zeros((900, 4), np.float32)
    g = np.stack(np.meshgrid(np.arange(10), np.arange(9), np.arange(10), indexing="ij"), -1).reshape(-1, 3)
    pos[:, :3] = (g * 0.06 + np.array([-0.3, -0.3, 1.2]) + rng.uniform(-0.01, 0.01, (900, 3))).astype(np.float32)
    p = pbf.ssf_default_params(96, 72)
    pbf.ssf.look_at(p, (0.6, -1.8, 1.9), (0.0, 0.0, 1.45))
    out.append(("block", p, pos, None))
    # scattered droplets over the floor, seen from above, a sky cube map, one bilateral pass
    pos2 = np.zeros((400, 4), np.float32)
    pos2[:, :3] = rng.uniform([-1.0, -1.0, 0.2], [1.0, 1.0, 1.0], (400, 3)).astype(np.float32)
    q = pbf.ssf_default_params(80, 64)
    pbf.ssf.look_at(q, (0.5, -2.5, 2.5), (0.0, 0.0, 0.4))
    q.smooth_niter, q.kernel_r, q.keep_edge = 1, 6, 0
    sky = rng.uniform(0.0, 1.0, (6, 4, 4, 3)).astype(np.float32)
    out.append(("droplets", q, pos2, sky))
    # gaussian smoothing, three passes
    r = pbf.ssf_default_params(64, 48)
    pbf.ssf.look_at(r, (0.6, -1.8, 1.9), (0.0, 0.0, 1.45))
    r.blur_option, r.smooth_niter, r.kernel_r = 1, 3, 4
    out.append(("gaussian", r, pos, None))
    return out


def main():
    import __graft_entry__

    pbf = __graft_entry__.load()
    from oracle import oracle

    if not oracle.ssf_ref_available():
        raise SystemExit("the reference's shader sources are not here")
    for name, p, pos, sky in cases(pbf):
        depth, thick, frags = oracle.ssf_ref_splat(p, pos)
        smooth = oracle.ssf_ref_smooth(p, depth)
        nd = oracle.ssf_ref_normals(p, smooth)
        colors = []
        for opt in range(8):
            q = p.copy()
            q.shading_option = opt
            fill = np.full((p.height, p.width, 4), -1.0, np.float32)
            colors.append(oracle.ssf_ref_shade(q, smooth, nd, thick, fill, sky))
        fields = {f: np.array(getattr(p, f)[:] if hasattr(getattr(p, f), "_length_") else getattr(p, f))
                  for f, _ in p._fields_}
        np.savez_compressed(ROOT / "tests" / "golden" / f"ssf_ref_{name}.npz", pos=pos,
                            sky=sky if sky is not None else np.zeros((0,), np.float32), depth=depth, thick=thick,
                            fragments=np.array(frags), smooth=smooth, normal_D=nd, colors=np.stack(colors),
                            **{f"param_{k}": v for k, v in fields.items()})
        print(name, "fragments", frags, "covered", int((depth < 99).sum()))


if __name__ == "__main__":
    main()
