#!/usr/bin/env python
"""Benchmark of the PBF step: particle-updates/s on the 1M-particle large sweep.

Workload: 1,048,576 particles (128 x 64 x 128 lattice, spacing 0.05, seeded
+-0.005 jitter) in a 12.8 x 6.4 x 6.4 box whose x-max wall moves as
x_w(t) = 12.8 - 1.6 (1 - cos(2 pi t / 4 s)); h = 0.1, 4 solver iterations,
dt = 1/120 s (one 1/60 s frame = 2 steps).  A step is one Simulator::step
over all particles; particle-updates/s = particles x steps / second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:       W untimed steps, then K steps timed with CUDA events on the
            launching stream, L2 flushed (a 512 MB write) before every timed
            step, inputs resident in HBM.  Prints one JSON line (rank 0).
reference:  the reference has no CPU implementation, so its CPU arm is the
            float OpenMP port of its kernels (oracle/), on all host threads,
            same workload, each step a full 1M-particle step; a bounded sample:
            at most 3 warm-up steps, then timed steps for about 20 s, from the
            initial lattice (later steps of this workload pile particles into
            a few cells and cost the CPU minutes per step).
N > 1 runs N independent replicas (one per GPU); the path does not shard.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-updates/s at 1M (4 iters)"
UNIT = "particle-updates/s"
L2_FLUSH_BYTES = 512 << 20


def load_pkg():
    import __graft_entry__

    return __graft_entry__.load()


def measured_peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(n: int, cells: int) -> dict:
    """Algorithmic HBM bytes per launch of the two solver passes: each array a
    pass logically uses is read or written once; c = cells per particle.
    lambda: R x* 16, W lambda 4, cell table 8c;  delta_p: R x* 16, R lambda 4,
    W x 16, cell table 8c."""
    c = cells / max(n, 1)
    return {"lambda": n * (20 + 8 * c), "delta_p": n * (36 + 8 * c)}


def fp32_roofline(n: int, steps: int, total_ms: float, sms, sm_mhz, niter: int = 4) -> dict:
    """The pair work of the step against the FP32 pipes: ~27 true neighbours per
    particle, ~25 flops per lambda pair, ~35 per delta_p pair, ~15 per XSPH
    pair, so 27 (60 niter + 15) algorithmic flops per particle-step (candidates
    outside h not counted).  Peak: SMs x 128 FP32 lanes x 2 (FMA) x the SM
    clock (nominal; none is measured), or None without an SM count and clock."""
    flops = 27 * (60 * niter + 15) * n
    achieved = flops * steps / (total_ms / 1e3) / 1e12
    peak = sms * 128 * 2 * sm_mhz * 1e6 / 1e12 if sms and sm_mhz else None
    return {"bound": "fp32", "algorithmic_flops_per_step": flops, "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
            "peak_kind": "nominal: SMs x 128 lanes x 2 x max SM clock"}


TRAFFIC_PROFILE = ROOT / "profiles" / "neighbour_passes_step16_large_sweep_1m.md"


def ncu_traffic(kernel: str, path: Path = TRAFFIC_PROFILE):
    """DRAM bytes per launch of ``kernel``'s pass (sparse + dense kernel, read +
    write) on the timed regime of this workload, from the committed ncu
    summary (line: 'traffic_bytes_per_launch <kernel>: <bytes>'), or None."""
    if not path.exists():
        return None
    m = re.search(rf"traffic_bytes_per_launch {kernel}: ([0-9.eE+]+)", path.read_text())
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.proc = None
        self.lines = []
        exe = shutil.which("nvidia-smi")
        if exe:
            self.proc = subprocess.Popen([exe, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        return self.summarize(out)

    @staticmethod
    def summarize(out: str):
        """The samples (nvidia-smi CSV rows of FIELDS, no header, no units) as
        the JSON line's clocks: median SM MHz, max SM MHz, the throttle reasons
        seen Active at least once."""
        rows = [r.split(",") for r in out.strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def whole_job_rate(units_per_rank: float, local_ms: float, dist=None, device: str = "cuda"):
    """Replicas (the path does not shard): every rank processed units_per_rank
    units in local_ms.  The job took the slowest rank's time (max over ranks)
    and processed every rank's units: returns (units / s, max ms).  dist is
    torch.distributed with a process group, or None for one process."""
    world, total_ms = 1, float(local_ms)
    if dist is not None:
        import torch

        tt = torch.tensor([total_ms], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
        world = dist.get_world_size()
    return world * units_per_rank / (total_ms / 1e3), total_ms


def make_scene(pkg, name: str, params: str):
    """The workload's scene (pure Python: loads no CUDA code)."""
    scene = getattr(pkg.scenes, name)(seed=0)
    if params == "reference":
        p = pkg.scenes.reference_params()
        p.up[0], p.up[1], p.up[2] = 0.0, 1.0, 0.0
        p.dt = scene.params.dt
        scene.params = p
    return scene


def cpu_port_rate(oracle, scene, pos, vel, iid, t0: float, budget_s: float, max_steps: int):
    """Run the float OpenMP port from (pos, vel, iid) at time t0 for up to
    max_steps steps or budget_s seconds; returns (updates/s, steps, seconds)."""
    p = scene.params
    steps, spent = 0, 0.0
    t = t0
    while steps < max_steps and (spent < budget_s or steps == 0):
        ulim, llim = scene.limits_at(t)
        a = time.perf_counter()
        r = oracle.step(p, ulim, llim, pos, vel, iid, prec="f32")
        spent += time.perf_counter() - a
        pos, vel, iid = r["npos"], r["nvel"], r["iid"]
        t += p.dt
        steps += 1
    return scene.n * steps / spent, steps, spent


def run_reference(args):
    """The reference arm: the float OpenMP port of the reference's kernels
    (oracle/; the reference has no CPU path of its own) on all host threads.
    It loads none of this repository's CUDA code: the scene is generated in
    Python and the port is the oracle library.  Same workload and parameters
    as the GPU arm; the same W warm-up steps from the lattice (time-bounded),
    then as many of the K timed steps as fit in --cpu-budget seconds."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    pkg = load_pkg()
    from oracle import oracle

    scene = make_scene(pkg, args.scene, args.params)
    iid = np.arange(scene.n, dtype=np.uint32)
    pos, vel = scene.pos, scene.vel
    t = 0.0
    w_done = 0
    a = time.perf_counter()
    while w_done < min(args.warmup, args.cpu_warmup_steps) and (time.perf_counter() - a < args.cpu_warmup_budget):
        ulim, llim = scene.limits_at(t)
        r = oracle.step(scene.params, ulim, llim, pos, vel, iid, prec="f32")
        pos, vel, iid = r["npos"], r["nvel"], r["iid"]
        t += scene.params.dt
        w_done += 1
    rate, steps, spent = cpu_port_rate(oracle, scene, pos, vel, iid, t, args.cpu_budget, args.steps)
    cores = oracle.threads()
    first = w_done + 1
    sample = (f"{scene.n} particles per step; steps {first}-{first + steps - 1} of the workload "
              f"({steps} of {args.steps} timed steps, after {w_done} of {args.warmup} warm-up steps; time-bounded)")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": w_done, "ms_per_step": 1e3 * spent / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(scene, args),
        "steps_timed": [first, first + steps - 1],
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(scene, args) -> dict:
    p = scene.params
    if scene.name == "large_sweep_1m":
        what = ("128x64x128 lattice (d=0.05, +-0.005 jitter) in a 12.8x6.4x6.4 box, x-max wall "
                "x_w(t)=12.8-1.6(1-cos(2 pi t/4s))")
    else:
        what = f"{scene.pos.shape[0]} particles in a {'x'.join(f'{u:g}' for u in scene.ulim)} box"
    return {
        "workload": f"{scene.name}: {scene.n} particles, {what}, h=0.1, "
                    f"{p.niter} solver iterations, dt=1/120 s (2 steps per 1/60 s frame)",
        "particles": scene.n, "niter": p.niter, "params": args.params,
        "pho0": round(float(p.pho0), 3), "lambda_eps": float(p.lambda_eps), "k_corr": round(float(p.k_corr), 6),
        "delta_q": round(float(p.delta_q), 6), "n_corr": float(p.n_corr), "c_XSPH": round(float(p.c_XSPH), 6),
        "parallelism": "replicas" if args.gpus > 1 else "single",
        "l2": f"flushed before every timed step ({L2_FLUSH_BYTES >> 20} MB write, outside the timed events)",
    }


def run_ours(args):
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    pkg = load_pkg()
    scene = make_scene(pkg, args.scene, args.params)
    p = scene.params
    n = scene.n
    stream = torch.cuda.current_stream()
    st = pkg.ParticleState(scene.pos, scene.vel)
    ulim0, llim0 = scene.limits_at(0.0)
    sim = pkg.Simulator(p, scene.ulim, scene.llim, n)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    t = 0.0

    def one_step():
        nonlocal t
        ulim, llim = scene.limits_at(t)
        sim.setLim(ulim, llim)
        st.step(sim)
        t += p.dt

    if args.load_state:
        # profiling: the saved state after `warmup` steps, then `steps` untimed steps
        pos_s, vel_s, iid_s = pkg.scenes.load_state(args.load_state)
        st = pkg.ParticleState(pos_s, vel_s, iid_s)
        t = args.warmup * p.dt
        for _ in range(args.steps):
            one_step()
        torch.cuda.synchronize()
        print(json.dumps({"profile_steps": args.steps, "from_step": args.warmup, "state": str(args.load_state)}))
        sim.close()
        return
    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    if args.save_state:
        pkg.scenes.save_state(args.save_state, st.pos, st.vel, st.iid[:n])
        print(json.dumps({"saved_after_steps": args.warmup, "state": str(args.save_state)}))
        sim.close()
        return
    # the dense-kernel choice, tuned once on the state the timed steps start from
    # (pbf_autotune: trial steps on copies of the state, outside the timed region)
    tuning = tune(sim, st, n, args)
    state0 = (st.pos.cpu().numpy(), st.vel.cpu().numpy(), st.iid[:n].cpu().numpy().astype(np.uint32), t)
    sim.profile(True)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    profs = []
    ev = []
    for _ in range(args.steps):
        flush.fill_(1.0)                      # evict L2 (outside the timed events)
        torch.cuda._sleep(2_000_000)          # let the host enqueue the whole step ahead of the GPU
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        one_step()
        e1.record(stream)
        ev.append((e0, e1))
        profs.append(sim.last_profile())      # waits for this step's last phase event
    torch.cuda.synchronize()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    value, total_ms = whole_job_rate(n * args.steps, sum(step_ms), dist)
    if dist is not None:
        dist.barrier()
    sim.profile(False)

    # -- end to end through the public API with host buffers ------------------------
    e2e = measure_e2e(pkg, torch, sim, scene, state0, args.e2e_steps or args.steps, stream, dist)
    sweep = args.scene == "large_sweep"
    alt = measure_reference_params(pkg, torch, args, stream) if args.params == "scene" and sweep else None
    # the workload's own window (60 warm-up frames, 120 timed frames), when
    # the main run timed another one
    window = (time_window(pkg, torch, args, stream, args.params, 120, 240)
              if args.extras and sweep and (args.warmup, args.steps) != (120, 240) and rank == 0 else None)
    ensemble = ensemble_rates(pkg, torch, args, 3, 10) if args.extras and rank == 0 else None
    adjoint = adjoint_times(pkg, torch, args, 2, 60) if args.extras and rank == 0 else None
    ref_gpu = measure_reference_gpu(scene, args) if args.ref_gpu and rank == 0 else None

    if rank != 0:
        sim.close()
        if dist is not None:
            dist.destroy_process_group()
        return

    # -- roofline of the dominant kernel --------------------------------------------
    dims = sim.grid_dims()
    cells = dims[0] * dims[1] * dims[2]
    lam_ms = statistics.mean(pr["lambda_ms"] / pr["iterations"] for pr in profs)
    dp_ms = statistics.mean(pr["delta_p_ms"] / pr["iterations"] for pr in profs)
    alg = algorithmic_bytes(n, cells)
    kernel = "delta_p" if dp_ms >= lam_ms else "lambda"
    launch_ms = dp_ms if kernel == "delta_p" else lam_ms
    peak, peak_kind = measured_peaks()
    achieved = alg[kernel] / (launch_ms / 1e3) / 1e9
    phases = {k: round(statistics.mean(pr[k] for pr in profs), 4)
              for k in ("grid_ms", "reorder_ms", "lambda_ms", "delta_p_ms", "xsph_ms", "total_ms")}
    # the kernels time far above HBM: an FP32 figure explains them (pair work)
    launches = profs[-1]["launches"]

    # -- CPU baseline: the float OpenMP port on a bounded sample of the workload ---------
    # The timed GPU steps (after the warm-up) are far too costly for the CPU once
    # particles have piled up, so the sample is the workload's first steps from
    # the initial lattice, and the GPU is timed on exactly those steps beside it.
    from oracle import oracle

    cpu_line = None
    if args.cpu_steps > 0:
        cpu_steps_max = min(args.cpu_steps, args.steps)
        cpu_rate, cpu_steps, cpu_s = cpu_port_rate(oracle, scene, scene.pos, scene.vel,
                                                   np.arange(n, dtype=np.uint32), 0.0, args.cpu_budget,
                                                   cpu_steps_max)
        gpu_same = gpu_rate_first_steps(pkg, torch, scene, cpu_steps, stream)
        cpu_line = {"value": cpu_rate, "unit": UNIT, "cores": oracle.threads(), "kind": "port",
                    "sample": f"the workload's first {cpu_steps} steps from the initial lattice, {n} "
                              f"particles ({cpu_s:.1f} s of CPU time); the GPU on the same steps: "
                              f"{gpu_same:.4g} {UNIT}",
                    "gpu_same_sample": gpu_same}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {**workload_config(scene, args), "tuning": tuning},
        "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": alg[kernel], "launch_ms": launch_ms,
                     "traffic": ncu_traffic(kernel)},
        "fp32": fp32_roofline(n, args.steps, total_ms, torch.cuda.get_device_properties(local).multi_processor_count,
                              (clk or {}).get("sm_max_mhz"), p.niter),
        "phases_ms": phases,
        "cpu_baseline": cpu_line,
        "e2e": e2e,
        "gpu_launches": launches * args.steps,
        "clocks": clk,
        "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)},
        "reference_params": alt,
        "reference_gpu": ref_gpu,
        "window_120_240": window,
        "ensemble": ensemble,
        "adjoint": adjoint,
    }
    print(json.dumps(line), flush=True)
    sim.close()
    if dist is not None:
        dist.destroy_process_group()


def tune(sim, st, n, args):
    """pbf_autotune on the current state (unless --no-tune, --dense-window or
    --order); returns the choice."""
    if args.dense_window or args.order is not None:
        order = -1 if args.order is None else args.order
        sim.set_tuning(args.dense_window, 0 if args.dense_window else -1, order)
        return {**sim.tuning(), "set": "--dense-window / --order"}
    if not args.tune:
        return None
    t = sim.autotune(st.pos, st.vel, st.iid, n, steps=6)
    keys = ("dense_window", "dense_all", "order", "dense_split", "dense_interleave", "queue_sparse", "queue_dense",
            "stage_sparse", "stage_dense")
    return {**{k: int(t[k]) for k in keys}, "trial_ms_per_step": round(float(t["ms_per_step"]), 4),
            "trial_ms_per_step_default": round(float(t["ms_default"]), 4)}


def gpu_rate_first_steps(pkg, torch, scene, steps, stream):
    """GPU particle-updates/s over the workload's first `steps` steps from the
    initial lattice, L2 flushed before each, CUDA events on the stream."""
    p = scene.params
    st = pkg.ParticleState(scene.pos, scene.vel)
    sim = pkg.Simulator(p, scene.ulim, scene.llim, scene.n)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    total, t = 0.0, 0.0
    for _ in range(steps):
        ulim, llim = scene.limits_at(t)
        flush.fill_(1.0)
        torch.cuda._sleep(2_000_000)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.setLim(ulim, llim)
        st.step(sim)
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1)
        t += p.dt
    sim.close()
    return scene.n * steps / (total / 1e3)


def time_window(pkg, torch, args, stream, params: str, warmup: int, steps: int) -> dict:
    """The workload with the given parameter set from the lattice: `warmup`
    untimed steps, the choice of pbf_autotune (as the main run makes it), then
    `steps` steps timed with CUDA events, L2 flushed before every step."""
    scene = make_scene(pkg, args.scene, params)
    p = scene.params
    st = pkg.ParticleState(scene.pos, scene.vel)
    sim = pkg.Simulator(p, scene.ulim, scene.llim, scene.n)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    t = 0.0
    total = 0.0
    tuning = None
    for k in range(warmup + steps):
        ulim, llim = scene.limits_at(t)
        if k == warmup:
            torch.cuda.synchronize()
            tuning = tune(sim, st, scene.n, args)
        if k >= warmup:
            flush.fill_(1.0)
            torch.cuda._sleep(2_000_000)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        sim.setLim(ulim, llim)
        st.step(sim)
        if k >= warmup:
            e1.record(stream)
            e1.synchronize()
            total += e0.elapsed_time(e1)
        t += p.dt
    sim.close()
    return {"value": scene.n * steps / (total / 1e3), "unit": UNIT, "ms_per_step": total / steps,
            "warmup": warmup, "steps": steps, "tuning": tuning,
            "params": {"pho0": float(p.pho0), "lambda_eps": float(p.lambda_eps), "k_corr": round(float(p.k_corr), 6),
                       "delta_q": round(float(p.delta_q), 6), "c_XSPH": float(p.c_XSPH)}}


def measure_reference_params(pkg, torch, args, stream):
    """The same workload (particles, box, moving wall, iterations, dt) with the
    reference's own solver parameters (fluids/FluidSystem.cpp:15-25), under
    which the fluid stays a fluid: warm-up and timed steps as the main run."""
    return time_window(pkg, torch, args, stream, "reference", args.warmup, args.steps)


def measure_reference_gpu(scene, args):
    """The reference's own CUDA kernels rebuilt for sm_103a (oracle/ref_harness:
    its unmodified fluids/Simulator.cu, driven with Simulator::step's host
    sequencing, fluids/Simulator.cpp:10-99) on the same workload and steps as
    the main run: W warm-up steps from the lattice, then the timed steps, the
    moving wall stepped the same way; with the reference's per-phase
    cudaDeviceSynchronize and without it.  The timed steps are bounded: a
    3-step probe first, then as many of the K steps as fit in
    --ref-gpu-budget seconds."""
    try:
        from oracle.ref_harness import ref
    except Exception as e:  # noqa: BLE001 - reported, not raised
        return {"unavailable": f"reference harness import failed: {e}"}
    if not ref.available():
        return {"unavailable": "reference kernels not built (the cubin is built where the reference sources are)"}
    p = scene.params
    n = scene.n

    def walls(k_steps):
        return np.array([scene.limits_at(k * p.dt)[0][0] for k in range(args.warmup + k_steps)], np.float32)

    out = {"kind": "the reference's kernels rebuilt for sm_103a", "warmup": args.warmup}
    try:
        probe = min(3, args.steps)
        a = time.perf_counter()
        ms = ref.bench(p, scene.ulim, scene.llim, scene.pos, scene.vel, args.warmup, probe, walls(probe), sync=True)
        per_call_s = time.perf_counter() - a
        per_step_s = per_call_s / (args.warmup + probe)
        k = max(probe, min(args.steps, int(args.ref_gpu_budget / max(per_step_s, 1e-6)) - args.warmup))
        if k > probe:
            ms = ref.bench(p, scene.ulim, scene.llim, scene.pos, scene.vel, args.warmup, k, walls(k), sync=True)
        out["steps"] = k
        out["phase_syncs"] = {"value": n * k / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / k}
        ms2 = ref.bench(p, scene.ulim, scene.llim, scene.pos, scene.vel, args.warmup, k, walls(k), sync=False)
        out["no_syncs"] = {"value": n * k / (ms2 / 1e3), "unit": UNIT, "ms_per_step": ms2 / k}
    except Exception as e:  # noqa: BLE001
        out["unavailable"] = f"reference harness failed: {e}"
    return out


def measure_e2e(pkg, torch, sim, scene, state0, steps, stream, dist=None):
    """Same metric through Simulator.step with HOST buffers: every step copies
    pos/vel/iid host->device from pinned memory, steps, and reads npos/nvel/iid
    back; the copies are inside the timed region.  With several ranks the
    whole job's rate (every replica's steps over the slowest rank's time)."""
    pos0, vel0, iid0, t = state0
    n = scene.n
    p = scene.params
    h_pos = torch.from_numpy(pos0.copy()).pin_memory()
    h_vel = torch.from_numpy(vel0.copy()).pin_memory()
    h_iid = torch.from_numpy(iid0.astype(np.int32)).pin_memory()
    d = {k: torch.empty(n, 4, device="cuda") for k in ("pos", "vel", "npos", "nvel")}
    d_iid = torch.empty(n, dtype=torch.int32, device="cuda")
    h2d = h_pos.numel() * 4 + h_vel.numel() * 4 + h_iid.numel() * 4
    d2h = h2d
    for k in range(2):  # warm-up
        d["pos"].copy_(h_pos, non_blocking=True)
        d["vel"].copy_(h_vel, non_blocking=True)
        d_iid.copy_(h_iid, non_blocking=True)
        sim.step(d["pos"], d["npos"], d["vel"], d["nvel"], d_iid, n)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        ulim, llim = scene.limits_at(t)
        sim.setLim(ulim, llim)
        d["pos"].copy_(h_pos, non_blocking=True)
        d["vel"].copy_(h_vel, non_blocking=True)
        d_iid.copy_(h_iid, non_blocking=True)
        sim.step(d["pos"], d["npos"], d["vel"], d["nvel"], d_iid, n)
        h_pos.copy_(d["npos"], non_blocking=True)
        h_vel.copy_(d["nvel"], non_blocking=True)
        h_iid.copy_(d_iid, non_blocking=True)
        t += p.dt
    e1.record(stream)
    torch.cuda.synchronize()
    rate, ms = whole_job_rate(n * steps, e0.elapsed_time(e1), dist)
    return {"value": rate, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": steps, "ms_per_step": ms / steps}


def ensemble_rates(pkg, torch, args, warmup: int, steps: int) -> dict:
    """Scene-steps/s of the 256-scene ensemble (dam-break scenes, a x b x c
    lattices with a, b, c uniform in [12, 40], each in its own (2a d, 2b d,
    2c d) box), batched (pbf_batch_step: one launch per pass for all scenes,
    choices from pbf_batch_autotune after the warm-up) and one scene per
    launch (a solver per scene, stepped in turn); same steps, same stream,
    CUDA events around the timed steps."""
    scenes = pkg.scenes.ensemble(seed=0, count=args.scenes)
    p = scenes[0].params
    if args.params == "reference":
        q = pkg.scenes.reference_params()
        q.up[0], q.up[1], q.up[2] = 0.0, 1.0, 0.0
        q.dt = p.dt
        p = q
    stream = torch.cuda.current_stream()
    counts = [sc.n for sc in scenes]
    pos = np.concatenate([sc.pos for sc in scenes])
    st = pkg.ParticleState(pos, np.zeros_like(pos))
    ens = pkg.Ensemble(p, [sc.ulim for sc in scenes], [sc.llim for sc in scenes], counts)
    for _ in range(warmup):
        st.step(ens)
    tuning = ens.autotune(st.pos, st.vel, st.iid, steps=2)
    torch.cuda.synchronize()
    torch.cuda._sleep(5_000_000)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        st.step(ens)
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1)
    ens.close()
    sts = [pkg.ParticleState(sc.pos, sc.vel) for sc in scenes]
    sims = [pkg.Simulator(p, sc.ulim, sc.llim, sc.n) for sc in scenes]
    for _ in range(warmup):
        for s_, m in zip(sts, sims):
            s_.step(m)
    torch.cuda.synchronize()
    torch.cuda._sleep(5_000_000)
    e0.record(stream)
    for _ in range(steps):
        for s_, m in zip(sts, sims):
            s_.step(m)
    e1.record(stream)
    torch.cuda.synchronize()
    single_ms = e0.elapsed_time(e1)
    for m in sims:
        m.close()
    k = len(scenes) * steps
    return {"value": k / (batched_ms / 1e3), "unit": "scene-steps/s", "steps": steps, "warmup": warmup,
            "ms_per_step": batched_ms / steps, "scenes": len(scenes), "particles": sum(counts),
            "params": args.params, "autotune": tuning,
            "one_scene_per_launch": {"value": k / (single_ms / 1e3), "ms_per_step": single_ms / steps},
            "batched_over_per_scene": single_ms / batched_ms}


def run_ensemble(args):
    """Ensemble scenes/s (see ensemble_rates): one scene-step = one scene
    advanced one step."""
    import torch

    pkg = load_pkg()
    r = ensemble_rates(pkg, torch, args, args.warmup, args.steps)
    line = {
        "metric": "ensemble scenes/s", "value": r["value"], "unit": "scene-steps/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{r['scenes']} dam-break scenes, a,b,c ~ U{{12..40}} (seed 0), "
                               f"{r['particles']} particles, 4 iterations, dt=1/120 s",
                   "params": args.params, "particles": r["particles"]},
        "autotune": r["autotune"],
        "one_scene_per_launch": r["one_scene_per_launch"],
        "batched_over_per_scene": r["batched_over_per_scene"],
    }
    print(json.dumps(line), flush=True)


def adjoint_times(pkg, torch, args, evals: int, frames: int) -> dict:
    """fwd+bwd ms/frame of the inverse problem: 15,625 particles (25^3
    lattice) in a 2 x 1 x 1 box, `frames` frames of 2 steps, the loss on a
    32 x 16 x 16 density grid, checkpoints every 10 frames.  One evaluation =
    the forward rollout + the density grid + the reverse sweep (which re-runs
    each 10-frame segment from its checkpoint with the tape on) + the adjoint
    of the grid; timed with CUDA events around whole evaluations.  The forward
    alone (the same steps through pbf_step, no tape) is timed beside it."""
    scene = pkg.scenes.inverse_scene()
    if args.params == "reference":
        q = pkg.scenes.reference_params()
        q.up[0], q.up[1], q.up[2] = 0.0, 1.0, 0.0
        q.dt = scene.params.dt
        scene.params = q
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    warm = 3

    lane_choice = {}

    def fwd_bwd(keep):
        ip = pkg.inverse.InverseProblem(scene, frames=frames, every=10, keep=keep)
        ip.make_target()
        v0 = torch.zeros((ip.n, 3), device="cuda")
        for _ in range(warm):
            ip.loss_and_grad(v0, 0.0)
        # the reverse pass's lanes per particle, chosen by timing (outside the timed evaluations)
        if not lane_choice:
            lane_choice.update(ip.autotune_backward(v0, 0.0))
        else:
            ip.sim.set_tuning(**{**ip.sim.tuning(), "bwd_lanes": lane_choice["bwd_lanes"]})
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(evals):
            L, gv, ga = ip.loss_and_grad(v0, 0.0)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / evals
        fin = bool(torch.isfinite(gv).all()) and bool(np.isfinite(ga))
        steps, lim = ip.steps, ip.limits(0.0)
        ip.close()
        return ms, fin, steps, lim

    # checkpoints every 10 frames, the last 10-frame segment taped by the forward
    fb_ms, finite, nsteps, limits = fwd_bwd(1)
    # the whole rollout taped by the forward (no segment re-run; 10-frame checkpoints kept)
    fb_all_ms = fwd_bwd(1 << 20)[0]
    sim = pkg.Simulator(scene.params, scene.ulim, scene.llim, scene.n)
    st = pkg.ParticleState(scene.pos, scene.vel)
    for _ in range(warm):
        st.step(sim)
    torch.cuda.synchronize()
    p0 = torch.from_numpy(scene.pos).cuda()
    iid0 = torch.arange(scene.n, dtype=torch.int32, device="cuda")
    e0.record(stream)
    for _ in range(evals):
        st.a_pos[: st.n].copy_(p0)
        st.a_vel.zero_()
        st.iid[: st.n].copy_(iid0)
        st.tictoc = False
        for k in range(nsteps):
            sim.setLim(*limits(k))
            st.step(sim)
    e1.record(stream)
    torch.cuda.synchronize()
    f_ms = e0.elapsed_time(e1) / evals
    sim.close()
    nframes = nsteps // pkg.inverse.STEPS_PER_FRAME
    return {"value": fb_ms / nframes, "unit": "ms/frame", "evals": evals, "warmup": warm, "frames": nframes,
            "particles": scene.n, "params": args.params, "ms_per_step": fb_ms / nsteps,
            "forward_ms_per_frame": f_ms / nframes, "fwd_bwd_over_fwd": fb_ms / f_ms,
            "gradient_finite": finite, "backward_tuning": lane_choice,
            "whole_rollout_taped": {"value": fb_all_ms / nframes, "fwd_bwd_over_fwd": fb_all_ms / f_ms}}


def run_adjoint(args):
    """fwd+bwd ms/frame of the inverse problem (see adjoint_times)."""
    import torch

    pkg = load_pkg()
    r = adjoint_times(pkg, torch, args, args.evals, args.frames)
    line = {
        "metric": "fwd+bwd ms/frame", "value": r["value"], "unit": "ms/frame", "n_gpus": 1,
        "steps": args.evals, "warmup": r["warmup"], "ms_per_step": r["ms_per_step"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"inverse problem: {r['particles']} particles (25^3 lattice, spacing 0.04) in a "
                               f"2x1x1 box, {r['frames']} frames x 2 steps, 4 iterations, density loss on "
                               f"32x16x16, checkpoints every 10 frames",
                   "params": args.params, "particles": r["particles"]},
        "forward_ms_per_frame": r["forward_ms_per_frame"],
        "fwd_bwd_over_fwd": r["fwd_bwd_over_fwd"],
        "gradient_finite": r["gradient_finite"],
        "backward_tuning": r["backward_tuning"],
        "whole_rollout_taped": r["whole_rollout_taped"],
    }
    print(json.dumps(line), flush=True)


def covered_pixels(renderer) -> int:
    """Pixels of the last render with fluid depth (the ones smoothing filters)."""
    return int((renderer.images()["depth"] < 99).sum().item())


def run_ssf(args):
    """frames/s of the screen-space fluid render (include/pbf_ssf.h): the 1M
    particles of the large sweep's lattice at 1600 x 1200 with the reference's
    renderer settings (2 bilateral passes, kernel_r 10, sigma_r 6, sigma_z 0.1,
    Fresnel shading), camera 11.7 units off the lattice.  A step = one render:
    clear, depth + thickness splat, resolve, 2 smoothing passes, normals,
    shading.  e2e: host positions copied in, the colour image copied back."""
    import torch

    pkg = load_pkg()
    from oracle import oracle

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    scene = pkg.scenes.large_sweep(seed=0)
    pos_y = torch.from_numpy(scene.pos).cuda()
    pos = pkg.ssf.z_up(pos_y).contiguous()
    n = pos.shape[0]
    p = pkg.ssf_default_params(1600, 1200)
    pkg.ssf.look_at(p, (3.2, -14.0, 6.0), (3.2, -3.2, 1.6))
    r = pkg.SSFRenderer(p)
    color = torch.zeros((p.height, p.width, 4), device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    warm = max(3, args.warmup)
    for _ in range(warm):
        r.render(pos, color=color)
    r.profile_enable(True)
    r.render(pos, color=color)
    prof = r.profile()
    r.profile_enable(False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = []
    clocks = ClockSampler(torch.cuda.current_device())
    for _ in range(args.steps):
        flush.fill_(1.0)  # L2 flushed before every timed render, outside the events
        e0.record(stream)
        r.render(pos, color=color)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    ms = statistics.mean(times)
    # e2e: pinned host positions in, the colour image out, every frame
    host_pos = pos.cpu().pin_memory()
    host_img = torch.empty(color.shape, dtype=torch.float32).pin_memory()
    dev_pos = torch.empty_like(pos)
    e2e_frames = args.e2e_steps or args.steps
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(e2e_frames):
        dev_pos.copy_(host_pos, non_blocking=True)
        r.render(dev_pos, color=color)
        host_img.copy_(color, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e2e_frames
    # CPU baseline: the float oracle renders one frame of the same workload
    cpu_line = None
    if args.cpu_steps > 0:
        host = pos.cpu().numpy()
        a = time.perf_counter()
        o = oracle.ssf_render(p, host, prec="f32")
        cpu_s = time.perf_counter() - a
        cpu_line = {"value": 1.0 / cpu_s, "unit": "frames/s", "cores": oracle.threads(), "kind": "port",
                    "sample": f"one frame of the same workload ({n} particles, 1600x1200, {o['fragments']} "
                              f"fragments; splat on one thread, smoothing/normals/shading on all), "
                              f"{cpu_s:.1f} s"}
    phases = {k: round(prof[k], 4) for k in ("splat_ms", "smooth_ms", "normal_ms", "shade_ms", "total_ms")}
    dominant = max(("splat_ms", "smooth_ms", "normal_ms", "shade_ms"), key=lambda k: prof[k])
    npix = p.width * p.height
    # algorithmic HBM bytes: the splat reads the positions and leaves two images
    # (4 B depth key + 8 B fixed-point thickness per pixel; its per-fragment
    # atomics resolve in L2, where the 23 MB images stay); clear and resolve
    # write / read those images and write depth_a, depth_b, thickness; a
    # smoothing pass reads and writes one float per pixel
    alg = {"splat_ms": 16 * n + 12 * npix + 12 * npix + 24 * npix, "smooth_ms": 8 * npix * p.smooth_niter,
           "normal_ms": 20 * npix, "shade_ms": 40 * npix}
    peak, peak_kind = measured_peaks()
    achieved = alg[dominant] / (prof[dominant] / 1e3) / 1e9
    line = {
        "metric": "SSF frames/s at 1M particles, 1600x1200", "value": 1e3 / ms, "unit": "frames/s",
        "n_gpus": 1, "steps": args.steps, "warmup": warm, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"SSF render: {n} particles (128x64x128 lattice, z-up) at 1600x1200, "
                               f"2 bilateral passes (kernel_r 10), Fresnel shading, camera (3.2,-14,6)->(3.2,-3.2,1.6)",
                   "particles": n, "l2": "flushed before every timed render (512 MB write, outside the events)"},
        "phases_ms": phases, "fragments": prof["fragments"], "gpu_launches": prof["launches"] * args.steps,
        "fragments_per_s": prof["fragments"] / (prof["splat_ms"] / 1e3),
        "bilateral_taps_per_s": (2 * p.kernel_r + 1) ** 2 * covered_pixels(r) * p.smooth_niter
                                / (prof["smooth_ms"] / 1e3),
        "roofline": {"bound": "hbm", "kernel": dominant.replace("_ms", ""), "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": alg[dominant], "traffic": None},
        "e2e": {"value": 1e3 / e2e_ms, "unit": "frames/s", "h2d_bytes_per_step": int(host_pos.numel() * 4),
                "d2h_bytes_per_step": int(host_img.numel() * 4), "steps": e2e_frames, "ms_per_step": e2e_ms},
        "cpu_baseline": cpu_line,
        "clocks": clk,
    }
    r.close()
    print(json.dumps(line), flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=240, help="timed steps (default: 120 frames x 2 steps)")
    ap.add_argument("--warmup", type=int, default=120, help="untimed steps (default: 60 frames x 2 steps)")
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--scene", default="large_sweep", choices=("large_sweep", "double_dam", "dam_break", "clustered"))
    ap.add_argument("--workload", choices=("step", "ensemble", "adjoint", "ssf"), default="step",
                    help="step: particle-updates/s of one scene; ensemble: scene-steps/s of 256 scenes; "
                         "adjoint: fwd+bwd ms/frame of the inverse problem; "
                         "ssf: frames/s of the screen-space fluid render of 1M particles at 1600x1200")
    ap.add_argument("--frames", type=int, default=60, help="frames of the inverse problem (adjoint workload)")
    ap.add_argument("--evals", type=int, default=5, help="timed gradient evaluations (adjoint workload)")
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--params", choices=("scene", "reference"), default="scene",
                    help="scene: the dam-break parameter set; reference: the reference's own defaults")
    ap.add_argument("--no-tune", dest="tune", action="store_false",
                    help="keep the default dense-kernel choice instead of pbf_autotune after the warm-up")
    ap.add_argument("--dense-window", type=int, default=0,
                    help="set this dense-kernel window after the warm-up instead of tuning (no trial steps)")
    ap.add_argument("--order", type=int, choices=(0, 1), default=None,
                    help="set the particle order after the warm-up instead of tuning (1: current cell, 0: grid)")
    ap.add_argument("--e2e-steps", type=int, default=None,
                    help="steps of the end-to-end measurement (default: the timed steps, from the same state)")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU-port timing")
    ap.add_argument("--cpu-steps", type=int, default=20,
                    help="most steps the CPU baseline times (0: no CPU baseline, for profiling runs)")
    ap.add_argument("--cpu-warmup-steps", type=int, default=8, help="most warm-up steps of the reference arm")
    ap.add_argument("--save-state", default=None,
                    help="profiling: after the warm-up steps, save the particle state to this file and exit")
    ap.add_argument("--load-state", default=None,
                    help="profiling: start from this state (saved after --warmup steps), run --steps untimed "
                         "steps and exit (a short command for ncu)")
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="skip the sub-measurements (120/240 window, ensemble, adjoint) of the step workload")
    ap.add_argument("--no-ref-gpu", dest="ref_gpu", action="store_false",
                    help="skip timing the reference's own kernels (rebuilt for sm_103a) beside the run")
    ap.add_argument("--ref-gpu-budget", type=float, default=40.0,
                    help="seconds of reference-kernel steps per variant (bounds its timed steps)")
    ap.add_argument("--cpu-warmup-budget", type=float, default=60.0)
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.workload == "ensemble":
        run_ensemble(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "ssf":
        run_ssf(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
