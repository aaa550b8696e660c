#!/usr/bin/env python3
"""Benchmark of the PICurv particle hot path on one GB300 (and N replicas under torchrun).

One step = ResetAllParticleStatuses -> UpdateAllParticlePositions ->
LocateAllParticlesInGrid -> remove LOST / out-of-bounds -> InterpolateAllFieldsToSwarm
-> ScatterAllParticleFieldsToEulerFields -> face deposit, with the particles re-sorted
by cell (simulation.c:240-311).  Metric: particle-steps/s = sum over timed steps of
the live particles at step start / wall time of the timed steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl fdf|reference]

--impl reference times the reference algorithm on the host cores: the reference
itself cannot be built (it needs PETSc + MPI), so this is the CPU restatement in
oracle/ (OpenMP over all cores), on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300: learned+FP32 vs plain FP64 walk, exact cells"
UNIT = "particle-steps/s"

# Algorithmic bytes ("Roofline accounting").
ROW_BYTES = 296          # 36 plane doubles + threshold read per walk evaluation
LOCATE_PER_PARTICLE = 53 + 61
GATHER_PER_PARTICLE = 8 + 64 + 93


def workload(name: str):
    from fdf_gb300 import workloads as W
    if name == "sinusoidal":           # the curvilinear plain-FP64 configuration
        return W.config_sinusoidal(64, 64, 1024, n=1_000_000, cfl=0.5, steps=50)
    if name == "uniform":
        return W.config1()
    if name == "sinusoidal96":
        return W.config_sinusoidal(96, 96, 1536, n=16_000_000, cfl=1.0, steps=100)
    if name == "bent_pipe":
        return W.config_bent_pipe()
    if name == "curved_pipe":
        return W.config_curved_pipe()
    if name == "sinusoidal_medium":
        return W.config_sinusoidal(64, 64, 256, n=250_000, cfl=0.5, steps=10)
    if name.startswith("sinusoidal_small"):
        return W.config_sinusoidal(32, 32, 256, n=200_000, cfl=0.5, steps=10)
    raise SystemExit(f"unknown workload {name}")


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist
    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return rank, ws, local, dist


def reduce_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.lines = index, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        rows = [[c.strip() for c in l.split(",")] for l in out.strip().splitlines() if l.count(",") >= 8]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def pinned_like(a: np.ndarray) -> np.ndarray:
    try:
        import torch
        if torch.cuda.is_available():
            t = torch.empty(a.size * a.itemsize, dtype=torch.uint8, pin_memory=True)
            out = t.numpy().view(a.dtype).reshape(a.shape)
            out[...] = a
            out._keep = t  # noqa: keep the pinned tensor alive with the view
            return out
    except Exception:
        pass
    return a.copy()


# ----------------------------------------------------------------------------- CPU (oracle) timing

def time_oracle(wl, budget_s: float, max_steps: int, nthreads: int):
    """Times reference steps of the CPU restatement on the workload (after its initial
    location).  If a full step would exceed the budget, a random particle sample is
    stepped and the measured per-particle time is combined with the grid-sized work
    (center->corner + scatter) measured on the full grid."""
    from oracle import oracle as O
    g = O.Grid(wl.coor)
    n = wl.n
    t_est = 1.5e-6 * n / max(nthreads, 1) + 0.05
    sample = n
    if t_est * 2 > budget_s:
        sample = max(10_000, int(n * (budget_s / 2) / t_est / 2))
        sample = min(sample, n)
    idx = np.arange(n) if sample == n else np.sort(np.random.default_rng(0).choice(n, sample, replace=False))
    s = O.Swarm.create(wl.pos[idx], cell=wl.cell0[idx], pid=idx)
    sim = O.Simulation(g, wl.ucat_node_sized(), s, wl.dt, nthreads=nthreads)
    sim.initial_setup()
    sim.step()   # warm-up step
    steps, psteps, t0 = 0, 0, time.perf_counter()
    while steps < max_steps:
        n0 = s.n
        sim.step()
        steps += 1
        psteps += n0
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    if sample == n:
        return psteps / el, steps, el, f"full workload, {steps} steps"
    # grid-sized part of a step on the full grid (independent of the particle count)
    empty = O.Swarm.create(np.zeros((0, 3)))
    sim_g = O.Simulation(g, wl.ucat_node_sized(), empty, wl.dt, nthreads=nthreads)
    tg0 = time.perf_counter()
    sim_g.step()
    t_grid = time.perf_counter() - tg0
    per_particle = max(el / steps - t_grid, 1e-12) / (psteps / steps)
    t_full = t_grid + per_particle * n
    return n / t_full, steps, el, (f"{sample} of {n} particles (random, seed 0) x {steps} steps on the full grid; "
                                   f"per-particle time scaled to {n} plus the grid-sized work ({t_grid:.3f} s/step)")


def run_reference(args, rank):
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    wl = workload(args.workload)
    nthreads = os.cpu_count() or 1
    vals = []
    samples = ""
    for _ in range(args.warmup):
        time_oracle(wl, budget_s=2.0, max_steps=1, nthreads=nthreads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, st, el, samples = time_oracle(wl, budget_s=float(args.cpu_seconds) / max(args.steps, 1),
                                         max_steps=1000, nthreads=nthreads)
        vals.append(v)
    total = time.perf_counter() - t0
    value = float(np.median(vals))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl.name, "form": "reference algorithm (CPU restatement)", "cores": nthreads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": samples},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU

def run_gpu(args, rank, ws, local, dist):
    from fdf_gb300.context import PicContext, SwarmArrays
    import torch

    wl = workload(args.workload)
    IM, JM, KM = wl.dims
    Nc, Nn = IM * JM * KM, (IM + 1) * (JM + 1) * (KM + 1)
    Nf = (IM + 1) * JM * KM + IM * (JM + 1) * KM + IM * JM * (KM + 1)
    ctx = PicContext(local)
    ctx.load_workload(wl)
    ctx.initial_setup()
    ctx.steps(args.warmup)
    ctx.synchronize()
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ps0, e0, nd0 = ctx.counters()
    l0 = ctx.launches
    ctx.set_profiling(True)
    clocks = ClockSampler(local)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev0.record(stream)
    ctx.steps(args.steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    ms_max = reduce_max(dist, ms)
    ps1, e1, nd1 = ctx.counters()
    launches = ctx.launches - l0
    stages = ctx.stage_times()
    ctx.set_profiling(False)
    psteps = ps1 - ps0
    evals = e1 - e0
    n_avg = psteps / max(args.steps, 1)
    total_psteps = psteps * ws            # replicas: every rank advanced its own copy
    value = total_psteps / (ms_max / 1000.0)

    # roofline of the dominant stage (algorithmic bytes / its average event-timed duration)
    hbm, peak_kind = peaks()
    alg = {
        "center_to_corner": 48 * (nd1 - nd0) / max(args.steps, 1),   # 8 cells' ucat via cache + node write
        "advect_locate": LOCATE_PER_PARTICLE * n_avg + ROW_BYTES * evals / max(args.steps, 1),
        # keys + slot writes + PID reads of the per-cell ordering + the histogram scan (read + write)
        "sort_by_cell": 24 * n_avg + 12 * (Nc + 2),
        "wait_corner": 0,
        "gather_interpolate": GATHER_PER_PARTICLE * n_avg + 24 * Nn,
        "deposit": 4 * (Nc + 1) + 32 * n_avg + 16 * Nn + 8 * Nf,
    }
    per = {k: (v[0] / max(v[1], 1)) for k, v in stages.items()}
    dom = max((k for k in per if alg.get(k)), key=per.get)
    achieved = alg[dom] / (per[dom] / 1000.0) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": alg[dom], "traffic": None,
                "stage_ms_per_step": {k: round(v, 4) for k, v in per.items()},
                "stage_gbs": {k: round(alg[k] / (per[k] / 1000.0) / 1e9, 1) for k in per if per[k] > 0 and alg.get(k)}}

    # end to end through the C ABI with host (pinned) buffers
    e2e = None
    if not args.no_e2e:
        s_host = ctx.get_swarm()
        n0 = s_host.n
        bufs = SwarmArrays(*[pinned_like(a) for a in (s_host.position, s_host.velocity, s_host.weight, s_host.P,
                                                       s_host.cell, s_host.pid, s_host.status)])
        count = pinned_like(np.zeros((KM + 1, JM + 1, IM + 1)))
        avg = pinned_like(np.zeros((KM + 1, JM + 1, IM + 1)))
        fi = pinned_like(np.zeros((KM, JM, IM + 1))); fj = pinned_like(np.zeros((KM, JM + 1, IM)))
        fk = pinned_like(np.zeros((KM + 1, JM, IM)))
        from fdf_gb300.context import _ptr
        lib, h = ctx.lib, ctx.h
        import ctypes
        got = ctypes.c_int64()
        k_e2e = max(3, min(args.steps, 10))
        barrier(dist)
        t0 = time.perf_counter()
        ps = 0
        n_cur = n0
        for _ in range(k_e2e):
            ctx._check(lib.fdf_SetSwarm(h, n_cur, _ptr(bufs.position), _ptr(bufs.velocity), _ptr(bufs.weight),
                                        _ptr(bufs.P), _ptr(bufs.cell), _ptr(bufs.pid), _ptr(bufs.status)))
            ctx._check(lib.fdf_AdvanceStep(h, None))
            ctx._check(lib.fdf_GetSwarm(h, n0, ctypes.byref(got), _ptr(bufs.position), _ptr(bufs.velocity),
                                        _ptr(bufs.weight), _ptr(bufs.P), _ptr(bufs.cell), _ptr(bufs.pid),
                                        _ptr(bufs.status)))
            ctx._check(lib.fdf_GetScatteredFields(h, _ptr(count), _ptr(avg)))
            ctx._check(lib.fdf_GetFaceDeposits(h, _ptr(fi), _ptr(fj), _ptr(fk)))
            ps += n_cur
            n_cur = got.value
        el = reduce_max(dist, time.perf_counter() - t0)
        e2e = {"value": ps * ws / el, "unit": UNIT, "h2d_bytes_per_step": int(120 * n0),
               "d2h_bytes_per_step": int(120 * n0 + 16 * Nn + 8 * Nf), "steps": k_e2e,
               "path": "fdf_SetSwarm + fdf_AdvanceStep + fdf_GetSwarm/GetScatteredFields/GetFaceDeposits, "
                       "pinned host DMSwarm-layout arrays"}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        from oracle import oracle as O
        O.build()
        nthreads = os.cpu_count() or 1
        v, st, el, sample = time_oracle(wl, budget_s=float(args.cpu_seconds), max_steps=1000, nthreads=nthreads)
        cpu = {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": wl.name, "form": "plain_fp64", "grid": f"{IM}x{JM}x{KM}",
                           "particles": wl.n, "cfl": wl.meta.get("cfl"), "dt": wl.dt,
                           "parallelism": "replicas" if ws > 1 else "single",
                           "initial_cell": ("corner cell (0,0,0), as the reference" if wl.meta.get("corner_start")
                                            or wl.meta.get("family") == "uniform" else
                                            "generating cell of each particle (harness choice)"),
                           "l2": "inputs larger than L2 (plane table %.2f GB, swarm %.0f MB)"
                                 % (38 * 8 * Nc / 1e9, 2 * 93 * wl.n / 1e6),
                           "walk_evals_per_particle_step": evals / max(psteps, 1)},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
                "clocks": clk}
        print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="fdf", choices=["fdf", "reference"])
    ap.add_argument("--workload", default="sinusoidal")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, ws, local, dist = dist_init()
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        run_gpu(args, rank, ws, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
