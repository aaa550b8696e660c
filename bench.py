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

# Algorithmic bytes: particle state per particle, plus
# one FP32 plane-table row per walk evaluation beyond the first (the first evaluation's row is
# the particle's own cell, shared by the cell's particles in the cell-sorted order; so is the
# FP64 row of the cell the plain walk concludes in, whose six distances give the weights).
ROW_BYTES = 128          # one 128-B FP32 plane-table row (8 x 16 B) read per walk evaluation
LOCATE_PER_PARTICLE = 53 + 61
GATHER_PER_PARTICLE = 8 + 64 + 93


def workload(name: str):
    from fdf_gb300 import workloads as W
    if name == "sinusoidal":           # the curvilinear plain-FP64 configuration
        return W.config_sinusoidal(64, 64, 1024, n=1_000_000, cfl=0.5, steps=50)
    if name == "uniform":
        return W.config1()
    if name == "sinusoidal96":
        return W.config_sinusoidal(96, 96, 1536, n=16_000_000, cfl=1.0, steps=100, materialize=False)
    if name == "bent_pipe":
        return W.config_bent_pipe(materialize=False)
    if name == "bent_pipe_8m":
        return W.config_bent_pipe(n=8_000_000, materialize=False)
    if name == "bent_pipe_small":      # profiling case: 885K cells, 2M particles (> L2)
        return W.config_bent_pipe(48, 48, 384, n=2_000_000, materialize=False)
    if name.startswith("bent_pipe_8m_cfl"):   # displacement sweep: bent_pipe_8m_cfl<C>
        return W.config_bent_pipe(n=8_000_000, cfl=float(name[len("bent_pipe_8m_cfl"):]), materialize=False)
    if name == "curved_pipe":
        return W.config_curved_pipe(materialize=False)
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


def bf16_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def host_link_gbs(device: int) -> dict:
    """Raw copy rate between pinned host memory and the GPU (1 GiB each way, best of 3)."""
    import torch
    n = 1 << 27
    x = torch.empty(n, dtype=torch.float64, device=f"cuda:{device}")
    hbuf = torch.empty(n, dtype=torch.float64, pin_memory=True)
    best = {"h2d": 0.0, "d2h": 0.0}
    for _ in range(3):
        torch.cuda.synchronize()
        a = time.perf_counter()
        x.copy_(hbuf, non_blocking=True)
        torch.cuda.synchronize()
        b = time.perf_counter()
        hbuf.copy_(x, non_blocking=True)
        torch.cuda.synchronize()
        c = time.perf_counter()
        best["h2d"] = max(best["h2d"], 8 * n / (b - a) / 1e9)
        best["d2h"] = max(best["d2h"], 8 * n / (c - b) / 1e9)
    return {k: round(v, 1) for k, v in best.items()}


_PINNED = []   # the page-locked tensors behind pinned_like's arrays (numpy views do not keep them)


def pinned_like(a: np.ndarray) -> np.ndarray:
    """A page-locked copy of a (torch pinned memory, 16-byte aligned); fails loudly if the
    allocation fails, since the end-to-end leg is defined on page-locked caller arrays."""
    import torch
    t = torch.empty(a.size * a.itemsize + 16, dtype=torch.uint8, pin_memory=True)
    start = (-t.data_ptr()) % 16
    out = t.numpy()[start:start + a.size * a.itemsize].view(a.dtype).reshape(a.shape)
    out[...] = a
    _PINNED.append(t)
    return out


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
    pos_s, cell_s, pid_s = wl.sample(sample)      # the first `sample` particles: an i.i.d. sample
    s = O.Swarm.create(pos_s, cell=cell_s, pid=pid_s)
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
    return n / t_full, steps, el, (f"first {sample} of {n} particles (i.i.d.) x {steps} steps on the full grid; "
                                   f"per-particle time scaled to {n} plus the grid-sized work ({t_grid:.3f} s/step)")


def run_reference(args, rank):
    """The reference algorithm on the host cores: the CPU restatement of the path (OpenMP over all
    cores), on the whole workload -- every particle, the full grid -- from its initial setup, then
    W warm-up steps and K timed steps, each one full step of the reference's loop."""
    if rank != 0:
        return
    from fdf_gb300.context import SwarmArrays
    from oracle import oracle as O
    O.build()
    wl = workload(args.workload)
    nthreads = os.cpu_count() or 1
    pos, cell, pid = wl.sample(wl.n)
    s0 = SwarmArrays.create(pos, cell=cell, pid=pid)
    del pos, cell, pid
    os_ = O.Swarm(pos=s0.position, vel=s0.velocity, weight=s0.weight, P=s0.P, cell=s0.cell, pid=s0.pid,
                  status=s0.status, n=s0.n)
    sim = O.Simulation(O.Grid(wl.coor), wl.ucat_node_sized(), os_, wl.dt, nthreads=nthreads)
    sim.initial_setup()
    for _ in range(args.warmup):
        sim.step()
    psteps = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        psteps += os_.n
        sim.step()
    total = time.perf_counter() - t0
    value = psteps / total
    sample = f"full workload: {wl.n} particles, {args.warmup} warm-up + {args.steps} timed steps"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl.name, "form": "reference algorithm (CPU restatement, pinned bit for bit to "
                                                    "the reference's own C compiled here)", "cores": nthreads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU

FORMS = {"plain_fp64": 0, "fp32": 1, "learned_fp32": 2}
FORM_DTYPE = {"plain_fp64": "f64", "fp32": "f32 (positions and walk decisions f64)",
              "learned_fp32": "f32 (positions and walk decisions f64; MLP trained in bf16, inference {} "
                              "operands, f32 accumulate)"}
LOCATOR_TYPES = {"bf16": 0, "f16": 1}
MLP_FLOPS = 2 * (3 * 128 + 128 * 128 + 128 * 128 + 128 * 3)   # per particle, one inference

# DRAM bytes (read + write) per launch of a stage's kernels, measured by ncu
# (dram__bytes_read.sum + dram__bytes_write.sum, one pass) on this workload at full size, with
# the units the stage processed then: live particles, or guessed particles for the network and
# the walk from the guess.  The precision forms' sort stage: scan and slot scatter as captured
# with the PID-ordered sort, plus the ordering kernel captured since it orders by previous slot
# (0.364 GB instead of 1.02 GB per launch).
TRAFFIC = {
    ("bent_pipe_96x96x1536_n64000000_cfl4", "learned_fp32", "advect_locate"): (7.757e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "learned_fp32", "learned_guess"): (0.596e9, "guesses", 12.92e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "learned_fp32", "guess_walk"): (2.063e9, "guesses", 12.92e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "learned_fp32", "sort_by_cell"): (1.213e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "learned_fp32", "gather_interpolate"): (7.906e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "learned_fp32", "deposit"): (1.345e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "fp32", "advect_locate"): (7.623e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "fp32", "sort_by_cell"): (1.213e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "fp32", "gather_interpolate"): (7.906e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "fp32", "deposit"): (1.345e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "plain_fp64", "advect_locate"): (13.444e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "plain_fp64", "gather_interpolate"): (10.885e9, "particles", 63.81e6),
    ("bent_pipe_96x96x1536_n64000000_cfl4", "plain_fp64", "deposit"): (2.651e9, "particles", 63.81e6),
}


def stage_traffic(wl, form: str, stage: str, n_avg: float, guesses: float):
    """Measured DRAM bytes per launch of the stage, scaled to this run's units, or None."""
    t = TRAFFIC.get((wl.name, form, stage))
    if t is None:
        return None
    total, unit, units = t
    return total * ((guesses if unit == "guesses" else n_avg) / units)

_TRAINED = {}   # workload name -> (trained parameters, training report)


def momentum_on(wl) -> bool:
    """The curved-pipe configuration deposits particle momentum as well as volume."""
    return wl.meta.get("family") == "curved_pipe"


def prepare(ctx, wl, form, args):
    """Loads the workload in a form; the learned form gets its locator (trained once per
    workload on the device, then reinstalled)."""
    ctx.load_workload(wl, form=FORMS[form])
    if momentum_on(wl):
        ctx.set_momentum_deposit(True)
    if form != "learned_fp32":
        return
    if args.guess_min_cells is not None:
        ctx.locator_min_distance(args.guess_min_cells)
    ctx.locator_inference_type(LOCATOR_TYPES[args.locator_type])
    if wl.name not in _TRAINED:
        import torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hist = ctx.locator_train(args.train_samples, seed=17, steps=args.train_steps, batch=args.train_batch,
                                 lr=args.train_lr)
        el = time.perf_counter() - t0
        _TRAINED[wl.name] = (ctx.locator_get_params(), {
            "samples": args.train_samples, "steps": args.train_steps, "batch": args.train_batch, "lr": args.train_lr,
            "seconds": round(el, 3), "loss_first": float(np.mean(hist[:20])), "loss_last": float(np.mean(hist[-50:])),
            "loss_unit": "mean squared error in cells per axis"})
    else:
        ctx.locator_set_params(_TRAINED[wl.name][0])


def algorithmic_bytes(form: str, n_avg: float, evals_per_step: float, nodes_per_step: float, Nc: int, Nn: int,
                      Nf: int, momentum: bool = False, pending: float = 0.0, pending_evals: float = 0.0) -> dict:
    """Algorithmic bytes per launch of each stage; the momentum deposit adds the particles'
    velocities and three components per face."""
    if form == "learned_fp32":
        # first pass: one evaluation per particle, the per-warp pending masks and counts (under a
        # byte per particle with their scan and compaction); walk from the guess: the pending
        # particles' state and the remaining evaluations
        return {
            "center_to_corner": 24 * nodes_per_step,
            "advect_locate": 86 * n_avg + 1 * n_avg + ROW_BYTES * max(evals_per_step - n_avg - pending_evals, 0.0),
            "guess_walk": 57 * pending + ROW_BYTES * pending_evals,
            "sort_by_cell": 24 * n_avg + 12 * (Nc + 2),
            "wait_corner": 0,
            "gather_interpolate": 121 * n_avg + 12 * Nn,
            "deposit": 4 * (Nc + 1) + 16 * n_avg + 8 * Nn + 4 * Nf + (12 * n_avg + 12 * Nf if momentum else 0),
        }
    if form == "fp32":
        return {
            "center_to_corner": 24 * nodes_per_step,
            "advect_locate": 86 * n_avg + ROW_BYTES * max(evals_per_step - n_avg, 0.0),
            "sort_by_cell": 24 * n_avg + 12 * (Nc + 2),
            "wait_corner": 0,
            "gather_interpolate": 121 * n_avg + 12 * Nn,
            "deposit": 4 * (Nc + 1) + 16 * n_avg + 8 * Nn + 4 * Nf + (12 * n_avg + 12 * Nf if momentum else 0),
        }
    return {
        "center_to_corner": 48 * nodes_per_step,
        "advect_locate": LOCATE_PER_PARTICLE * n_avg + ROW_BYTES * max(evals_per_step - n_avg, 0.0),
        "sort_by_cell": 24 * n_avg + 12 * (Nc + 2),
        "wait_corner": 0,
        "gather_interpolate": GATHER_PER_PARTICLE * n_avg + 24 * Nn,
        "deposit": 4 * (Nc + 1) + 32 * n_avg + 16 * Nn + 8 * Nf + (24 * n_avg + 24 * Nf if momentum else 0),
    }


def time_form(ctx, wl, form, args, dist, local, with_clocks):
    """Warm-up, then the timed steps of one form; returns its measurements."""
    import torch
    IM, JM, KM = wl.dims
    Nc, Nn = IM * JM * KM, (IM + 1) * (JM + 1) * (KM + 1)
    Nf = (IM + 1) * JM * KM + IM * (JM + 1) * KM + IM * JM * (KM + 1)
    prepare(ctx, wl, form, args)
    ctx.initial_setup()
    ctx.steps(args.warmup)
    ctx.synchronize()
    guess0 = ctx.locator_stats() if form == "learned_fp32" else None
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ps0, e0, nd0 = ctx.counters()
    l0 = ctx.launches
    clocks = ClockSampler(local) if with_clocks else None
    barrier(dist)
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
        time.sleep(0.3)
    ev0.record(stream)
    ctx.steps(args.steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    barrier(dist)
    clk = clocks.stop() if clocks else None
    ms_max = reduce_max(dist, ev0.elapsed_time(ev1))
    ps1, e1, nd1 = ctx.counters()
    launches = ctx.launches - l0
    if form == "learned_fp32":
        guess1 = ctx.locator_stats()
    # stage breakdown: separate eager steps with CUDA events between the stages (the timed
    # steps above replay the captured step graph, which has no events inside)
    ctx.set_profiling(True)
    ctx.steps(min(args.steps, 5))
    stages = ctx.stage_times()
    ctx.set_profiling(False)
    psteps, evals = ps1 - ps0, e1 - e0
    K = max(args.steps, 1)
    n_avg = psteps / K
    runs = max(stages["sort_by_cell"][1], 1)     # one span per pipeline run
    per = {k: (v[0] / runs) for k, v in stages.items() if v[1] > 0}
    learned = None
    asked = taken = gev = fev = 0
    if form == "learned_fp32":
        asked, taken, gev, fev = (b - a for a, b in zip(guess0, guess1))
    alg = algorithmic_bytes(form, n_avg, evals / K, (nd1 - nd0) / K, Nc, Nn, Nf, momentum_on(wl), asked / K,
                            (gev + fev) / K)
    if form == "learned_fp32":
        mlp_ms = per.get("learned_guess", 0.0)
        tfl = MLP_FLOPS * asked / K / (mlp_ms / 1000.0) / 1e12 if mlp_ms > 0 else None
        learned = {"guesses_per_step": asked / K, "guess_fraction": asked / max(psteps, 1),
                   "walk_evals_from_P1_per_guess": gev / max(asked, 1),
                   "evals_after_P1_on_predicted_path": taken / max(gev - asked, 1),
                   "mlp_tflops": tfl, "mlp_flops_per_particle": MLP_FLOPS,
                   "inference_operands": args.locator_type, "training": _TRAINED[wl.name][1]}
    traffic = {k: stage_traffic(wl, form, k, n_avg, asked / K) for k in per}
    return dict(form=form, psteps=psteps, evals=evals, ms=ms_max, launches=launches, clocks=clk, per=per, alg=alg,
                learned=learned, traffic=traffic,
                value=psteps * int(os.environ.get("WORLD_SIZE", "1")) / (ms_max / 1000.0))


def learned_identity(ctx, wl, args, steps: int) -> dict:
    """The learned form against the FP32 form from the same initial state on the full
    workload: the swarms (cells, statuses, positions, velocities, weights) and the face
    deposits must be identical."""
    out = {}
    for form in ("fp32", "learned_fp32"):
        prepare(ctx, wl, form, args)
        ctx.initial_setup()
        ctx.steps(steps)
        out[form] = (ctx.get_swarm(), ctx.get_faces())
    (sa, fa), (sb, fb) = out["fp32"], out["learned_fp32"]
    same = {f: bool(np.array_equal(getattr(sa, f), getattr(sb, f)))
            for f in ("cell", "status", "pid", "position", "velocity", "weight", "P")}
    same["faces"] = all(bool(np.array_equal(x, y)) for x, y in zip(fa, fb))
    return {"steps": steps, "particles": int(sa.n), "identical": same,
            "cells_differing": int(np.any(sa.cell != sb.cell, axis=1).sum()) if sa.n == sb.n else None}


def _by_pid(pid: np.ndarray, a: np.ndarray, n_ids: int, fill) -> np.ndarray:
    """a scattered into a PID-indexed array of n_ids rows (PIDs are 0 .. n_ids-1), O(n)."""
    out = np.full((n_ids,) + a.shape[1:], fill, dtype=a.dtype)
    out[pid] = a
    return out


def compare_by_pid(gpu, ref: dict, n_ids: int) -> dict:
    """Bit-for-bit comparison of two swarms by PID (any order): the particle sets, then every field
    (floating-point fields compared as bit patterns).  Returns per-field identical flags and the
    number of particles that differ in each."""
    present_g = np.zeros(n_ids, bool)
    present_g[gpu.pid] = True
    present_r = np.zeros(n_ids, bool)
    present_r[ref["pid"]] = True
    out = {"particles": int(len(gpu.pid)), "oracle_particles": int(len(ref["pid"])),
           "same_particle_set": bool(np.array_equal(present_g, present_r))}
    both = present_g & present_r
    for name, g, r in (("cell", gpu.cell, ref["cell"]), ("status", gpu.status, ref["status"]),
                       ("position", gpu.position, ref["pos"]), ("velocity", gpu.velocity, ref["vel"]),
                       ("weight", gpu.weight, ref["weight"]), ("P", gpu.P, ref["P"])):
        gi = g.view(np.int64) if g.dtype == np.float64 else g
        ri = r.view(np.int64) if r.dtype == np.float64 else r
        a = _by_pid(gpu.pid, gi, n_ids, -7)
        b = _by_pid(ref["pid"], ri, n_ids, -7)
        diff = (a != b).reshape(n_ids, -1).any(axis=1) & both
        out[name] = {"identical": bool(not diff.any()), "particles_differing": int(diff.sum())}
        del a, b, diff
    return out


def plain_parity_full(ctx, wl, steps: int, nthreads: int) -> dict:
    """The plain FP64 form against the FP64 oracle on the whole workload (every particle, the full
    grid) from the same initial state: initial setup, then `steps` steps; every swarm field, the
    removal counts, ParticleCount, the P average and the face deposits (with momentum where the
    workload deposits it), bit for bit."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    ctx.load_workload(wl, form=FORMS["plain_fp64"])
    mom = momentum_on(wl)
    if mom:
        ctx.set_momentum_deposit(True)
    s0 = ctx.get_swarm()
    n0 = s0.n
    os_ = O.Swarm(pos=s0.position, vel=s0.velocity, weight=s0.weight, P=s0.P, cell=s0.cell, pid=s0.pid,
                  status=s0.status, n=n0)
    del s0
    ctx.initial_setup()
    removed_gpu = []
    for _ in range(steps):
        info = ctx.step()
        removed_gpu.append((int(info.removed_lost), int(info.removed_oob)))
    gpu = ctx.get_swarm()
    gcount, gavg = ctx.get_scattered()
    gfaces = ctx.get_faces()
    gmom = ctx.get_face_momentum() if mom else None
    t_gpu = time.perf_counter() - t0
    t1 = time.perf_counter()
    g = O.Grid(wl.coor)
    sim = O.Simulation(g, wl.ucat_node_sized(), os_, wl.dt, nthreads=nthreads)
    sim.initial_setup()
    removed_ref = []
    for _ in range(steps):
        info = sim.step()
        removed_ref.append((int(info.removed_lost), int(info.removed_oob)))
    t_oracle = time.perf_counter() - t1
    t2 = time.perf_counter()
    out = compare_by_pid(gpu, os_.view(), n0)
    out["removed_per_step"] = {"gpu": removed_gpu, "oracle": removed_ref, "identical": removed_gpu == removed_ref}
    out["count"] = bool(np.array_equal(gcount.view(np.int64), sim.count.view(np.int64)))
    out["P_avg"] = bool(np.array_equal(gavg.view(np.int64), sim.avg.view(np.int64)))
    del gpu
    f = O.deposit_faces(g, os_, volume=wl.volume, momentum=mom)
    out["faces"] = all(bool(np.array_equal(a.view(np.int64), f[k].view(np.int64)))
                       for a, k in zip(gfaces, ("fi", "fj", "fk")))
    if mom:
        out["momentum_faces"] = all(bool(np.array_equal(a.view(np.int64), f[k].view(np.int64)))
                                    for a, k in zip(gmom, ("mom_i", "mom_j", "mom_k")))
    fields = ("same_particle_set", "cell", "status", "position", "velocity", "weight", "P")
    out["identical"] = bool(all(out[k] if isinstance(out[k], bool) else out[k]["identical"] for k in fields)
                            and out["removed_per_step"]["identical"] and out["count"] and out["P_avg"]
                            and out["faces"] and out.get("momentum_faces", True))
    out.update({"workload": wl.name, "steps_after_initial_setup": steps, "initial_particles": int(n0),
                "oracle_threads": nthreads,
                "seconds": {"gpu_and_transfers": round(t_gpu, 1), "oracle": round(t_oracle, 1),
                            "compare": round(time.perf_counter() - t2, 1)}})
    return out


def fp32_errors_full(ctx, wl, steps: int, sample: int, nthreads: int) -> dict:
    """The precision form on the whole workload for `steps` steps, against the FP64 oracle.
    Particles do not interact, so every particle's trajectory in the full run is its trajectory
    alone: the per-particle errors are measured on the particles with PID < sample (an i.i.d.
    sample of the seeded swarm, stepped by the oracle from the same initial state), and the grid
    fields (face volume and momentum deposits, ParticleCount, P average) on a run of that sample
    alone, whose per-particle values are checked to equal the full run's."""
    from dataclasses import replace

    from fdf_gb300.context import FORM_FP32, SwarmArrays
    from oracle import oracle as O
    t0 = time.perf_counter()
    mom = momentum_on(wl)
    ctx.load_workload(wl, form=FORM_FP32)
    if mom:
        ctx.set_momentum_deposit(True)
    ctx.initial_setup()
    ctx.steps(steps)
    full = ctx.get_swarm()
    keep = full.pid < sample
    sub_full = SwarmArrays(*(getattr(full, f)[keep] for f in ("position", "velocity", "weight", "P", "cell", "pid",
                                                               "status"))).sorted_by_pid()
    n_full = int(full.n)
    del full
    pos_m, cell_m, _ = wl.sample(sample)
    wl_s = replace(wl, pos=pos_m, cell0=cell_m, seed_n=len(pos_m))
    ctx.load_workload(wl_s, form=FORM_FP32)
    if mom:
        ctx.set_momentum_deposit(True)
    ctx.initial_setup()
    ctx.steps(steps)
    sub_run = ctx.get_swarm().sorted_by_pid()
    gfaces = ctx.get_faces()
    gmom = ctx.get_face_momentum() if mom else None
    gcount, gavg = ctx.get_scattered()
    same_as_full = all(bool(np.array_equal(getattr(sub_full, f), getattr(sub_run, f)))
                       for f in ("position", "velocity", "weight", "P", "cell", "pid", "status"))
    t_gpu = time.perf_counter() - t0
    t1 = time.perf_counter()
    g = O.Grid(wl.coor)
    s0 = SwarmArrays.create(pos_m, cell=cell_m)
    os_ = O.Swarm(pos=s0.position, vel=s0.velocity, weight=s0.weight, P=s0.P, cell=s0.cell, pid=s0.pid,
                  status=s0.status, n=s0.n)
    sim = O.Simulation(g, wl.ucat_node_sized(), os_, wl.dt, nthreads=nthreads)
    sim.initial_setup()
    for _ in range(steps):
        sim.step()
    t_oracle = time.perf_counter() - t1
    ref = os_.sorted_by_pid()
    common, ia, ib = np.intersect1d(sub_run.pid, ref["pid"], return_indices=True)

    def stats(err):
        err = np.asarray(err, dtype=np.float64).ravel()
        return {"max": float(err.max()) if err.size else 0.0,
                "rms": float(np.sqrt((err ** 2).mean())) if err.size else 0.0}

    # Particles whose FP32 trajectory (positions within ~1e-8 of the FP64 ones) crossed a cell face,
    # a k-face gap or the box on a different side than the FP64 one: counted, and kept out of the
    # per-particle statistics; the grid fields are compared away from the cells they touched.
    same = np.all(sub_run.cell[ia] == ref["cell"][ib], axis=1)
    ja, jb = ia[same], ib[same]
    IM, JM, KM = wl.dims
    touched = np.zeros((KM, JM, IM), bool)
    for cells in (sub_run.cell[ia[~same]], ref["cell"][ib[~same]],
                  sub_run.cell[np.setdiff1d(np.arange(len(sub_run.pid)), ia)],
                  ref["cell"][np.setdiff1d(np.arange(len(ref["pid"])), ib)]):
        cells = cells[np.all(cells >= 0, axis=1)]
        touched[cells[:, 2], cells[:, 1], cells[:, 0]] = True
    pad = np.pad(touched, 1)   # a face is touched when a cell on either side is
    face_masks = (~(pad[1:-1, 1:-1, :-1] | pad[1:-1, 1:-1, 1:]), ~(pad[1:-1, :-1, 1:-1] | pad[1:-1, 1:, 1:-1]),
                  ~(pad[:-1, 1:-1, 1:-1] | pad[1:, 1:-1, 1:-1]))
    node_ok = np.ones(gcount.shape, bool)
    node_ok[:KM, :JM, :IM] = ~touched
    umag = np.maximum(np.linalg.norm(ref["vel"][jb], axis=1, keepdims=True), 1e-30)
    f = O.deposit_faces(g, os_, volume=wl.volume, momentum=mom)
    face_err = np.concatenate([(np.abs(a - f[k]) / wl.volume)[mk].ravel()
                               for a, k, mk in zip(gfaces, ("fi", "fj", "fk"), face_masks)])
    occupied = (sim.count > 0) & node_ok
    out = {"workload": wl.name, "steps": steps, "full_run_particles": n_full, "sample_particles": int(len(pos_m)),
           "sample": f"PID < {sample} (i.i.d. seeding): per-particle values from the full run; grid fields "
                     f"from a run of the sample alone",
           "sample_run_equals_full_run": same_as_full,
           "particles_compared": int(len(common)),
           "particles_removed_by_one_side_only": int(len(sub_run.pid) + len(ref["pid"]) - 2 * len(common)),
           "particles_in_another_cell": int((~same).sum()),
           "same_cell_fraction": float(same.mean()),
           "statistics_over": "particles in the same cell on both sides; grid fields away from the cells of the "
                              "particles counted above",
           "velocity_rel": stats(np.abs(sub_run.velocity[ja] - ref["vel"][jb]) / umag),
           "position_abs": stats(np.abs(sub_run.position[ja] - ref["pos"][jb])),
           "weight_abs": stats(np.abs(sub_run.weight[ja] - ref["weight"][jb])),
           "face_volume_abs_per_particle_volume": stats(face_err),
           "count_abs": stats(np.abs(gcount - sim.count)[node_ok]),
           "P_avg_rel": stats(np.abs(gavg[occupied] - sim.avg[occupied]) / np.abs(sim.avg[occupied])),
           "oracle_threads": nthreads,
           "seconds": {"gpu_and_transfers": round(t_gpu, 1), "oracle": round(t_oracle, 1)}}
    if mom:
        scale = np.abs(ref["vel"]).max() * wl.volume
        out["face_momentum_abs_per_particle_momentum"] = stats(np.concatenate(
            [(np.abs(a - f[k]) / scale)[mk].ravel() for a, k, mk in zip(gmom, ("mom_i", "mom_j", "mom_k"),
                                                                         face_masks)]))
    return out


FP64_OPS_C2C = 21      # 3 face sums, 9 products, 6 sums, 3 scalings per interior cell
CLOCK_MAX_MHZ = 2070   # GB300 maximum SM clock


def time_contra2cart(ctx, wl, calls: int) -> dict:
    """Contra2Cart (setup.c:1294-1420) on the workload's grid: the face fluxes of a uniform
    flow are uploaded once, the first call builds the metric table (timed on the host), then
    `calls` calls are timed with CUDA events on the context stream.  Inputs (face velocity,
    table) are larger than L2."""
    from fdf_gb300.workloads import uniform_flow_fluxes
    IM, JM, KM = wl.dims
    Nc, Nn = IM * JM * KM, (IM + 1) * (JM + 1) * (KM + 1)
    n_int = (IM - 1) * (JM - 1) * (KM - 1)
    ctx.set_grid(wl.coor)
    ctx.set_ucat(wl.ucat)
    csi, eta, zet, _, flipped = ctx.grid_metrics()
    u = np.array([0.3, -0.2, 1.1])
    ctx.set_ucont(uniform_flow_fluxes(u, csi, eta, zet))
    del csi, eta, zet
    ctx.synchronize()
    t0 = time.perf_counter()
    ctx.contra2cart()
    ctx.synchronize()
    table_ms = 1000.0 * (time.perf_counter() - t0)
    ctx.set_profiling(True)
    for _ in range(calls):
        ctx.contra2cart()
    ms_total, runs = ctx.stage_times()["contra2cart"]
    ctx.set_profiling(False)
    ms = ms_total / max(runs, 1)
    err = float(np.abs(ctx.get_ucat(node_sized=False)[1:, 1:, 1:] - u).max())
    alg = 116 * n_int + 24 * Nn        # table 80 + ucat 24 + ucat32 12 per interior cell, face velocity per node
    hbm, peak_kind = peaks()
    gbs = alg / (ms / 1000.0) / 1e9
    # the bound: GB300's FP64 pipe, two lanes per clock per SM (ncu: sm__pipe_fp64_cycles_active
    # 83 % with 21 FP64 instructions per cell)
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    fp64_peak = 2.0 * sms * CLOCK_MAX_MHZ * 1e6 / 1e9
    gops = FP64_OPS_C2C * n_int / (ms / 1000.0) / 1e9
    return {"ms_per_call": ms, "calls": runs, "table_build_ms": table_ms, "interior_cells": n_int,
            "bound": "fp64", "fp64_ops_per_cell": FP64_OPS_C2C, "achieved_fp64_gops": gops,
            "fp64_pipe_peak_gops": fp64_peak, "fp64_frac": gops / fp64_peak,
            "fp64_peak_source": f"2 FP64 lanes per clock x {sms} SMs x {CLOCK_MAX_MHZ} MHz",
            "algorithmic_bytes_per_call": alg, "achieved_gbs": gbs, "hbm_frac": gbs / hbm,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "uniform_flow_max_abs_error": err, "grid_flipped": flipped}


def run_gpu(args, rank, ws, local, dist):
    from fdf_gb300.context import PicContext, SwarmArrays
    import torch

    wl = workload(args.workload)
    IM, JM, KM = wl.dims
    Nc, Nn = IM * JM * KM, (IM + 1) * (JM + 1) * (KM + 1)
    Nf = (IM + 1) * JM * KM + IM * (JM + 1) * KM + IM * JM * (KM + 1)
    forms = [f.strip() for f in args.forms.split(",") if f.strip()]
    ctx = PicContext(local)
    results = {}
    for q, form in enumerate(forms):
        results[form] = time_form(ctx, wl, form, args, dist, local, with_clocks=(q == 0))
    prim = results[forms[0]]
    value, ms_max, psteps, evals, launches, clk = (prim["value"], prim["ms"], prim["psteps"], prim["evals"],
                                                   prim["launches"], prim["clocks"])

    # roofline of the dominant stage of the primary form (algorithmic bytes / mean event-timed duration)
    hbm, peak_kind = peaks()
    per, alg = prim["per"], prim["alg"]
    dom = max((k for k in per if alg.get(k)), key=per.get)
    achieved = alg[dom] / (per[dom] / 1000.0) / 1e9
    tr = prim["traffic"].get(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": alg[dom], "traffic": tr,
                "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum at this configuration, "
                                   "scaled to this run's particles" if tr is not None else None),
                "dram_gbs": (tr / (per[dom] / 1000.0) / 1e9 if tr is not None else None),
                "stage_ms_per_step": {k: round(v, 4) for k, v in per.items()},
                "stage_gbs": {k: round(alg[k] / (per[k] / 1000.0) / 1e9, 1) for k in per if per[k] > 0 and alg.get(k)}}
    lp = prim.get("learned")
    if lp and lp["mlp_tflops"] and per.get("learned_guess", 0.0) > per[dom]:
        # the network inference dominates: its roofline is the tensor one
        tf, tf_kind = bf16_peak()
        roofline.update({"bound": "tensor", "kernel": "learned_guess (k_mlp_guess_tc)", "achieved": lp["mlp_tflops"],
                         "traffic": prim["traffic"].get("learned_guess"),
                         "peak": tf, "unit": "TFLOP/s", "frac": lp["mlp_tflops"] / tf,
                         "peak_source": f"{tf_kind} (MEASURED_PEAKS.json bf16_tflops)",
                         "algorithmic_flops_per_launch": MLP_FLOPS * lp["guesses_per_step"],
                         "hbm_stage": {"kernel": dom, "achieved_gbs": achieved, "frac": achieved / hbm}})
        roofline.pop("algorithmic_bytes_per_launch", None)
    form_lines = {f: {"particle_steps_per_s": r["value"], "ms_per_step": r["ms"] / max(args.steps, 1),
                      "walk_evals_per_particle_step": r["evals"] / max(r["psteps"], 1),
                      "stage_ms_per_step": {k: round(v, 4) for k, v in r["per"].items()},
                      **({"learned_locator": r["learned"]} if r["learned"] else {})}
                  for f, r in results.items()}
    identity = None
    if "learned_fp32" in forms and args.identity_steps > 0 and ws == 1:   # a check, not a measurement
        identity = learned_identity(ctx, wl, args, args.identity_steps)
    prepare(ctx, wl, forms[0], args)
    ctx.initial_setup()

    # end to end through the C ABI with host (pinned) buffers
    e2e = None
    if not args.no_e2e:
        s_host = ctx.get_swarm()
        n0 = s_host.n
        bufs = SwarmArrays(*[pinned_like(np.ascontiguousarray(a)) for a in (s_host.position, s_host.velocity,
                                                                                s_host.weight, s_host.P,
                                                       s_host.cell, s_host.pid, s_host.status)])
        count = pinned_like(np.zeros((KM + 1, JM + 1, IM + 1)))
        avg = pinned_like(np.zeros((KM + 1, JM + 1, IM + 1)))
        fi = pinned_like(np.zeros((KM, JM, IM + 1))); fj = pinned_like(np.zeros((KM, JM + 1, IM)))
        fk = pinned_like(np.zeros((KM + 1, JM, IM)))
        mom = None
        if momentum_on(wl):
            mom = (pinned_like(np.zeros((KM, JM, IM + 1, 3))), pinned_like(np.zeros((KM, JM + 1, IM, 3))),
                   pinned_like(np.zeros((KM + 1, JM, IM, 3))))
        from fdf_gb300.context import TRANSFER_AUTO, TRANSFER_IN_PLACE, TRANSFER_STAGED, _ptr
        lib, h = ctx.lib, ctx.h
        import ctypes
        got = ctypes.c_int64()

        def e2e_steps(route, k: int):
            """k steps through the C ABI with the host arrays: set, step, get (swarm and fields);
            route None keeps the context's route (and what AUTO has measured)."""
            if route is not None:
                ctx.set_transfer_route(route)
            split = {"set_swarm": 0.0, "step": 0.0, "get_swarm": 0.0, "get_fields": 0.0}
            ps, n_cur, moved = 0, live[0], 0
            barrier(dist)
            t0 = time.perf_counter()
            for _ in range(k):
                ta = time.perf_counter()
                ctx._check(lib.fdf_SetSwarm(h, n_cur, _ptr(bufs.position), _ptr(bufs.velocity), _ptr(bufs.weight),
                                            _ptr(bufs.P), _ptr(bufs.cell), _ptr(bufs.pid), _ptr(bufs.status)))
                tb = time.perf_counter()
                ctx._check(lib.fdf_AdvanceStep(h, None))
                ctx._check(lib.fdf_Synchronize(h))
                tc = time.perf_counter()
                ctx._check(lib.fdf_GetSwarm(h, n0, ctypes.byref(got), _ptr(bufs.position), _ptr(bufs.velocity),
                                            _ptr(bufs.weight), _ptr(bufs.P), _ptr(bufs.cell), _ptr(bufs.pid),
                                            _ptr(bufs.status)))
                td = time.perf_counter()
                ctx._check(lib.fdf_GetScatteredFields(h, _ptr(count), _ptr(avg)))
                ctx._check(lib.fdf_GetFaceDeposits(h, _ptr(fi), _ptr(fj), _ptr(fk)))
                if mom is not None:
                    ctx._check(lib.fdf_GetFaceMomentum(h, _ptr(mom[0]), _ptr(mom[1]), _ptr(mom[2])))
                te = time.perf_counter()
                for key, v in zip(split, (tb - ta, tc - tb, td - tc, te - td)):
                    split[key] += v
                ps += n_cur
                moved += n_cur + got.value
                n_cur = got.value
            live[0] = n_cur
            el = reduce_max(dist, time.perf_counter() - t0)
            ms = {kk: round(1000.0 * v / k, 2) for kk, v in split.items()}
            gbs = {"set_swarm": round(120 * ps / split["set_swarm"] / 1e9, 1),
                   "get_swarm": round(120 * (moved - ps) / split["get_swarm"] / 1e9, 1)}
            return ps * ws / el, ms, gbs

        live = [n0]
        k_e2e = max(3, min(args.steps, 10))
        # the library's default route (AUTO: per direction, the route it measured faster on this
        # machine during an untimed first step) is the headline; the staged route (copy engines
        # through the staging buffer) and the in-place route (layout kernels reading and writing
        # the pinned arrays over the host link) are timed beside it in the same process
        e2e_steps(TRANSFER_AUTO, 1)
        chosen = ctx.transfer_routes()
        v_st, ms_st, gbs_st = e2e_steps(None, k_e2e)
        v_s2, ms_s2, gbs_s2 = e2e_steps(TRANSFER_STAGED, max(3, k_e2e // 2))
        v_ip, ms_ip, gbs_ip = e2e_steps(TRANSFER_IN_PLACE, max(3, k_e2e // 2))
        ctx.set_transfer_route(TRANSFER_AUTO)
        names = {TRANSFER_STAGED: "staged", TRANSFER_IN_PLACE: "in place", -1: "staged (not measured)"}
        link = host_link_gbs(local)
        e2e = {"value": v_st, "unit": UNIT, "h2d_bytes_per_step": int(120 * n0),
               "d2h_bytes_per_step": int(120 * n0 + 16 * Nn + 8 * Nf + (24 * Nf if mom is not None else 0)),
               "steps": k_e2e,
               "route": f"auto (the library default): upload {names[chosen[0]]}, download {names[chosen[1]]}",
               "path": "fdf_SetSwarm + fdf_AdvanceStep + fdf_GetSwarm/GetScatteredFields/GetFaceDeposits, "
                       "pinned host DMSwarm-layout arrays",
               "ms_per_step": ms_st, "transfer_gbs": gbs_st,
               "staged_route": {"value": v_s2, "ms_per_step": ms_s2, "transfer_gbs": gbs_s2},
               "in_place_route": {"value": v_ip, "ms_per_step": ms_ip, "transfer_gbs": gbs_ip},
               "host_link_gbs": link}

    # full-size checks against the FP64 oracle (all host cores): the plain form bit for bit on whole
    # workloads, and the precision form's per-field errors
    accuracy = fp32_cfg3 = None
    parity = []
    if rank == 0 and ws == 1:
        nthreads = os.cpu_count() or 1
        if args.parity_steps > 0:
            for name in [args.workload] + [w for w in args.parity_workloads.split(",") if w and w != args.workload]:
                parity.append(plain_parity_full(ctx, workload(name), args.parity_steps, nthreads))
        if args.accuracy_steps > 0 and ("fp32" in forms or "learned_fp32" in forms):
            accuracy = fp32_errors_full(ctx, wl, args.accuracy_steps, args.accuracy_sample, nthreads)
        if args.cfg3_steps > 0:
            fp32_cfg3 = fp32_errors_full(ctx, workload("sinusoidal96"), args.cfg3_steps, args.accuracy_sample,
                                         nthreads)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        from oracle import oracle as O
        O.build()
        nthreads = os.cpu_count() or 1
        v, st, el, sample = time_oracle(wl, budget_s=float(args.cpu_seconds), max_steps=1000, nthreads=nthreads)
        cpu = {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample}

    c2c = None
    if rank == 0 and not args.no_contra2cart:
        c2c = time_contra2cart(ctx, wl, max(args.steps, 5))

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": FORM_DTYPE[forms[0]].format(args.locator_type), "data": "synthetic",
                "config": {"workload": wl.name, "form": forms[0], "grid": f"{IM}x{JM}x{KM}",
                           "particles": wl.n, "cfl": wl.meta.get("cfl"), "dt": wl.dt,
                           "parallelism": "replicas" if ws > 1 else "single",
                           "initial_cell": ("corner cell (0,0,0), as the reference" if wl.meta.get("corner_start")
                                            or wl.meta.get("family") == "uniform" else
                                            "generating cell of each particle (harness choice)"),
                           "l2": "inputs larger than L2 (plane table %.2f GB, swarm %.0f MB)"
                                 % (38 * 8 * Nc / 1e9, 2 * 93 * wl.n / 1e6),
                           "walk_evals_per_particle_step": evals / max(psteps, 1),
                           "deposits": "face volume" + (" and momentum" if momentum_on(wl) else "")},
                "roofline": roofline, "forms": form_lines,
                "plain_vs_oracle_full": [{"config": c["workload"], "particles": c["initial_particles"],
                                          "steps": c["steps_after_initial_setup"], "identical": c["identical"],
                                          "detail": c} for c in parity] or None,
                "fp32_accuracy_vs_fp64_oracle": accuracy, "fp32_errors_cfg3": fp32_cfg3,
                "learned_vs_fp32_form": identity,
                "cpu_baseline": cpu, "e2e": e2e, "contra2cart": c2c,
                "gpu_launches": launches, "clocks": clk}
        print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="fdf", choices=["fdf", "reference"])
    ap.add_argument("--workload", default="bent_pipe")
    ap.add_argument("--forms", default="learned_fp32,fp32,plain_fp64",
                    help="comma list; the first is the headline value, the others are reported beside it")
    ap.add_argument("--train-samples", type=int, default=4_000_000)
    ap.add_argument("--train-steps", type=int, default=16000)
    ap.add_argument("--train-batch", type=int, default=8192)
    ap.add_argument("--train-lr", type=float, default=2e-3)
    ap.add_argument("--locator-type", default="bf16", choices=sorted(LOCATOR_TYPES),
                    help="learned form: operand type of the network's tensor-core inference")
    ap.add_argument("--guess-min-cells", type=float, default=None,
                    help="learned form: particles at least this many cells past their cell get a guess")
    ap.add_argument("--identity-steps", type=int, default=3,
                    help="steps of the learned-vs-FP32-form identity check on the full workload (0 = skip)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-contra2cart", action="store_true",
                    help="skip timing the Eulerian input (Contra2Cart on the workload's grid)")
    ap.add_argument("--accuracy-steps", type=int, default=10,
                    help="steps of the FP32-form vs FP64-oracle comparison on the full workload (0 = skip)")
    ap.add_argument("--accuracy-sample", type=int, default=1_000_000,
                    help="particles (the first PIDs, an i.i.d. sample) the oracle steps for the FP32-form errors")
    ap.add_argument("--cfg3-steps", type=int, default=100,
                    help="steps of the FP32-form errors on the 96x96x1536 sinusoidal grid, 16M particles (0 = skip)")
    ap.add_argument("--parity-steps", type=int, default=2,
                    help="steps after the initial setup of the plain-form full-size parity legs (0 = skip)")
    ap.add_argument("--parity-workloads", default="sinusoidal96",
                    help="workloads of the plain-form full-size parity legs besides the benchmarked one")
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
