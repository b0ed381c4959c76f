#!/usr/bin/env python
"""Benchmark: particle-updates/s of the explicit MPM step on one GB300.

Workload: the Taylor-bar impact (3-D TLMPM, MUSL, cubic B-spline, Johnson-Cook
strength + linear EOS, copper bar R = 3.2 mm, L = 32.4 mm at 190 m/s on a rigid
wall, 2x2x2 particles per cell), at cellsize 0.1 mm: 8,354,016 particles and
1,373,125 grid nodes (``--cellsize 0.2``: 1,045,872 and 177,507).  As in the
reference script, one step runs before the wall fix is added; the timed steps
follow.  Inputs are synthetic and deterministic (the populate lattice).
Particle state (~2.9 GB touched per step) is far larger than the 129 MB L2, so
no flush is needed between steps.

The CPU leg (the FP64 oracle on the host cores) runs a bounded sample: a few
steps of the same bar at ``--cpu-cellsize`` (0.2 mm by default, 1/8 of the
particles; its frozen FP64 neighbour lists take ~5 GB there and ~40 GB at
0.1 mm).  Its per-particle cost does not depend on the bar's resolution.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs independent replicas (one per GPU, launched by torchrun); the path
has no data-path collective.  ``--impl reference`` times the CPU
implementation of the step (the oracle port) on the host cores.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-updates/s on 1 GB300: learned/FP32 vs plain GPU, at <=1e-3 rel err"
NETWORK = os.path.join(ROOT, "karamelo_gb300", "data", "taylor_copper_mlp.npz")
UNIT = "particle-updates/s"

# Algorithmic bytes of every phase (FP32 = 4 B): particle fields read or
# written once per pass, plus 4 B per grid value per touched node per access.
# (per particle, per node)
PHASE_BYTES = {
    "p2g": (64, 24),            # x0, v, m, vol0*PK1 -> nodal p, f
    # TLMPM MUSL after a step of the same particle state: the forces only
    # (the momentum is the last re-map's nodal sum)
    "p2g_force": (48, 12),      # x0, vol0*PK1 -> nodal f
    # the velocity scatter where the momentum is not the last re-map's
    "p2g_momentum": (28, 28),   # x0, m, v -> nodal p (kept, 16 B per node)
    "grid_update": (0, 52),     # m, p, f -> v, v_update (+ fixes)
    "g2p_advance": (60, 24),    # x0, u, v -> u, v ; gathers v, v_update
    "p2g_velocity": (28, 12),   # x0, m, v -> nodal p
    # the two above in one pass (MUSL, k_g2p1_remap_row): x0, u, v, m -> u, v;
    # gathers v, v_update and writes nodal p
    "g2p_advance_remap": (64, 36),
    "grid_velocity": (0, 52),   # m, p -> v (+ BC), x += dt v
    "g2p_stress": (200, 12),    # x0, v, F, sigma, eps_p, epsdot, vol0 -> F, sigma, eps_p, epsdot, vol0*PK1
}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() in ("active", "0x1", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_min_mhz": min(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def aggregate_replicas(ms, units, device):
    """Max of the timed milliseconds and sum of the processed units over all
    ranks.  Replicas share no data; this reduction of two scalars after the
    timed region is the only collective."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms), float(units)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def run_cpu_sample(cellsize, steps, time_budget, threads):
    """The oracle (FP64 CPU restatement of the reference step) on the host
    cores, over a bounded number of steps of the same workload.  Step 1
    (which builds the frozen TLMPM neighbour lists) is untimed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from karamelo_gb300 import workloads as W
    orc.lib().om_set_threads(threads)
    sim = W.taylor_bar(lambda s: orc.OracleBackend(s, threads=threads), cellsize=cellsize, method="tlmpm")
    n = sim.s.solids[0].np
    sim.run(1)
    W.taylor_bar_wall(sim)
    done, t0 = 0, time.perf_counter()
    while done < steps:
        sim.run(1)
        done += 1
        if time.perf_counter() - t0 > time_budget:
            break
    dt = time.perf_counter() - t0
    return n * done / dt, n, done, dt


def bench_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    steps = max(1, min(args.steps, args.ref_steps))
    v, n, done, dt = run_cpu_sample(args.cpu_cellsize, steps, args.ref_budget, threads)
    sample = f"{done} steps of the {n}-particle bar (cellsize {args.cpu_cellsize} mm) after the untimed first step"
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": done, "warmup": 1,
            "ms_per_step": 1000 * dt / done, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (populate lattice, deterministic)", "impl": "reference",
            "config": {"workload": f"taylor_bar_tlmpm_musl_cubic_jc h={args.cellsize}mm",
                       "cpu_sample_cellsize_mm": args.cpu_cellsize, "cpu_sample_particles": n},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_ours(args):
    world, rank, local = dist_env()
    import torch
    from karamelo_gb300 import workloads as W
    from karamelo_gb300.gpu import GpuBackend

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    sim = W.taylor_bar(None, cellsize=args.cellsize)
    n = sim.s.solids[0].np
    nn = sim.s.grids[0].nnodes
    sim.backend = GpuBackend(sim.s, precision=args.precision, track_strain=False)
    sim.run(1)
    W.taylor_bar_wall(sim)
    be = sim.backend
    be.run(args.warmup)
    # per-phase device time (CUDA events on the library's stream, eager launches)
    phases = be.profile(args.profile_steps)
    stream = torch.cuda.ExternalStream(be.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks.start()
    time.sleep(0.3)
    e0.record(stream)
    be.run(args.steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    plain_sigma, plain_x = sim.particles(0, "sigma"), sim.particles(0, "x")
    learned = None if args.no_learned else bench_learned(args, be, plain_sigma, plain_x, n, ms)
    islands = None if (args.no_islands or args.precision) else bench_islands(args, plain_sigma, plain_x, n, ms)
    ms, units = aggregate_replicas(ms, n * args.steps, "cuda")
    value = units / (ms / 1000.0)
    launches = be.launches_per_step() * args.steps

    # end to end through the C ABI with host buffers: context creation and the
    # upload of the particle state, the first step and the wall fix, then the
    # timed steps with a dump (x, v, rotated sigma downloaded to host) every
    # 10 steps, as the reference script's set_output(10)
    # the steps are queued without waiting (kmpm_run_async) and the dumps
    # asynchronously into page-locked buffers (two sets, alternating): the
    # host queues ahead while the GPU steps and the copies run beside the
    # next steps; kmpm_sync at the end reports any step's error
    sim2 = W.taylor_bar(None, cellsize=args.cellsize)
    widths = {"x": 3, "v": 3, "sigma6": 6}  # the rotated stress as the reference dump writes it
    pinned = [{f: torch.empty(n * w, dtype=torch.float64, pin_memory=True) for f, w in widths.items()}
              for _ in range(2)]
    for s in pinned:  # the caller's dump buffers, in use before (first touch of page-locked pages)
        for t in s.values():
            t.zero_()
    # the caller's particle arrays in page-locked host memory too: the upload
    # inside the timed region then runs at the link's rate, not at the rate of
    # the driver's staging copy of pageable memory (9-150 GB/s from machine to machine)
    keep = []
    for sol in sim2.s.solids:
        for f in ("x0", "v", "mass", "vol0"):
            a = np.ascontiguousarray(getattr(sol, f), np.float64)
            t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
            t.numpy()[...] = a
            keep.append(t)
            setattr(sol, f, t.numpy())
    # no collector pass inside the timed region: freeing a context there
    # (cudaFree) would synchronise the device in the middle of the steps
    gc.collect()
    gc.disable()
    clocks_e2e = ClockSampler(local)  # started before the timed region
    clocks_e2e.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim2.backend = GpuBackend(sim2.s, precision=args.precision, track_strain=False)
    t_create = time.perf_counter()
    sim2.run(1)
    W.taylor_bar_wall(sim2)
    be2 = sim2.backend
    t_first = time.perf_counter()
    done, dumps, t_runs, t_waits, t_queue = 0, 0, 0.0, 0.0, 0.0
    while done < args.steps:
        k = min(10, args.steps - done)
        a0 = time.perf_counter()
        be2.run_async(k)
        a1 = time.perf_counter()
        done += k
        if dumps >= 2:  # the set about to be reused has landed (the other may still be in flight)
            for t in pinned[dumps % 2].values():
                be2.wait_download(t)
        a2 = time.perf_counter()
        for f in widths:
            be2.particles_async(0, f, pinned[dumps % 2][f])
        dumps += 1
        t_runs, t_waits, t_queue = t_runs + (a1 - a0), t_waits + (a2 - a1), t_queue + (time.perf_counter() - a2)
    t_loop = time.perf_counter()
    be2.sync()
    be2.sync_downloads()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    clk_e2e = clocks_e2e.stop()
    gc.enable()
    e2e_parts = {"create": t_create - t0, "first_step_and_wall": t_first - t_create, "run_calls": t_runs,
                 "download_waits": t_waits, "download_queueing": t_queue, "final_sync": e2e_s - (t_loop - t0)}
    e2e = n * (done + 1) / e2e_s
    h2d = n * (3 + 3 + 3 + 1 + 1) * 8  # x0, x, v, mass, vol0 as FP64 from the caller
    d2h = dumps * n * sum(widths.values()) * 8

    if rank != 0:
        return
    peak, peak_kind = load_peaks()
    dom = max((k for k in phases if k in PHASE_BYTES), key=lambda k: phases[k])
    bp, bn = PHASE_BYTES[dom]
    alg = bp * n + bn * nn
    achieved = alg / (phases[dom] * 1e-3) / 1e9
    step_bytes = sum(PHASE_BYTES[k][0] * n + PHASE_BYTES[k][1] * nn for k in phases if k in PHASE_BYTES)
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            traffic = json.load(f).get(f"taylor_bar h={args.cellsize:g}mm", {}).get(dom)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (populate lattice, deterministic); inputs larger than L2, no flush",
        "config": {"workload": f"taylor_bar_tlmpm_musl_cubic_jc h={args.cellsize}mm", "particles": n, "nodes": nn,
                   "parallelism": f"replicas{world}", "precision": "fp64_islands" if args.precision else "fp32",
                   "graph": "one CUDA graph per step, replayed"},
        "gpu_launches": launches,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d // (done + 1),
                "d2h_bytes_per_step": d2h // (done + 1),
                "note": "C ABI from host FP64 arrays (page-locked): upload + binning + steps queued 10 at a "
                        "time without waiting (kmpm_run_async) + an asynchronous dump (x, v and the six "
                        "components of the rotated stress, FP64, into two alternating sets of page-locked "
                        "buffers, first touched before the timed region) every 10 steps + kmpm_sync, which "
                        "reports any step's error; launch shapes as tuned by the first context of the process",
                "seconds": {k: round(v, 4) for k, v in e2e_parts.items()}, "clocks": clk_e2e},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                     "alg_bytes_per_launch": alg},
        "step_roofline": {"alg_bytes_per_step": step_bytes, "achieved_gbs": step_bytes / (ms / args.steps * 1e-3) / 1e9,
                          "frac": step_bytes / (ms / args.steps * 1e-3) / 1e9 / peak},
        "phases_ms": phases,
        "autotune": be.tuning(),
        "clocks": clk,
    }
    if learned is not None:
        line["learned"] = learned
    if islands is not None:
        line["fp64_islands"] = islands
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, npart, done_c, dtc = run_cpu_sample(args.cpu_cellsize, args.cpu_steps, args.ref_budget, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{done_c} oracle steps of the same bar at cellsize {args.cpu_cellsize} mm "
                                          f"({npart} particles) after its untimed first step"}
    print(json.dumps(line), flush=True)


def bench_islands(args, plain_sigma, plain_x, n, plain_ms):
    """The same bar and steps with the FP64 islands (KMPM_PREC_FP64_ISLANDS:
    nodal sums and v = p/m, det and inverse of F, and the EOS and strength
    update in FP64; the rest FP32): throughput against the plain FP32 path
    and the final state's distance from it."""
    import numpy as np
    import torch
    from karamelo_gb300 import workloads as W
    from karamelo_gb300.gpu import GpuBackend
    sim = W.taylor_bar(None, cellsize=args.cellsize)
    sim.backend = GpuBackend(sim.s, precision=1, track_strain=False)
    sim.run(1)
    W.taylor_bar_wall(sim)
    be = sim.backend
    be.run(args.warmup)
    phases = be.profile(args.profile_steps)  # as the plain arm: same step count before the timed steps
    stream = torch.cuda.ExternalStream(be.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    be.run(args.steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    out = {"value": n * args.steps / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / args.steps,
           "over_plain": plain_ms / ms,
           "rel_l2_sigma_vs_plain": rel(sim.particles(0, "sigma"), plain_sigma),
           "rel_l2_x_vs_plain": rel(sim.particles(0, "x"), plain_x),
           "phases_ms": phases}
    be.close()
    return out


def bench_learned(args, plain_backend, plain_sigma, plain_x, n, plain_ms):
    """The same bar and the same steps with the learned return map
    (kmpm_set_surrogate, residual tolerance 1e-3): throughput, share of
    plastic particle-steps the network answered, and the final stress and bar
    length against the plain FP32 run."""
    import numpy as np
    import torch
    from karamelo_gb300 import workloads as W
    from karamelo_gb300.gpu import GpuBackend
    from karamelo_gb300.surrogate import load_network
    if not os.path.exists(NETWORK):
        return {"unavailable": f"no trained network at {os.path.relpath(NETWORK, ROOT)}"}
    mlp, meta = load_network(NETWORK)
    sim = W.taylor_bar(None, cellsize=args.cellsize)
    sim.backend = GpuBackend(sim.s, precision=args.precision, track_strain=False)
    sim.run(1)
    W.taylor_bar_wall(sim)
    be = sim.backend
    be.set_surrogate(mlp, args.tol)
    be.run(args.warmup)
    be.profile(args.profile_steps)
    stream = torch.cuda.ExternalStream(be.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    be.run(args.steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    st = be.surrogate_stats()
    sig, x = sim.particles(0, "sigma"), sim.particles(0, "x")
    be.close()
    length = lambda a: float(a[:, 0].max() - a[:, 0].min())
    value = n * args.steps / (ms / 1000.0)
    return {"value": value, "unit": UNIT, "ms_per_step": ms / args.steps, "plain_ms_per_step": plain_ms / args.steps,
            "learned_over_plain": (plain_ms / ms), "tol": args.tol,
            "rel_l2_sigma_vs_plain": float(np.linalg.norm(sig - plain_sigma) / np.linalg.norm(plain_sigma)),
            "rel_l2_x_vs_plain": float(np.linalg.norm(x - plain_x) / np.linalg.norm(plain_x)),
            "bar_length_rel_err_vs_plain": abs(length(x) - length(plain_x)) / length(plain_x),
            "plastic_particle_steps": st["plastic"], "served_by_network": st["network"],
            "outside_envelope": st["outside"], "residual_above_tol": st["residual"],
            "network": {"file": os.path.relpath(NETWORK, ROOT), "n_pairs": meta.get("n_pairs"),
                        "train_steps": meta.get("steps"), "holdout_tc_pass": meta.get("tc_pass")},
            "gpu_launches": be.launches_per_step() * args.steps}


def bench_sweep(args):
    """The batched parameter sweep: args.instances
    independent 2-D TLMPM tensile bars (Johnson-Cook + damage, seeded
    parameters) in one launch per phase, particle-updates/s over all."""
    import torch
    from karamelo_gb300.batch import Batch, tensile_sweep
    sims, _ = tensile_sweep(args.instances, seed=0)
    t0 = time.perf_counter()
    batch = Batch(sims, track_strain=False)
    batch.run(1)
    setup_s = time.perf_counter() - t0
    n = batch.total_particles
    be = batch.backend
    be.run(args.warmup)
    phases = be.profile(args.profile_steps)
    stream = torch.cuda.ExternalStream(be.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    e0.record(stream)
    be.run(args.steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    line = {"metric": "particle-updates/s on 1 GB300 (batched TLMPM sweep)", "value": n * args.steps / (ms / 1e3),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seed 0)", "gpu_launches": be.launches_per_step() * args.steps,
            "config": {"workload": f"tensile_sweep_2d_tlmpm_jc_damage instances={args.instances}", "particles": n,
                       "setup_s": setup_s},
            "phases_ms": phases, "autotune": be.tuning(), "clocks": clk}
    print(json.dumps(line), flush=True)


def bench_dam(args):
    """The dam break: 3-D ULMPM, MUSL, cubic B-spline, Tait fluid EOS with
    Newtonian viscosity and gravity, a 0.4 x 0.4 x 0.8 m water column in a
    1.6 x 0.4 x 0.8 m slip-wall box at cellsize 5 mm (8,192,000 particles);
    every step re-bins the particles (key, radix sort, permutation)."""
    import torch
    from karamelo_gb300 import workloads as W
    from karamelo_gb300.gpu import GpuBackend
    sim = W.dam_break(None, cellsize=args.dam_cellsize)
    n = sim.s.solids[0].np
    t0 = time.perf_counter()
    sim.backend = GpuBackend(sim.s, track_strain=False)
    sim.run(1)
    setup_s = time.perf_counter() - t0
    be = sim.backend
    be.run(args.warmup)
    phases = be.profile(args.profile_steps)
    stream = torch.cuda.ExternalStream(be.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    e0.record(stream)
    be.run(args.steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    g = sim.s.grids[0]
    line = {"metric": "particle-updates/s on 1 GB300 (dam break, ULMPM MUSL step)", "value": n * args.steps / (ms / 1e3),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (populate lattice, deterministic)", "gpu_launches": be.launches_per_step() * args.steps,
            "config": {"workload": f"dam_break_ulmpm_musl_cubic_tait h={args.dam_cellsize * 1000:g}mm", "particles": n,
                       "nodes": g.nnodes, "setup_s": setup_s},
            "phases_ms": phases, "autotune": be.tuning(), "clocks": clk}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cellsize", type=float, default=0.1)
    ap.add_argument("--cpu-cellsize", type=float, default=0.2)
    ap.add_argument("--precision", type=int, default=0)
    ap.add_argument("--profile-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--ref-steps", type=int, default=5)
    ap.add_argument("--ref-budget", type=float, default=60.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="taylor", choices=["taylor", "sweep", "dam"])
    ap.add_argument("--dam-cellsize", type=float, default=0.005)
    ap.add_argument("--instances", type=int, default=1024)
    ap.add_argument("--tol", type=float, default=1e-3)
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-islands", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        bench_reference(args)
    elif args.workload == "sweep":
        bench_sweep(args)
    elif args.workload == "dam":
        bench_dam(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
