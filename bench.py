"""Benchmark of the electrostatic PIC cycle (particle-steps/s).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl cupic|reference]

One "step" is one full cycle (Jacobi solve + field, push + binning +
deposition, injection) of the 512x2048-cell, 100-particles-per-cell
workload (about 2.1e8 particles).  Rank 0 prints one JSON line.

value      device time of K steps (CUDA events on the library's stream, inputs
           resident in HBM); particle arrays (3.4 GB) are far larger than L2
e2e        the same K steps through the public C-ABI from pinned host
           buffers: upload of both species (the reference's 4-double particle
           struct), K graph-launched steps each followed by a read of the
           step's counters, download of both species at the end
roofline   the dominant kernel's algorithmic bytes per launch / its mean
           event-timed duration, against the measured HBM copy bandwidth
cpu_baseline  the CPU oracle (the reference algorithm restated, FP64,
           OpenMP) on a strip of the same workload, rank 0 only
--impl reference  the same CPU oracle as the timed arm on the same metric
batched, serving, precision  (default run, N = 1) the other forms on the same
           GPU: 256 probe-bias instances stepped together against one at a
           time; a 32-request Poisson stream at 100/s served by continuous
           batching against one at a time (solves/s, p50, p99); the
           precision form of the workload

For N > 1 (torchrun), every rank runs an independent replica on its own GPU
(no collective on the data path); value sums particle-steps over ranks and
divides by the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s full PIC cycle"
UNIT = "particle-steps/s"
STATS_BYTES = 96
# kernels launched per step: jacobi (which also clears the next charge),
# push, room check, arrive, inject sched/gen/append, finalize
KERNELS_PER_STEP = 8


def kernels_per_step(p):
    """Kernels one step launches.  The precision form replaces the solve by
    the FP64 source, one Jacobi launch per correction up to the sweep cap
    (each with the residual, the stop test and the update fused in; the
    ones after the stop test return at once), a last test launch and the
    field; its step also clears the next charge with its own kernel."""
    if p.refine_every <= 0:
        return KERNELS_PER_STEP
    corrections = -(-max(p.max_sweeps, 0) // p.refine_every)
    return (KERNELS_PER_STEP - 1) + 1 + 1 + corrections + 1 + 1

# algorithmic bytes per unit of work (FP32 SoA, 16 B state per particle)
PUSH_BYTES_PER_PARTICLE = 32      # 16 B read + 16 B write
PUSH_BYTES_PER_NODE = 16          # E read once (8 B) + int64 charge flush (8 B)
JACOBI_BYTES_PER_NODE_SWEEP = 12  # phi read, source read, phi write


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["cupic", "reference"], default="cupic")
    ap.add_argument("--workload", choices=["large", "precision", "small", "tiny", "batched", "serving"],
                    default="large")
    ap.add_argument("--instances", type=int, default=256,
                    help="batched: probe-bias instances (sizes drawn from seed 2)")
    ap.add_argument("--requests", type=int, default=32, help="serving: requests in the stream")
    ap.add_argument("--rate", type=float, default=100.0, help="serving: Poisson arrivals per second")
    ap.add_argument("--solve-steps", type=int, default=300, help="serving: steps per request")
    ap.add_argument("--sweeps", type=int, default=200,
                    help="batched and serving: Jacobi sweeps per step of every instance")
    ap.add_argument("--no-plain", action="store_true", help="batched: skip the one-at-a-time run")
    ap.add_argument("--no-forms", action="store_true",
                    help="large: leave out the batched, serving and precision sub-objects")
    ap.add_argument("--form-steps", type=int, default=10,
                    help="large: timed steps of the batched and precision sub-objects")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ncy", type=int, default=0,
                    help="override the y cell count (smaller cases for profiling)")
    ap.add_argument("--ppc", type=float, default=0,
                    help="override particles per cell per species (profiling the mesh solve)")
    ap.add_argument("--cpu-rows", type=int, default=0,
                    help="rows of the CPU sample strip (0: sized to ~1 s per step)")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def allmax(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def workload_desc(p):
    ppc = p.ppr // p.ncx
    return (f"{p.ncx}x{p.ncy} cells, ds={p.ds}, {ppc} particles per cell per species, "
            f"mi/me={p.mi:g}, Ti/Te={p.kti:g}, phi_p={p.phi_p:g}, dt={p.dt:g}, "
            f"Jacobi {p.min_sweeps}-{p.max_sweeps} sweeps" +
            (f" to an FP64 residual of {p.tol:g} (correction every {p.refine_every})"
             if p.refine_every else "") + f", seed {p.seed}")


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel, units):
    """dram bytes per launch of `kernel` scaled to `units`, from the committed
    ncu summary (profiles/ncu_traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    k = d.get(kernel)
    if not k:
        return None
    return float(k["dram_bytes_per_unit"]) * units


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        rows = []
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]) if f[3] not in ("", "[N/A]") else 0.0,
                             f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        pmax = max(r[2] for r in rows)
        load = [r for r in rows if r[2] >= 0.5 * pmax] or rows
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in load:
            for name, v in zip(names, r[3:]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "samples_under_load": len(load),
                "power_w_max": pmax, "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU oracle (the reference algorithm restated) on a strip of the workload
# ---------------------------------------------------------------------------

def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), or None."""
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return None


def cpu_strip(p, rows_req, steps, warmup, target_s=1.0, threads=None):
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    O.set_threads(threads)
    rows = rows_req
    if rows <= 0:
        # size the strip so one step takes about target_s on this host
        probe = p.copy()
        probe.ncy = 16
        probe.finalize()
        o = O.Oracle(probe, fp64=True)
        o.init_plasma()
        t0 = time.perf_counter()
        o.step(1)
        dt = time.perf_counter() - t0
        o.close()
        rows = int(max(16, min(p.ncy, 16 * target_s / max(dt, 1e-4))))
    q = p.copy()
    q.ncy = rows
    q.finalize()
    o = O.Oracle(q, fp64=True)
    o.init_plasma()
    if warmup:
        o.step(warmup)
    n0 = sum(o.counts())
    t0 = time.perf_counter()
    o.step(steps)
    el = time.perf_counter() - t0
    n1 = sum(o.counts())
    ps = 0.5 * (n0 + n1) * steps
    sample = (f"FP64 oracle, {q.ncx}x{rows}-row strip of the workload ({n0} particles, "
              f"{q.max_sweeps} Jacobi sweeps per step), {steps} steps after {warmup} warm-up")
    return {"value": ps / el, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
            "seconds": el}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    p = make_params(args)
    cb = cpu_strip(p, args.cpu_rows, args.steps, args.warmup)
    # one thread on a small strip for a few steps, beside the all-core figure
    one = cpu_strip(p, 64, 2, 1, threads=1)
    line = {
        "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * cb["seconds"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded uniform/Maxwellian plasma (Philox4x32-10)",
        "config": {"workload": workload_desc(p), "sample": cb["sample"], "parallelism": "cpu"},
        "impl": "reference",
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "cpu": {"model": cpu_model(), "nproc": os.cpu_count(),
                "single_thread": {"value": one["value"], "unit": UNIT, "sample": one["sample"]}},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def pinned_f64(n):
    try:
        import torch
        t = torch.empty((max(n, 1), 4), dtype=torch.float64, pin_memory=True)
        return t.numpy(), True
    except Exception:
        import numpy as np
        return np.empty((max(n, 1), 4), dtype=np.float64), False


def run_e2e(sim, steps, pinned_state):
    """K steps through the public C-ABI from and back to host buffers."""
    import ctypes

    import cupic_gb300 as cg
    L = sim.L
    bufs, ns = pinned_state
    t, tin = sim.get_time()[1], sim.get_time()[2:]
    step0 = sim.get_time()[0]
    stats = (cg.StepStats * 1)()
    h2d = sum(ns) * 32
    t0 = time.perf_counter()
    for sp in (0, 1):
        rc = L.cupic_load_particles(sim.h, sp, bufs[sp].ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    ns[sp])
        if rc:
            raise cg.CupicError(rc, "load")
    for _ in range(steps):
        rc = L.cupic_step(sim.h, 1)
        rc = rc or L.cupic_get_stats(sim.h, stats, 1)
        if rc:
            raise cg.CupicError(rc, "step")
    got = [ctypes.c_int64(), ctypes.c_int64()]
    out = 0
    for sp in (0, 1):
        rc = L.cupic_store_particles(sim.h, sp, bufs[sp].ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     bufs[sp].shape[0], ctypes.byref(got[sp]))
        if rc:
            raise cg.CupicError(rc, "store")
        out += got[sp].value * 32
    el = time.perf_counter() - t0
    return el, h2d, out + steps * STATS_BYTES


def make_params(args):
    from cupic_gb300 import workload_params
    p = workload_params(args.workload)
    if args.ncy:
        p.ncy = args.ncy
    if args.ppc:
        p.n = args.ppc / p.ds ** 3
        p.eps0 = p.n
    p.finalize()
    return p


def run_cupic(args, world, rank, local):
    import cupic_gb300 as cg
    p = make_params(args)
    sim = cg.Sim(p, device=local)
    sim.init_plasma()
    if args.warmup:
        sim.step(args.warmup)
    nodes = p.nnx * p.nny
    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    total_ms, phases = sim.step_timed(args.steps)
    barrier(world)
    clocks = sampler.stop()
    st = sim.stats(args.steps)
    flags = 0
    for s in st:
        flags |= s["flags"]
    live = [sum(s["live"]) for s in st]
    before = [sum(st[0]["live"]) - st[0]["injected"][0] - st[0]["injected"][1]
              + sum(st[0]["absorbed"]) + sum(st[0]["removed"])] + live[:-1]
    pstep = float(sum(before))
    tmax = allmax(total_ms / 1e3, world)
    ps_all = allsum(pstep, world)
    value = ps_all / tmax
    mean_particles = pstep / args.steps
    sweeps = [s["sweeps"] for s in st]

    peak, peak_kind = measured_peaks()
    push_ms = phases["push"] / args.steps
    solve_ms = phases["solve"] / args.steps
    push_bytes = PUSH_BYTES_PER_PARTICLE * mean_particles + PUSH_BYTES_PER_NODE * nodes
    jac_bytes = JACOBI_BYTES_PER_NODE_SWEEP * nodes * statistics.mean(sweeps)
    push_gbs = push_bytes / (push_ms * 1e-3) / 1e9
    jac_gbs = jac_bytes / (solve_ms * 1e-3) / 1e9
    roof_push = {"kernel": "k_push_deposit", "bound": "hbm", "achieved": push_gbs, "peak": peak,
                 "unit": "GB/s", "frac": push_gbs / peak, "peak_source": peak_kind,
                 "traffic": ncu_traffic("k_push_deposit", mean_particles),
                 "algorithmic_bytes": push_bytes, "mean_ms": push_ms}
    roof_jac = {"kernel": "k_jacobi", "bound": "hbm", "achieved": jac_gbs, "peak": peak,
                "unit": "GB/s", "frac": jac_gbs / peak, "peak_source": peak_kind,
                "traffic": ncu_traffic("k_jacobi", nodes),
                "algorithmic_bytes": jac_bytes, "mean_ms": solve_ms,
                "note": "12 B/node/sweep counted per sweep; the mesh stays on chip"}
    dominant, other = (roof_push, roof_jac) if push_ms >= solve_ms else (roof_jac, roof_push)

    e2e = None
    if not args.no_e2e:
        ns = sim.counts()
        bufs = []
        pinned = True
        for sp in (0, 1):
            b, pin = pinned_f64(ns[sp])
            pinned = pinned and pin
            bufs.append(b)
            # the state to upload: the current one, as the reference's struct
            import ctypes
            got = ctypes.c_int64()
            sim.L.cupic_store_particles(sim.h, sp, b.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                        b.shape[0], ctypes.byref(got))
        barrier(world)
        el, h2d, d2h = run_e2e(sim, args.steps, (bufs, ns))
        el = allmax(el, world)
        e2e_ps = allsum(float(sum(ns)) * args.steps, world)
        e2e = {"value": e2e_ps / el, "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
               "d2h_bytes_per_step": d2h / args.steps, "pinned_host": pinned,
               "seconds": el}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_strip(p, args.cpu_rows, steps=8, warmup=1, target_s=1.5)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    plan = dict(zip(("ctas", "rows_per_cta", "halo_depth"), sim.solver_plan()))
    sim.close()
    forms = {}
    if rank == 0 and world == 1 and args.workload == "large" and not args.no_forms \
            and not args.ncy and not args.ppc:
        # the second half of the metric: bias-point solves/s and p50/p99
        # against the plain one-at-a-time method on the same GPU
        forms["batched"] = bench_batched(256, 200, args.form_steps, args.warmup, local)
        forms["serving"] = bench_serving(32, 100.0, 300, 200, local)
        forms["precision"] = bench_precision(args.form_steps, 1, local)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tmax * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if not p.refine_every else
                     f"f32 sweeps, f64 residual and correction every {p.refine_every} sweeps",
            "data": "synthetic: seeded uniform positions, Maxwellian velocities (Philox4x32-10)",
            "config": {"workload": workload_desc(p), "ncx": p.ncx, "ncy": p.ncy,
                       "particles_per_step": mean_particles, "nodes": nodes,
                       "jacobi_sweeps": statistics.mean(sweeps),
                       "l2": "inputs larger than L2 (particle arrays 3.4 GB); the 4 MB mesh "
                             "stays L2/shared-memory resident by design",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "jacobi_plan": plan},
            "e2e": e2e,
            "gpu_launches": kernels_per_step(p) * args.steps,
            "roofline": dominant,
            "roofline_other": other,
            "phases_ms_per_step": {k: v / args.steps for k, v in phases.items()},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "device_flags": flags,
        }
        line.update(forms)
        print(json.dumps(line), flush=True)
    return 0


def bench_batched(instances, sweeps, k, warmup, local, plain_run=True):
    """The batched form: probe-bias instances of uneven sizes stepped
    together, against the same instances stepped one at a time (each its own
    graph, one after another).  Both runs start from the same initial
    states and take the same steps, so every instance's results must be
    identical; the line says whether they are."""
    import numpy as np

    import cupic_gb300 as cg
    from cupic_gb300.params import bias_instances
    ps = bias_instances(instances, seed=2, sweeps=sweeps)

    def make():
        out = []
        for p in ps:
            s = cg.Sim(p, device=local)
            s.init_plasma()
            out.append(s)
        return out

    sims = make()
    parts = float(sum(sum(s.counts()) for s in sims))
    plain_s = float("nan")
    same = None
    if plain_run:
        alone = make()
        for s in alone:
            s.step(warmup)
        t0 = time.perf_counter()
        for s in alone:
            s.step(k)
        plain_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = cg.Batch(sims, device=local)  # builds the arrays, tunes the solve layout
    build_s = time.perf_counter() - t0
    layout = dict(zip(("depth_cap", "cta_mult", "ctas"), b.plan()))
    b.step(warmup)
    sampler = ClockSampler(local)
    sampler.start()
    t0 = time.perf_counter()
    b.step(k)
    batch_s = time.perf_counter() - t0
    clocks = sampler.stop()
    if plain_run:
        same = all(np.array_equal(a.phi(), m.phi()) and a.stats(k) == m.stats(k)
                   and all(np.array_equal(a.particles(sp), m.particles(sp)) for sp in (0, 1))
                   for a, m in zip(alone, sims))
        for s in alone:
            s.close()
    n = len(sims)
    line = {
        "metric": "instance-steps/s, probe-bias instances of uneven sizes (batched form)",
        "value": n * k / batch_s, "unit": "instance-steps/s", "n_gpus": 1, "steps": k,
        "warmup": warmup, "ms_per_step": 1e3 * batch_s / k, "higher_is_better": True,
        "particle_steps_per_s": parts * k / batch_s,
        "plain": {"value": n * k / plain_s, "particle_steps_per_s": parts * k / plain_s,
                  "ms_per_step_all_instances": 1e3 * plain_s / k},
        "speedup_vs_plain": plain_s / batch_s, "results_identical_to_plain": same,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n} instances: Nx in {{32,64,128,256}}, Ny=4Nx, 10-50 particles "
                               f"per cell per species, phi_p in [-10,2], mi/me=1836, Ti/Te=0.1, "
                               f"{sweeps} Jacobi sweeps, seeds from 2",
                   "particles": parts, "cells": sum(p.ncx * p.ncy for p in ps),
                   "solve_layout": layout, "build_and_tune_s": build_s,
                   "timing": "host wall clock around k batched steps (one graph launch per "
                             "step, synchronised at the end) and around the k steps of every "
                             "instance stepped alone"},
        "clocks": clocks,
    }
    b.close()
    for s in sims:
        s.close()
    return line


def run_batched(args, local):
    line = bench_batched(args.instances, args.sweeps, args.steps, args.warmup, local,
                         plain_run=not args.no_plain)
    print(json.dumps(line), flush=True)
    return 0


def bench_serving(requests, rate, solve_steps, sweeps, local):
    """The serving loop against the plain one-at-a-time method on the same
    Poisson request stream; every result must be identical."""
    import copy
    from cupic_gb300 import serve
    from cupic_gb300.params import bias_instances
    ps = bias_instances(requests, seed=3, sweeps=sweeps)
    t = serve.poisson_arrivals(requests, rate, seed=3)
    reqs = [serve.Request(k, p, float(t[k]), steps=solve_steps,
                          window=min(1000, solve_steps // 2)) for k, p in enumerate(ps)]
    plain = serve.serve_plain(copy.deepcopy(reqs), device=local)
    sampler = ClockSampler(local)
    sampler.start()
    mixed = serve.serve_batched(copy.deepcopy(reqs), device=local)
    clocks = sampler.stop()
    sp, sm = serve.summary(plain), serve.summary(mixed)
    same = all(a.current == b.current for a, b in
               zip(sorted(plain, key=lambda r: r.rid), sorted(mixed, key=lambda r: r.rid)))
    line = {
        "metric": "bias-point solves/s (continuous batching)", "value": sm["solves_per_s"],
        "unit": "solves/s", "n_gpus": 1, "higher_is_better": True,
        "p50_ms": sm["p50_ms"], "p99_ms": sm["p99_ms"], "failed": sm["failed"],
        "plain": sp, "speedup_vs_plain": sm["solves_per_s"] / max(sp["solves_per_s"], 1e-30),
        "results_identical_to_plain": same, "dtype": "f32", "data": "synthetic",
        "config": {"requests": requests, "rate_per_s": rate,
                   "steps_per_request": solve_steps, "window": reqs[0].window,
                   "jacobi_sweeps_per_step": sweeps,
                   "sizes": "Nx in {32,64,128,256}, Ny=4Nx, 10-50 ppc, phi_p in [-10,2]",
                   "admission": "16 B per particle + 12 B per cell within 96 GiB"},
        "clocks": clocks,
    }
    return line


def run_serving(args, local):
    line = bench_serving(args.requests, args.rate, args.solve_steps, args.sweeps, local)
    print(json.dumps(line), flush=True)
    return 0


def bench_precision(k, warmup, local):
    """The precision form of the 512x2048 workload: FP32 sweeps on a
    correction, an FP64 residual and update every 32 sweeps, to an FP64
    residual of 1e-10 or 2000 sweeps a step."""
    import cupic_gb300 as cg
    p = cg.workload_params("precision")
    sim = cg.Sim(p, device=local)
    sim.init_plasma()
    sim.step(warmup)
    sampler = ClockSampler(local)
    sampler.start()
    total_ms, phases = sim.step_timed(k)
    clocks = sampler.stop()
    st = sim.stats(k)
    parts = float(sum(sum(s["live"]) for s in st)) / k
    line = {"metric": METRIC, "value": parts * k / (total_ms / 1e3), "unit": UNIT, "steps": k,
            "warmup": warmup, "ms_per_step": total_ms / k,
            "solve_ms_per_step": phases["solve"] / k,
            "sweeps_per_step": statistics.mean(s["sweeps"] for s in st),
            "last_residual": st[-1]["residual"],
            "dtype": "f32 sweeps, f64 residual and correction every 32 sweeps",
            "config": {"workload": workload_desc(p)},
            "error_vs_fp64": "tests/test_gpu_fp64_contract.py prints it",
            "clocks": clocks}
    sim.close()
    return line


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.workload == "batched":
        return run_batched(args, local) if rank == 0 else 0
    if args.workload == "serving":
        return run_serving(args, local) if rank == 0 else 0
    return run_cupic(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
