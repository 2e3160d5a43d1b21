"""Benchmark of the per-particle nuclear burn on GB300.

One step = one burn of the whole workload over its hydro step, through the library's
C ABI, starting from the same seeded state every step (the state is restored from a
pristine HBM copy inside the timed region).  Default workload: net86 + Helmholtz EOS,
1,048,576 particles (rho log-uniform [1e6, 5e9], T log-uniform [5e8, 6e9], 0.3 12C /
0.7 16O with a 1e-10 floor, hydro dt 1e-4 s).  Metric: particle-burns/s (particles
carried through one hydro step per second of wall time).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--solver mixed|sparse|dense]
                  [--particles P] [--impl reference]

Under torchrun each rank burns its own seeded shard of P particles (weak scaling, no
collective on the data path); the step time is the max over ranks.  --strong splits one set
of P particles over the ranks in contiguous ranges of equal predicted cost (the previous
burn's Newton iterations per particle, exchanged once on the host).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "sph-exa-nnet_gb300")
for p in (os.path.join(PKG, "data"), PKG):
    sys.path.insert(0, p)

METRIC = "net86 particle-burns/s on 1 GB300, plain vs batched+FP32-LU @1e-8; p50/p99 latency"
UNIT = "particle-burns/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--solver", default=None)
    ap.add_argument("--particles", type=int, default=1048576)
    ap.add_argument("--plain-particles", type=int, default=4096,
                    help="particles of the plain FP64 comparison leg (0 disables it)")
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--cpu-sample", type=int, default=32768)
    ap.add_argument("--max-iter", type=int, default=20000)
    ap.add_argument("--serve-requests", type=int, default=48,
                    help="requests of the served-stream leg (0 disables it)")
    ap.add_argument("--serve-plain-requests", type=int, default=8,
                    help="requests of the plain-FP64 served-stream comparison (0 disables it)")
    ap.add_argument("--no-graph", action="store_true", help="launch the timed steps eagerly")
    ap.add_argument("--workload", default="c2",
                    help="c2 (default line), or c1 / c3 / c4 for the other configurations (one GPU)")
    ap.add_argument("--no-mixed-leg", action="store_true", help="skip the FP32-LU (mixed) leg of the c2 line")
    ap.add_argument("--no-fused-leg", action="store_true", help="skip the fused post-burn EOS leg of the c2 line")
    ap.add_argument("--strong", action="store_true",
                    help="N > 1: split ONE set of --particles particles over the ranks by cost-balanced contiguous "
                         "ranges (strong scaling) instead of one shard of --particles per rank (weak scaling)")
    return ap.parse_args()


def shard_seed(rank):
    """Seed of this rank's shard of the c2 workload (weak scaling: independent particles)."""
    return 2 + 1000 * rank


def max_over_ranks(ms, world, device="cpu"):
    """Step time of the job: the maximum over ranks (the only collective of the bench)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_info():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.proc = gpu, None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- reference (CPU) arm
def _oracle():
    """The oracle restatement of the reference's CPU path, built with the compiler line
    oracle/build.py reports (test infrastructure: used only as the timed baseline and checker)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(REPO, "oracle", "build.py"))
    ob = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ob)
    ob.build_oracle()
    import oracle
    import nnet_build
    o = oracle.Oracle("port")
    o.load_helmholtz(np.fromfile(nnet_build.helm_table(), dtype="<f8"))
    return o, oracle, ob.CPU_FLAGS


def status_summary(status, substeps, iterations, seconds):
    """Counts per status, throughput over completed (OK) particles, and p50 / p99 of the
    substeps and Newton iterations per particle."""
    names = ["OK", "SKIPPED", "LIVELOCK", "MAXITER", "ZERO_DT", "ABORTED"]
    counts = np.bincount(np.asarray(status, dtype=np.int64), minlength=len(names))
    it, sub = np.asarray(iterations), np.asarray(substeps)
    return {"status_counts": dict(zip(names, [int(c) for c in counts])),
            "completed_value": float(counts[0] / seconds),
            "substeps_p50": float(np.percentile(sub, 50)), "substeps_p99": float(np.percentile(sub, 99)),
            "iterations_p50": float(np.percentile(it, 50)), "iterations_p99": float(np.percentile(it, 99)),
            "iterations_max": int(it.max()) if it.size else 0}


def cpu_burn(o, w, sl, threads=0):
    """Burn particles `sl` of workload `w` with the oracle on the host cores (OpenMP dynamic
    schedule, as parallel_nuclear_net_impl.cpp:79-81); returns (seconds, threads, outputs)."""
    threads = threads or os.cpu_count()
    t0 = time.perf_counter()
    out = o.burn(w["net"], w["Y"][:, sl], w["T"][sl], w["rho"][sl], w["dt"][sl], w["hydro_dt"], w["eos"], w["mu"],
                 max_iter=20000, nthreads=threads)
    return time.perf_counter() - t0, threads, out


def run_reference(args):
    """The reference's CPU path (the oracle restatement, bit-identical to the reference compiled
    from its sources) on the machine's host cores: step k burns particles [k S, (k + 1) S) of the
    timed c2 set (S = --cpu-sample), so the steps walk through the particles the GPU arm burns."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import workloads
    o, _, flags = _oracle()
    w = workloads.make("c2", P=args.particles, seed=shard_seed(0))
    S = min(args.cpu_sample, args.particles)
    nslices = max(1, args.particles // S)
    cpu_burn(o, w, slice(0, 256))  # warm-up (thread pool, page-in)
    vals, outs = [], []
    for k in range(args.steps):
        a = (k % nslices) * S
        el, threads, out = cpu_burn(o, w, slice(a, a + S))
        vals.append(el)
        outs.append(out)
    value = statistics.median(S / e for e in vals)
    st = np.concatenate([x[3] for x in outs])
    summ = status_summary(st, np.concatenate([x[4] for x in outs]), np.concatenate([x[5] for x in outs]), sum(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(vals) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded, workload c2 distributions)",
            "config": {"workload": "net86+helmholtz c2 (CPU sample)", "particles_per_step": S, "hydro_dt": 1e-4,
                       "value_counts": "every particle carried through the call (any final status); "
                                       "completed_value counts status OK only",
                       **{k: v for k, v in summ.items() if k != "completed_value"}},
            "completed_value": summ["completed_value"],
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "build": flags,
                             "sample": f"step k: particles [k*{S}, (k+1)*{S}) of the timed c2 set"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm
def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import torch.distributed as dist
    import nnet_gb300 as nn
    import workloads

    rank, world, local = dist_info()
    if args.workload != "c2":
        if rank == 0:
            run_workload(args)
        return
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = nn.Context(local)
    solver = args.solver or "sparse"
    sv = nn.SOLVERS[solver]

    # ---- device-resident workload (this rank's shard)
    partition = None
    if args.strong and world > 1:
        w, partition = strong_shard(args, ctx, rank, world, dev)
    else:
        w = workloads.make("c2", P=args.particles, seed=shard_seed(rank))
    P = w["T"].size
    P_job = args.particles if partition else world * P
    Y0 = torch.tensor(w["Y"], device=dev)
    T0 = torch.tensor(w["T"], device=dev)
    rho = torch.tensor(w["rho"], device=dev)
    dt0 = torch.tensor(w["dt"], device=dev)
    Y, T, dt = torch.empty_like(Y0), torch.empty_like(T0), torch.empty_like(dt0)
    status = torch.empty(P, dtype=torch.int32, device=dev)
    substeps = torch.empty(P, dtype=torch.int32, device=dev)
    iterations = torch.empty(P, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def restore():
        Y.copy_(Y0), T.copy_(T0), dt.copy_(dt0)

    def step(st=None, sv_=sv, **kw):
        restore()
        ctx.burn(86, Y, T, rho, dt, w["hydro_dt"], eos=nn.EOS_HELMHOLTZ, solver=sv_, status=status,
                 substeps=substeps, iterations=iterations, max_iter=args.max_iter, stream=st or stream, **kw)

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    stats = ctx.stats()
    # one step (state restore + burn) captured in a CUDA graph and replayed per timed step
    graph, launch = None, "eager"
    if not args.no_graph:
        try:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                step(torch.cuda.current_stream(dev))
            graph, launch = g, "cuda-graph"
        except Exception as e:  # the eager launch path stays available
            launch = f"eager (graph capture failed: {e})"
        barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kt = []
    with ClockSampler(local) as clk:
        barrier()
        t0 = time.perf_counter()
        ev0.record(stream)
        for _ in range(args.steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            if graph is not None:
                graph.replay()
            else:
                step()
            b.record(stream)
            kt.append((a, b))
        ev1.record(stream)
        barrier()
        wall = time.perf_counter() - t0
    ms = ev0.elapsed_time(ev1) / args.steps
    kernel_ms = statistics.mean(a.elapsed_time(b) for a, b in kt)
    ms = max_over_ranks(ms, world, dev)
    value = P_job / (ms / 1e3)
    # every timed step burns the same state: the last one's per-particle results
    S = min(args.cpu_sample, P)
    res_fast = (Y[:, :S].cpu().numpy(), T[:S].cpu().numpy(), dt[:S].cpu().numpy(), status[:S].cpu().numpy())
    summ = status_summary(status.cpu().numpy(), substeps.cpu().numpy(), iterations.cpu().numpy(), ms / 1e3)

    # ---- end to end through the public API with host buffers
    Yh = torch.tensor(w["Y"]).pin_memory()
    Th, dth, rhoh = torch.tensor(w["T"]).pin_memory(), torch.tensor(w["dt"]).pin_memory(), torch.tensor(
        w["rho"]).pin_memory()
    Yo, To, dto = torch.empty_like(Yh).pin_memory(), torch.empty_like(Th).pin_memory(), torch.empty_like(
        dth).pin_memory()
    rho_d = torch.empty_like(rho)
    e2e_steps = max(1, min(args.steps, 2))
    # one untimed pass of every copy: the first transfer through a freshly pinned buffer pays a
    # one-time mapping cost that an application reusing its buffers pays once
    Y.copy_(Yh, non_blocking=True), T.copy_(Th, non_blocking=True), dt.copy_(dth, non_blocking=True)
    rho_d.copy_(rhoh, non_blocking=True)
    Yo.copy_(Y, non_blocking=True), To.copy_(T, non_blocking=True), dto.copy_(dt, non_blocking=True)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # per step: before the host -> device copies, after them, after the burn, after the copies back
    marks = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(e2e_steps)]
    e0.record(stream)
    for k in range(e2e_steps):
        marks[k][0].record(stream)
        Y.copy_(Yh, non_blocking=True), T.copy_(Th, non_blocking=True), dt.copy_(dth, non_blocking=True)
        rho_d.copy_(rhoh, non_blocking=True)
        marks[k][1].record(stream)
        ctx.burn(86, Y, T, rho_d, dt, w["hydro_dt"], eos=nn.EOS_HELMHOLTZ, solver=sv, status=status,
                 max_iter=args.max_iter, stream=stream)
        marks[k][2].record(stream)
        Yo.copy_(Y, non_blocking=True), To.copy_(T, non_blocking=True), dto.copy_(dt, non_blocking=True)
        marks[k][3].record(stream)
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    e2e_split = {name: statistics.mean(m[q].elapsed_time(m[q + 1]) for m in marks)
                 for q, name in enumerate(("h2d_ms", "burn_ms", "d2h_ms"))}
    h2d = (86 + 3) * 8 * P
    d2h = (86 + 2) * 8 * P

    # ---- the mixed-precision form (FP32 LU, FP64 residual refinement) on the same particles
    mixed = None
    if not args.no_mixed_leg and solver != "mixed" and rank == 0:
        step(sv_=nn.SOLVER_MIXED)  # warm-up: module load
        barrier()
        m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        restore()
        m0.record(stream)
        ctx.burn(86, Y, T, rho, dt, w["hydro_dt"], eos=nn.EOS_HELMHOLTZ, solver=nn.SOLVER_MIXED, status=status,
                 substeps=substeps, iterations=iterations, max_iter=args.max_iter, stream=stream)
        m1.record(stream)
        barrier()
        mms = m0.elapsed_time(m1)
        mst = ctx.stats()
        res_mixed = (Y[:, :S].cpu().numpy(), T[:S].cpu().numpy(), dt[:S].cpu().numpy(), status[:S].cpu().numpy())
        mixed = {"value": P / (mms / 1e3), "unit": UNIT, "ms_per_step": mms, "steps": 1,
                 "newton_iterations": mst["newton_iterations"], "refinement_steps": mst["refinement_steps"],
                 "fp64_fallbacks": mst["fp64_fallbacks"],
                 "fp64_fallback_frac": mst["fp64_fallbacks"] / max(1, mst["newton_iterations"]),
                 **status_summary(status.cpu().numpy(), substeps.cpu().numpy(), iterations.cpu().numpy(), mms / 1e3)}

    # ---- post-burn steps fused into the burn (normalisation + drift + Helmholtz EOS) against
    #      the burn followed by the stand-alone EOS kernel (nnet_helmholtz_eos)
    fused = None
    if not args.no_fused_leg and rank == 0:
        outs = [torch.empty(P, dtype=torch.float64, device=dev) for _ in range(5)]
        drift = torch.empty(P, dtype=torch.float64, device=dev)
        Z = nn.network_charges(86)
        q = slice(0, 1024)
        Y[:, q].copy_(Y0[:, q]), T[q].copy_(T0[q]), dt[q].copy_(dt0[q])
        ctx.burn(86, Y[:, q], T[q], rho[q], dt[q], w["hydro_dt"], eos=nn.EOS_HELMHOLTZ, solver=sv,
                 max_iter=args.max_iter, normalize_mass=True, mass_drift=drift[q], eos_out=[o[q] for o in outs],
                 stream=stream)  # warm-up: module load
        ctx.helmholtz_eos(Z, T, rho, Y, *outs, stream=stream)
        barrier()
        f0, f1, f2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        restore()
        f0.record(stream)
        ctx.burn(86, Y, T, rho, dt, w["hydro_dt"], eos=nn.EOS_HELMHOLTZ, solver=sv, max_iter=args.max_iter,
                 normalize_mass=True, mass_drift=drift, eos_out=outs, stream=stream)
        f1.record(stream)
        ctx.helmholtz_eos(Z, T, rho, Y, *outs, stream=stream)  # the separate pass, on the same state
        f2.record(stream)
        barrier()
        A = torch.tensor(workloads.mass_numbers(86)[:86], dtype=torch.float64, device=dev)[:, None]
        sum_err = ((A * Y).sum(0) - 1).abs().max().item()
        fused = {"fused_ms": f0.elapsed_time(f1), "separate_eos_ms": f1.elapsed_time(f2),
                 "burn_then_eos_ms": kernel_ms + f1.elapsed_time(f2),
                 "max_abs_sum_x_minus_1_after": sum_err, "max_abs_drift_before": drift.abs().max().item()}

    # ---- plain FP64 form on a sub-batch, for the plain-vs-fast ratio
    plain = None
    if args.plain_particles and solver != "dense":
        Pp = min(args.plain_particles, P)
        sl = slice(0, Pp)
        Y[:, sl].copy_(Y0[:, sl]), T[sl].copy_(T0[sl]), dt[sl].copy_(dt0[sl])
        ctx.burn(86, Y[:, sl], T[sl], rho[sl], dt[sl], w["hydro_dt"], eos=nn.EOS_HELMHOLTZ,
                 solver=nn.SOLVER_DENSE_FP64, max_iter=args.max_iter, stream=stream)
        barrier()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        Y[:, sl].copy_(Y0[:, sl]), T[sl].copy_(T0[sl]), dt[sl].copy_(dt0[sl])
        p0.record(stream)
        ctx.burn(86, Y[:, sl], T[sl], rho[sl], dt[sl], w["hydro_dt"], eos=nn.EOS_HELMHOLTZ,
                 solver=nn.SOLVER_DENSE_FP64, max_iter=args.max_iter, stream=stream)
        p1.record(stream)
        barrier()
        plain = {"value": Pp / (p0.elapsed_time(p1) / 1e3), "unit": UNIT, "particles": Pp}
        # the fast form on the same sub-batch (same occupancy as the plain measurement)
        Y[:, sl].copy_(Y0[:, sl]), T[sl].copy_(T0[sl]), dt[sl].copy_(dt0[sl])
        p0.record(stream)
        ctx.burn(86, Y[:, sl], T[sl], rho[sl], dt[sl], w["hydro_dt"], eos=nn.EOS_HELMHOLTZ, solver=sv,
                 max_iter=args.max_iter, stream=stream)
        p1.record(stream)
        barrier()
        plain["fast_form_same_particles"] = Pp / (p0.elapsed_time(p1) / 1e3)

    # ---- roofline: FP64 pipe (the kernel computes in FP64; no HBM or tensor bound applies)
    iters = stats["newton_iterations"]
    flops_per_iter = algorithmic_flops(nn, 86, solver)
    refine_flops = 2 * nn.solver_info(86, "sparse")[2] * stats["refinement_steps"]
    achieved = (flops_per_iter * iters + refine_flops) / (kernel_ms / 1e3) / 1e12
    try:
        peak, peak_src = nn.measure_fp64_peak(local), "FP64 FMA probe kernel measured live in this run"
    except Exception:
        peak, peak_src = FP64_PEAK_TFLOPS, "nominal GB300 FP64 (probe failed)"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "strong" if partition else "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, workload c2 distributions)",
            "config": {"workload": "net86+helmholtz c2", "particles_per_gpu": P, "particles_job": P_job,
                       "partition": partition, "hydro_dt": 1e-4,
                       "solver": solver, "l2": "inputs (700 MB of abundances) larger than L2",
                       "launch": launch, "layout": "batched (32 particles per warp)",
                       "value_counts": "every particle carried through the call (any final status); "
                                       "completed_value counts status OK only",
                       "newton_iterations_per_step": iters,
                       **{k: v for k, v in summ.items() if k != "completed_value"}},
            "completed_value": summ["completed_value"] * P_job / P,
            "e2e": {"value": P_job / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "split": e2e_split},
            "gpu_launches": args.steps,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": TRAFFIC_PER_PARTICLE * P,
                         "traffic_source": "dram read+write of one ncu capture (32,768 particles), "
                                           "scaled by the particles of one launch; that case is mostly "
                                           "tail (idle warps' spill traffic), so this overstates a full launch",
                         "peak_source": peak_src + "; MEASURED_PEAKS.json has no FP64 figure",
                         "flops_per_newton_iteration": flops_per_iter,
                         "refinement_steps": stats["refinement_steps"], "fp64_fallbacks": stats["fp64_fallbacks"]},
            "kernel_ms": kernel_ms, "wall_s": wall, "clocks": clk.summary()}
    if mixed:
        line["mixed_fp32lu"] = mixed
    if fused:
        line["post_burn_fused"] = fused
    if plain:
        line["plain_fp64"] = plain
    if args.serve_requests and rank == 0:
        # the c5 stream as specified (200 requests/s of 1k-500k particles: about 100x what one
        # GPU burns, so latency is mostly queueing) ...
        line["serving"] = serve_bench(nn, ctx, solver, args.serve_requests, 5)
        # ... and the same kind of stream at a sustainable load, so latency is service time:
        # sizes / 16 and a rate that offers half of the measured burn rate, for the fast and
        # the mixed-precision forms
        mean16 = (5e5 - 1e3) / np.log(500.0) / 16
        lam = 0.5 * value / mean16
        line["serving_sustainable"] = {f: serve_bench(nn, ctx, f, args.serve_requests, 7, scale=16, rate=lam)
                                       for f in dict.fromkeys([solver, "mixed"])}
        if args.serve_plain_requests and solver != "dense":
            # the plain form serves about 1/300 of the fast form's rate: both forms on the same
            # stream with request sizes divided by 128
            line["serving_small_stream"] = {
                "fast": serve_bench(nn, ctx, solver, args.serve_plain_requests, 6, scale=128),
                "plain_fp64": serve_bench(nn, ctx, "dense", args.serve_plain_requests, 6, scale=128)}
    if rank == 0:
        # the reference's CPU path on the first S particles of the timed set: timed as the
        # baseline, and the checker of the GPU results of those particles
        try:
            o, oracle, flags = _oracle()
            el, thr, out = cpu_burn(o, w, slice(0, S))
            line["cpu_baseline"] = {"value": S / el, "unit": UNIT, "cores": thr, "kind": "port", "build": flags,
                                    "sample": f"particles [0, {S}) of the timed c2 set, {el:.1f} s",
                                    "completed_value": float((out[3] == 0).sum() / el)}
            Ys = w["Y"][:, :S]
            line["parity"] = {"vs": "oracle (the reference's CPU path restated, bit-identical to the reference "
                                    f"built from its sources) on particles [0, {S}) of the timed set",
                              solver: oracle.compare_burns(86, Ys, res_fast, out)}
            if mixed:
                line["parity"]["mixed"] = oracle.compare_burns(86, Ys, res_mixed, out)
        except Exception as e:  # the baseline is reported, never the target
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "error": str(e)}
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def strong_shard(args, ctx, rank, world, dev):
    """Strong scaling: this rank's contiguous range of ONE c2 set, balanced on predicted cost.
    A first (untimed) burn of equal-count ranges gives each particle's Newton iterations; the
    ranks exchange them on the host (the only exchange: particles never move between steps) and
    cut the set with sharding.partition.  Returns (this rank's workload slice, the ranges)."""
    import torch
    import torch.distributed as dist
    import nnet_gb300 as nn
    import sharding
    import workloads
    w = workloads.make("c2", P=args.particles, seed=shard_seed(0))
    P = args.particles

    def piece(a, b):
        return dict(w, Y=w["Y"][:, a:b], T=w["T"][a:b], rho=w["rho"][a:b], dt=w["dt"][a:b])

    a, b = rank * P // world, (rank + 1) * P // world
    q = piece(a, b)
    Y, T = torch.tensor(q["Y"], device=dev), torch.tensor(q["T"], device=dev)
    rho, dt = torch.tensor(q["rho"], device=dev), torch.tensor(q["dt"], device=dev)
    it = torch.zeros(b - a, dtype=torch.int32, device=dev)
    ctx.burn(86, Y, T, rho, dt, w["hydro_dt"], eos=nn.EOS_HELMHOLTZ, solver=args.solver or "sparse",
             iterations=it, max_iter=args.max_iter)
    torch.cuda.synchronize(dev)
    parts = [None] * world
    dist.all_gather_object(parts, it.cpu().numpy())
    ranges = sharding.partition(sharding.cost_estimate(prev_iterations=np.concatenate(parts)), world)
    a, b = ranges[rank]
    return piece(a, b), ranges


# ---------------------------------------------------------------- other configurations
def run_workload(args):
    """One JSON line for configuration c1, c3 or c4 on one GPU: particle-burns/s of the device-
    resident burn (state restored from a pristine HBM copy inside each timed step, inputs larger
    than L2 except c1).  Their errors against the oracle are the parity tests' (tests/).
      c1  net14 + ideal gas, 4,096 particles (the reference's CPU-runnable case)
      c3  2,097,152 particles, 50 % net86 / 30 % net87 / 20 % net14, one nnet_burn_batch launch
      c4  net87 + Helmholtz, 2,097,152 particles, mixed-precision solver beside the FP64 one"""
    import torch
    import nnet_gb300 as nn
    import workloads
    dev = torch.device("cuda", 0)
    ctx = nn.Context(0)
    stream = torch.cuda.current_stream(dev)
    name = args.workload
    solver = args.solver or ("mixed" if name == "c4" else "sparse")
    parts = workloads.make(name) if name != "c3" else workloads.make("c3")
    parts = parts if isinstance(parts, list) else [parts]
    dev_parts = []
    for w in parts:
        dev_parts.append(dict(w=w, Y0=torch.tensor(w["Y"], device=dev), T0=torch.tensor(w["T"], device=dev),
                              dt0=torch.tensor(w["dt"], device=dev), rho=torch.tensor(w["rho"], device=dev),
                              st=torch.empty(w["T"].size, dtype=torch.int32, device=dev)))
    for d in dev_parts:
        d["Y"], d["T"], d["dt"] = torch.empty_like(d["Y0"]), torch.empty_like(d["T0"]), torch.empty_like(d["dt0"])
    P = sum(w["T"].size for w in parts)

    def step(sv):
        for d in dev_parts:
            d["Y"].copy_(d["Y0"]), d["T"].copy_(d["T0"]), d["dt"].copy_(d["dt0"])
        if len(dev_parts) > 1:
            ctx.burn_batch([dict(network=d["w"]["net"], Y=d["Y"], T=d["T"], rho=d["rho"], dt=d["dt"],
                                 hydro_dt=d["w"]["hydro_dt"], status=d["st"]) for d in dev_parts],
                           solver=sv, eos=nn.EOS_HELMHOLTZ, max_iter=args.max_iter, stream=stream)
        else:
            d, w = dev_parts[0], parts[0]
            ctx.burn(w["net"], d["Y"], d["T"], d["rho"], d["dt"], w["hydro_dt"], eos=w["eos"], mu=w["mu"],
                     solver=sv, status=d["st"], max_iter=args.max_iter, stream=stream)

    def timed(sv):
        for _ in range(args.warmup):
            step(sv)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(0) as clk:
            e0.record(stream)
            for _ in range(args.steps):
                step(sv)
            e1.record(stream)
            torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps, ctx.stats(), clk.summary()

    ms, stats, clocks = timed(solver)
    line = {"metric": METRIC, "value": P / (ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": f"synthetic (seeded, workload {name} distributions)",
            "config": {"workload": {"c1": "net14+ideal gas c1", "c3": "net86/net87/net14 mix c3 (one launch)",
                                    "c4": "net87+helmholtz c4"}[name], "particles": P, "solver": solver,
                       "newton_iterations_per_step": stats["newton_iterations"], "status_counts": stats["status"],
                       "refinement_steps": stats["refinement_steps"], "fp64_fallbacks": stats["fp64_fallbacks"]},
            "gpu_launches": args.steps, "clocks": clocks}
    if name == "c4" and solver != "sparse":
        ms2, stats2, _ = timed("sparse")
        line["fp64_sparse"] = {"value": P / (ms2 / 1e3), "unit": UNIT, "ms_per_step": ms2,
                               "newton_iterations_per_step": stats2["newton_iterations"],
                               "fp64_fallbacks_mixed": stats["fp64_fallbacks"]}
    print(json.dumps(line), flush=True)
    ctx.close()


def serve_requests(n, seed, scale=1, rate=200.0):
    """Served burn stream: Poisson arrivals (mean `rate` per second, 200 for the c5 stream),
    sizes log-uniform 1k-500k particles (divided by `scale`), network tag uniform over
    net14/net86/net87, states drawn from the c2 (net86/net87 with Y_e = 0.5, net14 with the
    same composition) distributions."""
    import workloads
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1 / rate, n)
    sizes = np.maximum(np.exp(rng.uniform(np.log(1e3), np.log(5e5), n)) / scale, 1).astype(int)
    nets = rng.choice([14, 86, 87], n)
    reqs = []
    for k in range(n):
        w = workloads.make("c2", P=int(sizes[k]), seed=seed * 1000 + k)
        net = int(nets[k])
        Y = workloads.composition(net, w["T"].size, 0.3, 0.7, 1e-10)
        if net == 87:
            Y[86] = 0.5
        reqs.append(dict(net=net, Y=Y, T=w["T"], rho=w["rho"], dt=w["dt"], hydro_dt=w["hydro_dt"], gap=gaps[k]))
    return reqs


def serve_bench(nn, ctx, solver, n, seed, scale=1, rate=200.0):
    """Submit the stream with its arrival gaps to a continuous-batching server (150 GB
    HBM budget) and report served particle-burns/s and request latency percentiles."""
    import torch
    reqs = serve_requests(n, seed, scale, rate)
    pinned = []
    for r in reqs:  # pinned host buffers: asynchronous copies
        arrs = [torch.from_numpy(np.ascontiguousarray(r[k])).pin_memory() for k in ("Y", "T", "rho", "dt")]
        arrs.append(torch.zeros(r["T"].size, dtype=torch.int32).pin_memory())
        pinned.append(arrs)
    srv = nn.Server(ctx, solver=solver, hbm_budget_bytes=150e9, slice_iterations=64, max_concurrent_requests=8)
    ids = []
    t0 = time.perf_counter()
    for r, a in zip(reqs, pinned):
        time.sleep(r["gap"])
        ids.append(srv.submit(r["net"], a[0].numpy(), a[1].numpy(), a[2].numpy(), a[3].numpy(), r["hydro_dt"],
                              status=a[4].numpy(), max_iter=20000))
    lat = [srv.wait(i) for i in ids]
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    particles = sum(r["T"].size for r in reqs)
    return {"solver": solver, "requests": n, "particles": particles, "value": particles / wall, "unit": UNIT,
            "wall_s": wall, "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p95_s": float(np.percentile(lat, 95)), "latency_p99_s": float(np.percentile(lat, 99)),
            "offered_load": f"Poisson {rate:g}/s, sizes log-uniform 1e3-5e5 / {scale}, nets uniform {{14,86,87}}",
            "offered_particles_per_s": rate * sum(r["T"].size for r in reqs) / n,
            "slices": st["slices"]}


def algorithmic_flops(nn, net, solver):
    """Algorithmic FP64 FLOPs of one Newton iteration: the linear solve as the form executes it
    (2 x multiply-adds of factorisation and triangular solves, plus the divisions), and the
    system assembly 2 (R (k^2 + k) + entries) with k = 2 reactants per reaction.  The mixed
    form's FP32 factorisation is not FP64 work; its FP64 residuals are added per refinement
    step from the run's counters.  Rate and EOS transcendentals are not counted as FLOPs."""
    n = net + 1
    R = nn.NUM_REACTIONS[net]
    f, s, e = nn.solver_info(net, "dense" if solver == "dense" else "sparse")
    if solver == "dense":
        return 2 * (f + s) + n * (n + 1) // 2 + 2 * (R * 6 + n * n)
    lu = 0 if solver == "mixed" else 2 * (f + s) + n
    return lu + 2 * (R * 6 + e)


FP64_PEAK_TFLOPS = 1.25
# dram__bytes_read.sum + dram__bytes_write.sum of burnBatchKernel<86, Helmholtz> on 32,768 c2
# particles (376.4 MB + 538.0 MB): the particle state, the batched slot scratch and register
# spills, most of them those of warps without particles polling for rebalancing hand-offs in
# that tail-dominated case; tables stay in L2
TRAFFIC_PER_PARTICLE = (376.443904e6 + 538.018304e6) / 32768

if __name__ == "__main__":
    main()
