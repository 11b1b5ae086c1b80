#!/usr/bin/env python
"""Benchmark of the GB300 qMC diagram-integration path.

A step is one regular inch step of `inchworm!` (src/inchworm.jl:474-493) on the two-orbital
eg Kanamori model with a discrete bath (beta = 8, n_tau = 256, orders 0:4, N_samples = 2^10
unscrambled Sobol points per topology group): all 16 sampled topology groups of the step in
one launch, the exact order-0 term, then set_ppgf!/normalize! on the host.  The metric is
topology-sample evaluations per second ("diagram evals/s": one (topology, qMC point) pair,
the unit of src/topology_eval.jl:392).

  value    device-resident throughput: kernel time (CUDA events on the library's stream).
  e2e      the same through the C ABI with host buffers: P upload, launch, result download
           and the host-side P update are inside the timed region.
  --impl reference  times the reference's algorithm on the host cores: the CPU oracle (a C
           restatement of src/topology_eval.jl; Julia and QInchworm.jl are not available),
           threaded over sample ranges like MPI ranks, on a bounded sample of the same step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "qinchworm.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "diagram evals/s (topology-sample evaluations per second), plain FP64 inch step"
UNIT = "topology-samples/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 8; batch mode: 1, a step there is the whole multi-solve run)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--samples", type=int, default=1024)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32", "fp32tc"],
                    help="fp32tc: FP32 chains with the 9-wide operator multiplies on tensor cores (t2g)")
    ap.add_argument("--model", default="eg", choices=["eg", "anderson", "t2g", "anderson_b40"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the GPU-vs-oracle check of the benchmarked step")
    ap.add_argument("--no-time-to-tol", action="store_true",
                    help="skip the time-to-tolerance comparison (warped FP32 vs plain FP64) on the eg model")
    ap.add_argument("--mode", default="throughput", choices=["throughput", "accuracy", "batch", "warp", "correlators"])
    ap.add_argument("--step", type=int, default=200, help="warp mode: inch step (tau_w index) the warps are fitted at")
    ap.add_argument("--warp-groups-only", action="store_true",
                    help="warp mode: per-group fits only (no 2^20-sample step reference; for t2g)")
    ap.add_argument("--solves", type=int, default=64, help="batch mode: independent Anderson solves")
    ap.add_argument("--seed", type=int, default=2024, help="batch mode: parameter seed (numpy PCG64)")
    ap.add_argument("--no-sequential", action="store_true", help="batch mode: skip the one-solve-at-a-time arm")
    ap.add_argument("--direct", action="store_true", help="batch mode: also time direct launches (no graph)")
    ap.add_argument("--n-tau", type=int, default=32, help="accuracy mode: tau grid size")
    ap.add_argument("--n-ref", type=int, default=2 ** 15, help="accuracy mode: samples of the FP64 reference")
    ap.add_argument("--n-max", type=int, default=2 ** 13, help="accuracy mode: largest swept N")
    ap.add_argument("--warp-n-max", type=int, default=0, help="accuracy mode: largest N of the warped FP32 arm (0: off)")
    ap.add_argument("--warp-refit", type=int, default=16, help="accuracy mode: refit the warps every this many steps")
    ap.add_argument("--seq-offset", type=int, default=0,
                    help="accuracy mode: skip this many leading Sobol points in every solve, the reference's too "
                         "(1 leaves out the origin; the device-resident loop arms are then not run)")
    return ap.parse_args()


def workload(model: str):
    """(expansion, description, highest order) of a benchmark model."""
    from qiw import models
    if model == "eg":
        return models.eg_discrete_bath(n_tau=256), "eg Kanamori U=2 J=0.2 beta=8 n_tau=256, 4-level bath", 4
    if model == "t2g":
        return (models.t2g_bethe(n_tau=512), "t2g Kanamori U=2.3 J=0.4 beta=20 n_tau=512, semi-elliptic bath D=2 V=0.4",
                3)
    return models.anderson(n_tau=200), "Anderson eps=0.1 U=1 beta=10 n_tau=200, semi-elliptic bath", 4


def bold_groups(orders, N):
    from qiw.diagrammatics import get_topologies_at_order
    from qiw.inchworm import TopologiesInputData
    tds = []
    for o in orders:
        for npa in ([0] if o == 0 else range(1, 2 * o)):
            tops = get_topologies_at_order(o, npa)
            if tops:
                tds.append(TopologiesInputData(o, npa, tops, N))
    return tds


class Clocks:
    """nvidia-smi sampling during the timed region (clocks and throttle reasons)."""

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons)}


def fp64_peak_tflops() -> float:
    """Measured FP64 rate of this GPU: cuBLAS DGEMM 4096^3, best of 3 (CUDA events)."""
    import torch
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * 4096 ** 3 / best / 1e12


def cpu_baseline(exp, tds, samples_cap: int, n: int, budget_s: float = 15.0):
    """Oracle (C restatement of the reference evaluator) on inch step n (tau_w index n), all host
    cores, bounded number of samples per group; returns (topology-samples/s, cores, description)."""
    import oracle as orc
    cores = os.cpu_count() or 1
    pb = orc.OracleProblem(exp)
    g = exp.grid
    t = (g.tau(0), g.tau(n), g.tau(n + 1))
    # calibrate on the heaviest group
    heavy = max(tds, key=lambda td: (td.order, len(td.topologies)))
    n_try = max(cores, 16)
    t0 = time.perf_counter()
    pb.integrate("bold", heavy.order, heavy.n_pts_after, [(x.pairs, x.parity) for x in heavy.topologies], *t,
                 n_try, n_ranks=cores)
    dt = time.perf_counter() - t0
    per_sample_heavy = dt / n_try
    est = sum(per_sample_heavy * len(td.topologies) / len(heavy.topologies) for td in tds if td.order > 0)
    N = int(max(cores, min(samples_cap, budget_s / max(est, 1e-9))))
    t0 = time.perf_counter()
    units = 0
    for td in tds:
        if td.order == 0:
            continue
        pb.integrate("bold", td.order, td.n_pts_after, [(x.pairs, x.parity) for x in td.topologies], *t, N,
                     n_ranks=cores)
        units += len(td.topologies) * N
    el = time.perf_counter() - t0
    return units / el, cores, f"one inch step (tau_w index {n}), {N} Sobol samples per group, {len(tds)} groups"


def parity_check(dev, ses, exp, tds, t, prec, slices):
    """GPU vs oracle on the benchmarked step's groups after the timed region: every sampled group
    on Sobol slices [first, first + n) of its N-point sequence (weights of the full sequence, as
    one rank of rank_sub_range), the exact order 0 once; the oracle runs on all host cores.
    Returns the parity record of the bench line."""
    from concurrent.futures import ThreadPoolExecutor
    import oracle as orc
    from qiw import _lib
    from qiw.device import Work
    dev.set_ppgf(exp.P)
    ob = orc.OracleProblem(exp)
    works, jobs = [], []
    for td in tds:
        gid = ses.group(_lib.QIW_GROUP_BOLD, td)
        tl = [(x.pairs, x.parity) for x in td.topologies]
        for (k, n) in ([(0, 1)] if td.order == 0 else slices):
            N = 1 if td.order == 0 else td.N_samples
            works.append(Work(gid, *t, k, n, N))
            jobs.append((td.order, td.n_pts_after, tl, (k, n), N))
    got = dev.integrate(works, prec)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        want = list(ex.map(lambda j: ob.integrate("bold", j[0], j[1], j[2], *t, j[4], sample_range=j[3]), jobs))
    worst = 0.0
    for a, w in zip(got, want):
        scale = max(float(np.abs(x).max()) for x in w)
        err = max(float(np.abs(x - y).max()) for x, y in zip(a, w))
        worst = max(worst, err / scale if scale > 0 else err)
    n_samp = sum(j[3][1] for j in jobs)
    return {"max_rel_err": worst, "tol": 1e-12 if prec == 0 else 1e-4, "samples_checked": n_samp,
            "topology_samples_checked": sum(j[3][1] * len(j[2]) for j in jobs), "work_items": len(jobs),
            "slices": [list(x) for x in slices], "against": "CPU oracle (C restatement of src/topology_eval.jl)",
            "oracle_s": time.perf_counter() - t0}


def time_to_tol(dev, step=200, n_loop=256, tols=(1e-3, 1e-4), n_ref=2 ** 20, n_max=2 ** 18):
    """Time to a target error on one late eg inch step: warped FP32 (learned warps fitted on the
    step's groups, fit time included) against plain FP64, errors max|sum of the step's groups -
    reference| / max|reference|, reference = plain FP64 at n_ref samples per group.  P comes from
    a plain GPU inchworm loop up to the step (n_loop samples).  A tolerance counts as resolved
    only where the reference's own error (plain vs warped estimate at n_ref) is below half of it.
    Two estimator families: the reference's algorithm (unscrambled Sobol points 0..N-1 from the
    origin x = 0, src/qmc_integrate.jl:497-507), and the same on points 1..N, leaving out the
    origin, whose single value (all integrated times at their segments' starts) puts an O(1/N)
    term into the first."""
    import torch
    from qiw import _lib, models
    from qiw import warp as qwarp
    from qiw.device import Work
    from qiw.diagrammatics import get_topologies_at_order
    from qiw.inchworm import inchworm
    exp = models.eg_discrete_bath(n_tau=256)
    g = exp.grid
    t0 = time.perf_counter()
    inchworm(exp, range(0, 5), range(0, 5), n_loop, dev=dev, n_steps=step - 1)
    loop_s = time.perf_counter() - t0
    dev.set_ppgf(exp.P)
    t = (g.tau(0), g.tau(step), g.tau(step + 1))
    gids = []
    for o in range(0, 5):
        for npa in ([0] if o == 0 else range(1, 2 * o)):
            tops = get_topologies_at_order(o, npa)
            if tops:
                gids.append((o, dev.create_group(_lib.QIW_GROUP_BOLD, o, npa, tops)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    wmap, kept = {}, 0
    fitted = [gid for (o, gid) in gids if o > 0]
    for gid, fit in zip(fitted, qwarp.fit_group_warps(dev, [Work(gid, *t, 0, 0, 0) for gid in fitted])):
        wmap[gid] = -1 if fit.warp_id is None else fit.warp_id
        kept += fit.warp_id is not None
    torch.cuda.synchronize()
    fit_s = time.perf_counter() - t0

    def total(N, prec, warped):
        works = [Work(gid, *t, 0, N, N) for (_, gid) in gids]
        torch.cuda.synchronize()
        a = time.perf_counter()
        res = dev.integrate(works, prec, warps=[wmap.get(gid, -1) for (_, gid) in gids] if warped else None)
        el = time.perf_counter() - a
        return np.concatenate([sum(r[s_] for r in res).ravel() for s_ in range(len(res[0]))]), el

    def point(k, N, prec, warped):   # Sobol point k alone, weight 1/N (k = 0: the origin, every time at its segment's start)
        works = [Work(gid, *t, k, 1, N) for (_, gid) in gids]
        res = dev.integrate(works, prec, warps=[wmap.get(gid, -1) for (_, gid) in gids] if warped else None)
        return np.concatenate([sum(r[s_] for r in res).ravel() for s_ in range(len(res[0]))])

    ref, ref_s = total(n_ref, _lib.QIW_PREC_FP64, False)
    ref_w, _ = total(n_ref, _lib.QIW_PREC_FP32, True)
    # points 1..n_ref: the origin out, point n_ref in
    ref0 = ref - point(0, n_ref, _lib.QIW_PREC_FP64, False) + point(n_ref, n_ref, _lib.QIW_PREC_FP64, False)
    ref0_w = ref_w - point(0, n_ref, _lib.QIW_PREC_FP32, True) + point(n_ref, n_ref, _lib.QIW_PREC_FP32, True)
    sc = float(np.abs(ref).max())
    err = lambda v, r: float(np.abs(v - r).max()) / sc
    sweep, N = [], 2 ** 8
    while N <= n_max:
        vp, sp = total(N, _lib.QIW_PREC_FP64, False)
        vw, sw = total(N, _lib.QIW_PREC_FP32, True)
        vp0 = vp - point(0, N, _lib.QIW_PREC_FP64, False) + point(N, N, _lib.QIW_PREC_FP64, False)
        vw0 = vw - point(0, N, _lib.QIW_PREC_FP32, True) + point(N, N, _lib.QIW_PREC_FP32, True)
        sweep.append({"N": N, "s_plain_fp64": sp, "s_warped_fp32": sw,
                      "err_plain_fp64": err(vp, ref), "err_warped_fp32": err(vw, ref),
                      "err_plain_fp64_origin_skipped": err(vp0, ref0), "err_warped_fp32_origin_skipped": err(vw0, ref0)})
        N *= 2
    out = {"workload": "eg Kanamori U=2 J=0.2 beta=8 n_tau=256, orders 0:4, inch step tau_w index %d" % step,
           "reference": f"plain FP64, {n_ref} samples per group ({ref_s:.1f} s)",
           "fit_s": fit_s, "warps_kept": kept, "groups": len(gids) - 1, "loop_to_step_s": loop_s, "sweep": sweep,
           "target_speedup": 10.0,
           "origin_skipped": "the same estimates on Sobol points 1..N instead of 0..N-1 (the origin left out), "
                             "against the reference on points 1..n_ref"}
    for fam, suffix, r_err in (("reference_algorithm", "", err(ref, ref_w)),
                               ("origin_skipped", "_origin_skipped", err(ref0, ref0_w))):
        rec_f = {"reference_err": r_err}
        for tol in tols:
            key = f"{tol:g}"
            if r_err > 0.5 * tol:
                rec_f[key] = {"resolved": False, "why": f"the reference's own error {r_err:.1e} is above tol/2"}
                continue
            p = next((r for r in sweep if r["err_plain_fp64" + suffix] <= tol), None)
            w = next((r for r in sweep if r["err_warped_fp32" + suffix] <= tol), None)
            rec = {"resolved": True, "plain_fp64_N": p and p["N"], "plain_fp64_s": p and p["s_plain_fp64"],
                   "warped_fp32_N": w and w["N"], "warped_fp32_s": w and w["s_warped_fp32"]}
            if p and w:
                rec["speedup_fit_included"] = p["s_plain_fp64"] / (w["s_warped_fp32"] + fit_s)
                rec["speedup_step_only"] = p["s_plain_fp64"] / w["s_warped_fp32"]
                rec["speedup_fit_amortised_over_50_steps"] = p["s_plain_fp64"] / (w["s_warped_fp32"] + fit_s / 50)
            rec_f[key] = rec
        out[fam] = rec_f
    return out


def julia_probe():
    """Whether the reference itself (pure Julia) could run on this host."""
    import shutil
    jl = shutil.which("julia")
    if not jl:
        return {"julia": None, "qinchworm_loads": False,
                "note": "no julia on this host: the reference (pure Julia) cannot run here; the arm is the oracle port"}
    out = {"julia": None, "qinchworm_loads": False}
    try:
        out["julia"] = subprocess.run([jl, "--version"], capture_output=True, text=True, timeout=60).stdout.strip()
        r = subprocess.run([jl, "-e", "using QInchworm"], capture_output=True, text=True, timeout=300)
        out["qinchworm_loads"] = r.returncode == 0
        if r.returncode:
            out["note"] = "QInchworm.jl or its dependencies are not installed: the arm is the oracle port"
    except (OSError, subprocess.TimeoutExpired) as e:
        out["note"] = f"julia probe failed: {e}"
    return out


def bench_config(desc, kmax, N, tds):
    """The workload description both arms print (identical dicts)."""
    return {"workload": desc + f", orders 0:{kmax}, one regular inch step per bench step",
            "N_samples": N, "groups_per_step": len(tds), "topologies_per_step": sum(len(td.topologies) for td in tds)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    exp, desc, kmax = workload(args.model)
    tds = bold_groups(range(0, kmax + 1), args.samples)
    vals = []
    for i in range(args.warmup + args.steps):   # step i at tau_w index 1 + i, as the GPU arm steps
        v, cores, sample = cpu_baseline(exp, tds, args.samples, 1 + i, budget_s=8.0)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": bench_config(desc, kmax, args.samples, tds),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample + f"; steps at tau_w indices {1 + args.warmup}..{args.warmup + args.steps}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_probe": julia_probe()}
    print(json.dumps(line))


# DRAM bytes (read + write) of one eval_kernel launch of the default FP64 eg inch step, from one
# ncu capture of `python bench.py --steps 2 --warmup 3 --no-cpu-baseline --no-parity
# --no-time-to-tol` (dram__bytes_read.sum 22.88 GB + dram__bytes_write.sum 27.65 GB at 1024
# samples, one pass): the per-thread arenas spilling from L2.  It grows with the samples; other
# workloads report null.
EG_FP64_TRAFFIC_PER_1024 = 50.53e9


def _traffic(args):
    if args.model == "eg" and args.precision == "fp64":
        return EG_FP64_TRAFFIC_PER_1024 * args.samples / 1024
    return None


def bare_step(ses, exp, kmax, N_total, prec, comm):
    """The bench's bare step tau_0 -> tau_1 (orders 0:kmax), written into exp.P."""
    from qiw import _lib, ppgf
    from qiw.diagrammatics import get_topologies_at_order
    from qiw.inchworm import TopologiesInputData, _accumulate
    grid = exp.grid
    bare = [TopologiesInputData(o, 2 * o, get_topologies_at_order(o), N_total) for o in range(0, kmax + 1)]
    val, _, _ = _accumulate(ses.run(_lib.QIW_GROUP_BARE, bare, grid.tau(0), 0.0, grid.tau(1), prec, comm), bare,
                            exp.dims)
    ppgf.set_ppgf(exp.P, 1, val)


def make_step(ses, exp, tds, prec, comm):
    """One bench step n: inch step tau_n -> tau_{n+1} of every group (each rank its sample range,
    one all-reduce per launch through comm), set_ppgf! and normalize!(P, tau) on the host."""
    from qiw import _lib, ppgf
    from qiw.inchworm import _accumulate
    grid = exp.grid

    def step(n):
        ses.dev.set_ppgf(exp.P)
        res = ses.run(_lib.QIW_GROUP_BOLD, tds, grid.tau(0), grid.tau(n), grid.tau(n + 1), prec, comm)
        v, _, _ = _accumulate(res, tds, exp.dims)
        ppgf.set_ppgf(exp.P, n + 1, v)
        ppgf.normalize_tau(exp.P, n + 1)
    return step


def run_ours(args):
    import torch
    from qiw import _lib
    from qiw.device import Device
    from qiw.inchworm import _Session, Comm, TorchComm
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    comm = Comm()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        comm = TorchComm()
    torch.cuda.set_device(local)
    prec = {"fp64": _lib.QIW_PREC_FP64, "fp32": _lib.QIW_PREC_FP32, "fp32tc": _lib.QIW_PREC_FP32_TC}[args.precision]
    exp, desc, kmax = workload(args.model)
    grid = exp.grid
    # weak scaling: every rank evaluates N_samples per group; the step result is all-reduced
    N = args.samples
    tds = bold_groups(range(0, kmax + 1), N * world)
    dev = Device(local)
    ses = _Session(dev, exp)
    for td in tds:
        ses.group(_lib.QIW_GROUP_BOLD, td)
    stats = {id(td): dev.group_stats(ses.group(_lib.QIW_GROUP_BOLD, td)) for td in tds}
    units_rank = sum(len(td.topologies) * (N if td.order > 0 else 1) for td in tds if td.order > 0)
    flops_rank = sum(stats[id(td)].flops_per_sample * N for td in tds if td.order > 0)
    # bare step, then warm-up and timed regular steps
    bare_step(ses, exp, kmax, N * world, prec, comm)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    kernel_ms, wall_s = [], []
    step = make_step(ses, exp, tds, prec, comm)

    n = 1
    for _ in range(args.warmup):
        step(n)
        n += 1
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk = Clocks(local)
    for _ in range(args.steps):
        flush.fill_(float(n))  # write 256 MB (> L2) between timed steps
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step(n)
        wall_s.append(time.perf_counter() - t0)
        kernel_ms.append(dev.last_kernel_ms())
        n += 1
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = clk.stop()
    k_tot = sum(kernel_ms) / 1e3
    w_tot = sum(wall_s)
    if world > 1:
        t = torch.tensor([k_tot, w_tot], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        k_tot, w_tot = float(t[0]), float(t[1])
    units = units_rank * world * args.steps
    # bytes copied per step: i*P tables (FP64 + FP32), work/Sobol descriptors; results back
    S2 = int(np.sum(np.array(exp.dims) ** 2))
    h2d = grid.n_tau * S2 * (8 + 4) + len(tds) * (80 + 4 * 32 * 8 + 16)
    d2h = len(tds) * S2 * 16 + 4
    if rank != 0:
        return
    peak = dev.fma_peak_tflops(prec)
    dgemm = fp64_peak_tflops() if args.precision == "fp64" else None
    achieved = flops_rank * args.steps / k_tot / 1e12
    line = {
        "metric": METRIC if args.precision == "fp64" else METRIC.replace("plain FP64", "FP32 chain products"),
        "value": units / k_tot, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * k_tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64acc", "data": "synthetic",
        "config": bench_config(desc, kmax, N * world, tds),
        "l2_flush": "256 MB write between timed steps",
        "e2e": {"value": units / w_tot, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1e3 * w_tot / args.steps},
        "roofline": {"bound": "fp64_pipe" if args.precision == "fp64" else "fp32_pipe", "achieved": achieved,
                     "peak": peak, "unit": "TFLOP/s", "frac": (achieved / peak) if peak else None,
                     "traffic": _traffic(args),
                     "peak_source": "measured on this GPU: independent FMA chains on every SM (qiw_measure_fma_peak); "
                                    "MEASURED_PEAKS.json has no FP64 or FP32 CUDA-core entry",
                     "dgemm_tflops_measured": dgemm, "flops_per_step": flops_rank},
        "gpu_launches": 2 * args.steps,
        "clocks": clocks,
    }
    if not args.no_parity and world == 1:   # the benchmarked step against the oracle, after timing
        N_all = N * world
        starts = sorted({k for k in (0, N_all // 4 + 5, N_all // 2 + 11, max(N_all - 64, 0)) if k < N_all})
        sl = [(k, min(64, N_all - k)) for k in starts]
        line["parity"] = parity_check(dev, ses, exp, tds, (grid.tau(0), grid.tau(n), grid.tau(n + 1)), prec, sl)
    if not args.no_time_to_tol and world == 1 and args.model == "eg":
        line["time_to_tol"] = time_to_tol(dev)
    if not args.no_cpu_baseline and world == 1:   # the CPU leg runs at N = 1 only
        v, cores, sample = cpu_baseline(exp, tds, N, 1 + args.warmup + args.steps // 2)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
    print(json.dumps(line))


def _solve(model, n_tau, N, prec, dev, corr=False, device_loop=False, warp_policy=None, seq_offset=0):
    """Full inchworm! on the GPU; returns (P normalised by beta as arrays, G or None, seconds).
    device_loop: the whole loop on the device (qiw.batch, one CUDA graph) instead of the host
    loop with one launch per step.  Group plans come from the process's plan cache once a
    solve on the same operators has made them, for both loops alike."""
    import torch
    from qiw import models, ppgf
    from qiw.inchworm import inchworm, correlator_2p
    if model == "eg":
        exp = models.eg_discrete_bath(n_tau=n_tau, corr=corr)
    elif model == "anderson_b40":   # strongly correlated, low temperature: concentrated integrands
        exp = models.anderson(eps=-2.0, U=4.0, beta=40.0, n_tau=n_tau, corr=corr)
    else:
        exp = models.anderson(n_tau=n_tau, corr=corr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if device_loop:
        from qiw.batch import inchworm_batch
        inchworm_batch([exp], range(0, 5), range(0, 5), N, precision=prec, autotune=False)
    else:
        inchworm(exp, range(0, 5), range(0, 5), N, dev=dev, precision=prec, warp_policy=warp_policy,
                 seq_offset=seq_offset)
    el = time.perf_counter() - t0
    ppgf.normalize_beta(exp.P, exp.grid.beta)
    G = None
    if corr:
        G = np.array(correlator_2p(exp, range(0, 4), N, dev=dev, precision=prec, seq_offset=seq_offset))
    return [P_s.data.copy() for P_s in exp.P], G, el


def _perr(P, Q):
    return max(float(np.abs(a - b).max()) for a, b in zip(P, Q))


def run_accuracy(args):
    """Time to 1e-4 max |P(tau) - P_ref(tau)| for the plain FP64 and the FP32-chain paths
    against a plain FP64 run at args.n_ref samples, plus max |P_FP32 - P_FP64| and the G(tau)
    difference at equal N (same Sobol points)."""
    from qiw import _lib
    from qiw.device import Device
    dev = Device(int(os.environ.get("LOCAL_RANK", "0")))
    # one-time planning of every group (cold minus warm solve at N = 256); later solves reuse the plans
    dev.plan_cache_clear()
    off = args.seq_offset
    t_cold = _solve(args.model, args.n_tau, 256, _lib.QIW_PREC_FP64, dev)[2]
    t_warm = _solve(args.model, args.n_tau, 256, _lib.QIW_PREC_FP64, dev)[2]
    P_ref, _, t_ref = _solve(args.model, args.n_tau, args.n_ref, _lib.QIW_PREC_FP64, dev, seq_offset=off)
    sweep = []
    N = 256
    while N <= args.n_max:
        row = {"N": N}
        P64, G64, t64 = _solve(args.model, args.n_tau, N, _lib.QIW_PREC_FP64, dev, corr=(N == 1024), seq_offset=off)
        P32, G32, t32 = _solve(args.model, args.n_tau, N, _lib.QIW_PREC_FP32, dev, corr=(N == 1024), seq_offset=off)
        row.update(err_fp64=_perr(P64, P_ref), err_fp32=_perr(P32, P_ref), s_fp64=t64, s_fp32=t32,
                   fp32_vs_fp64_P=_perr(P32, P64))
        if G64 is not None:
            row["fp32_vs_fp64_G"] = float(np.abs(G32 - G64).max())
        if off:   # the device-resident loop runs the reference's sequences only
            sweep.append(row)
            N *= 2
            continue
        # the same solves with the loop on the device (warm: the first call pays the CUDA setup)
        if N == 256:
            _solve(args.model, args.n_tau, N, _lib.QIW_PREC_FP32, dev, device_loop=True)
        P64d, _, t64d = _solve(args.model, args.n_tau, N, _lib.QIW_PREC_FP64, dev, device_loop=True)
        P32d, _, t32d = _solve(args.model, args.n_tau, N, _lib.QIW_PREC_FP32, dev, device_loop=True)
        row.update(err_fp64_dev=_perr(P64d, P_ref), err_fp32_dev=_perr(P32d, P_ref), s_fp64_dev=t64d,
                   s_fp32_dev=t32d, dev_vs_host_P=_perr(P64d, P64))
        sweep.append(row)
        N *= 2

    warped = []
    if args.warp_n_max:
        from qiw.warp import WarpPolicy
        pol = WarpPolicy(refit_every=args.warp_refit, n_train=2 ** 14)
        N = 256
        while N <= args.warp_n_max:
            Pw, _, tw = _solve(args.model, args.n_tau, N, _lib.QIW_PREC_FP32, dev, warp_policy=pol, seq_offset=off)
            warped.append({"N": N, "err_warped_fp32": _perr(Pw, P_ref), "s_warped_fp32": tw})
            N *= 2

    def ttt(key_err, key_t):
        for r in sweep:
            if key_err in r and r[key_err] <= 1e-4:
                return r[key_t], r["N"]
        return None, None

    def first_below(rows, key_err, key_t, tol):
        for r in rows:
            if key_err in r and r[key_err] <= tol:
                return r[key_t], r["N"]
        return None, None

    thresholds = {}
    for tol in (3e-2, 1e-2, 3e-3, 1e-3, 1e-4):
        thresholds[f"{tol:g}"] = {"plain_fp64": first_below(sweep, "err_fp64", "s_fp64", tol),
                                  "fp32_device_loop": first_below(sweep, "err_fp32_dev", "s_fp32_dev", tol),
                                  "warped_fp32": first_below(warped, "err_warped_fp32", "s_warped_fp32", tol)}
    t64, n64 = ttt("err_fp64", "s_fp64")
    t32, n32 = ttt("err_fp32", "s_fp32")
    t64d, n64d = ttt("err_fp64_dev", "s_fp64_dev")
    t32d, n32d = ttt("err_fp32_dev", "s_fp32_dev")
    print(json.dumps({"mode": "accuracy", "metric": "time to 1e-4 max |P(tau) - P_ref(tau)|", "unit": "s",
                      "config": {"model": args.model, "n_tau": args.n_tau, "orders": "0:4", "N_ref": args.n_ref,
                                 "reference": "plain FP64 GPU run at N_ref (Sobol, same grid)", "seq_offset": off},
                      "time_to_1e-4_fp64": t64, "N_fp64": n64, "time_to_1e-4_fp32": t32, "N_fp32": n32,
                      "speedup_fp32": (t64 / t32) if (t64 and t32) else None,
                      "time_to_1e-4_fp64_device_loop": t64d, "N_fp64_device_loop": n64d,
                      "time_to_1e-4_fp32_device_loop": t32d, "N_fp32_device_loop": n32d,
                      "speedup_fp32_device_loop_vs_plain_fp64": (t64 / t32d) if (t64 and t32d) else None,
                      "reference_solve_s": t_ref, "planning_s": t_cold - t_warm,
                      "timing": "solves after the first reuse the group plans (process plan cache); planning_s is the one-time cost",
                      "sweep": sweep, "warped_sweep": warped,
                      "time_to_error": thresholds,
                      "warp_refit_every": args.warp_refit}))


def run_warp(args):
    """Learned warp on the eg model (beta = 8, n_tau = 256, orders 1:4): for every topology group
    at one inch step, a warp trained on 2^16 plain-qMC samples of the group, then the variance of
    R = 16 scrambled replicas of N = 1024 points with and without it (qiw.warp.fit_group_warp)."""
    import torch
    from qiw import _lib
    from qiw.device import Device, Work
    from qiw.diagrammatics import get_topologies_at_order
    from qiw import warp as qwarp
    exp, desc, kmax = workload(args.model)
    g = exp.grid
    dev = Device(int(os.environ.get("LOCAL_RANK", "0")))
    dev.set_problem(exp)
    dev.set_ppgf(exp.P)
    n = min(args.step, g.n_tau - 2)
    rows = []
    for o in range(1, kmax + 1):
        for npa in range(1, 2 * o):
            tops = get_topologies_at_order(o, npa)
            if not tops or 2 * o > 8:
                continue
            gid = dev.create_group(_lib.QIW_GROUP_BOLD, o, npa, tops)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fit = qwarp.fit_group_warp(dev, Work(gid, g.tau(0), g.tau(n), g.tau(n + 1), 0, 0, 0), n_train=2 ** 16, R=16)
            rows.append({"order": o, "n_pts_after": npa, "topologies": len(tops), "variance_gain": fit.gain,
                         "kept": fit.warp_id is not None, "bias_sigma": fit.bias_sigma, "loss": fit.loss,
                         "fit_s": time.perf_counter() - t0})
    if args.warp_groups_only:
        print(json.dumps({"mode": "warp", "config": {"workload": desc + f", inch step tau_w index {n}",
                                                      "train_samples": 2 ** 16, "replicas": 16, "N_per_replica": 1024},
                          "groups": rows}))
        return
    # the whole step: every group summed, plain vs warped (kept warps), against plain at 2^20
    fits = {}
    gids = []
    for o in range(0, kmax + 1):
        for npa in ([0] if o == 0 else range(1, 2 * o)):
            tops = get_topologies_at_order(o, npa)
            if tops:
                gids.append((o, npa, dev.create_group(_lib.QIW_GROUP_BOLD, o, npa, tops)))
    wmap = {}
    for (o, npa, gid) in gids:
        if o == 0 or 2 * o > 8:
            continue
        fit = qwarp.fit_group_warp(dev, Work(gid, g.tau(0), g.tau(n), g.tau(n + 1), 0, 0, 0), n_train=2 ** 16, R=16)
        wmap[gid] = fit.warp_id if fit.warp_id is not None else -1

    def step_total(N, prec, warped, step=n):
        works = [Work(gid, g.tau(0), g.tau(step), g.tau(step + 1), 0, N, N) for (_, _, gid) in gids]
        wl = [wmap.get(gid, -1) for (_, _, gid) in gids] if warped else None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = dev.integrate(works, prec, warps=wl)
        el = time.perf_counter() - t0
        return np.concatenate([sum(r[s] for r in res).ravel() for s in range(len(res[0]))]), el

    ref, t_ref = step_total(2 ** 20, _lib.QIW_PREC_FP64, False)
    ref_w, _ = step_total(2 ** 20, _lib.QIW_PREC_FP64, True)   # the warped estimate at the same N
    sc = float(np.abs(ref).max())
    sweep = []
    N = 2 ** 10
    while N <= 2 ** 16:
        row = {"N": N}
        for key, prec, warped in [("plain_fp64", _lib.QIW_PREC_FP64, False), ("warped_fp64", _lib.QIW_PREC_FP64, True),
                                  ("warped_fp32", _lib.QIW_PREC_FP32, True)]:
            v, el = step_total(N, prec, warped)
            row["err_" + key] = float(np.abs(v - ref).max()) / sc
            row["err_vs_warped_ref_" + key] = float(np.abs(v - ref_w).max()) / sc
            row["s_" + key] = el
        sweep.append(row)
        N *= 2
    # the same warps reused at later steps (no refit): does the gain persist?
    reuse = []
    for dn in (20, 50):
        m = min(n + dn, g.n_tau - 2)
        r_m, _ = step_total(2 ** 20, _lib.QIW_PREC_FP64, False, m)
        sc_m = float(np.abs(r_m).max())
        for Nr in (2 ** 10, 2 ** 13):
            vp, _ = step_total(Nr, _lib.QIW_PREC_FP64, False, m)
            vw, _ = step_total(Nr, _lib.QIW_PREC_FP32, True, m)
            reuse.append({"step": m, "N": Nr, "err_plain_fp64": float(np.abs(vp - r_m).max()) / sc_m,
                          "err_warped_fp32": float(np.abs(vw - r_m).max()) / sc_m})
    print(json.dumps({"mode": "warp", "config": {"workload": desc + f", inch step tau_w index {n}",
                                                  "train_samples": 2 ** 16, "replicas": 16, "N_per_replica": 1024,
                                                  "step_reference": "plain FP64 at 2^20 samples per group"},
                      "groups": rows, "reference_s": t_ref,
                      "plain_vs_warped_at_2^20": float(np.abs(ref - ref_w).max()) / sc, "step_sweep": sweep,
                      "reuse_at_later_steps": reuse}))


def run_correlators(args):
    """inchworm! then correlator_2p (G(tau) and <S+(tau) S->) on the t2g model, FP64 and FP32
    chains, with the FP32 error of P and of every correlator against the FP64 path (which the
    parity tests tie to the oracle group by group).  n_tau and N from --n-tau / --samples."""
    import torch
    from qiw import _lib, models, ppgf
    from qiw.device import Device
    from qiw.inchworm import correlator_2p, inchworm
    dev = Device(int(os.environ.get("LOCAL_RANK", "0")))
    out = {}
    for name, prec in (("fp64", _lib.QIW_PREC_FP64), ("fp32", _lib.QIW_PREC_FP32)):
        exp = models.t2g_bethe(n_tau=args.n_tau, corr=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        inchworm(exp, range(0, 4), range(0, 4), args.samples, dev=dev, precision=prec)
        t1 = time.perf_counter()
        ppgf.normalize_beta(exp.P, exp.grid.beta)
        gs = correlator_2p(exp, range(0, 4), args.samples, dev=dev, precision=prec)
        t2 = time.perf_counter()
        out[name] = ([P_s.data.copy() for P_s in exp.P], [np.asarray(g) for g in gs], t1 - t0, t2 - t1)
    P64, G64, ti64, tc64 = out["fp64"]
    P32, G32, ti32, tc32 = out["fp32"]
    print(json.dumps({"mode": "correlators", "config": {"workload": f"t2g Kanamori U=2.3 J=0.4 beta=20 n_tau={args.n_tau}, "
                                                        "orders 0:3, correlators G(tau) and <S+(tau) S-> of orbital 1",
                                                        "N_samples": args.samples},
                      "inchworm_s": {"fp64": ti64, "fp32": ti32}, "correlator_2p_s": {"fp64": tc64, "fp32": tc32},
                      "fp32_max_abs_dP": _perr(P32, P64), "P_max_abs": max(float(np.abs(p).max()) for p in P64),
                      "fp32_max_abs_dG": [float(np.abs(a - b).max()) for a, b in zip(G32, G64)],
                      "G_max_abs": [float(np.abs(g).max()) for g in G64],
                      "G_fp64_tau0_beta": [[[complex(g[0]).real, complex(g[0]).imag], [complex(g[-1]).real, complex(g[-1]).imag]]
                                           for g in G64]}))


def batch_solves(seed: int, n: int):
    """Seed-drawn Anderson solves: beta U[2, 40], n_tau U{64..512}, U U[0.5, 4], eps U[-1, 1],
    V U[0.2, 1], D = 2, max order U{2..6}, N = 2^U{8..14} (numpy PCG64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        beta = float(rng.uniform(2, 40))
        n_tau = int(rng.integers(64, 513))
        U = float(rng.uniform(0.5, 4))
        eps = float(rng.uniform(-1, 1))
        V = float(rng.uniform(0.2, 1.0))
        kmax = int(rng.integers(2, 7))
        N = 2 ** int(rng.integers(8, 15))
        out.append(dict(beta=beta, n_tau=n_tau, U=U, eps=eps, V=V, kmax=kmax, N=N))
    return out


def run_batch(args):
    """Independent solves in one device-resident launch queue (persistent kernel, CUDA graph,
    autotuned tiles) against the same solves one at a time through the host-driven loop."""
    import torch
    from qiw import _lib, models
    from qiw.batch import Batch
    from qiw.device import Device
    from qiw.inchworm import inchworm
    from qiw.batch import shard_solves, solve_cost
    prec = _lib.QIW_PREC_FP32 if args.precision == "fp32" else _lib.QIW_PREC_FP64
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:   # independent solves: each rank runs its share whole, no data exchange
        import torch.distributed as dist
        dist.init_process_group("gloo")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    specs_all = batch_solves(args.seed, args.solves)
    mine = shard_solves([solve_cost(p["n_tau"], p["kmax"], p["N"]) for p in specs_all], rank, world)
    specs = [specs_all[i] for i in mine]
    mk = lambda p: models.anderson(eps=p["eps"], U=p["U"], D=2.0, V=p["V"], beta=p["beta"], n_tau=p["n_tau"])
    exps = [mk(p) for p in specs]
    t0 = time.perf_counter()
    b = Batch(int(os.environ.get("LOCAL_RANK", "0")))
    for e, p in zip(exps, specs):
        b.add(e, range(0, p["kmax"] + 1), range(0, p["kmax"] + 1), p["N"])
    setup_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    first = b.run(prec, graph=True, autotune=True)          # tunes, captures, runs
    first_s = time.perf_counter() - t0
    runs = []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = b.run(prec, graph=True, autotune=True)
        P_batch = [b.P_table(i) for i in range(len(exps))]
        runs.append((r, time.perf_counter() - t0))
    r, wall = min(runs, key=lambda x: x[0].kernel_ms)
    kernel_s, samples = r.kernel_ms * 1e-3, r.topology_samples
    if world > 1:   # whole job: every rank's samples over the slowest rank's time
        import torch.distributed as dist
        t = torch.tensor([kernel_s, wall], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        u = torch.tensor([samples], dtype=torch.float64)
        dist.all_reduce(u)
        kernel_s, wall, samples = float(t[0]), float(t[1]), float(u[0])
        if rank != 0:
            return
    direct = b.run(prec, graph=False, autotune=True) if args.direct else None
    line = {"mode": "batch", "metric": "topology-sample evaluations per second, independent Anderson solves",
            "value": samples / kernel_s, "unit": "topology-samples/s", "n_gpus": world, "scaling": "strong",
            "steps": len(runs), "ms_per_step": kernel_s * 1e3, "higher_is_better": True, "dtype": args.precision.replace("fp", "f"),
            "data": "synthetic", "config": {"workload": f"{len(specs_all)} Anderson solves, seed {args.seed}",
                                            "ranges": "beta U[2,40], n_tau U{64..512}, U U[0.5,4], eps U[-1,1], V U[0.2,1], D=2, max order U{2..6}, N 2^U{8..14}",
                                            "total_steps": int(sum(p["n_tau"] - 1 for p in specs_all))},
            "e2e": {"value": samples / wall, "unit": "topology-samples/s", "seconds": wall},
            "solves_on_rank0": len(specs),
            "flops_rank0": r.flops, "tflops_rank0": r.flops / (r.kernel_ms * 1e-3) / 1e12,
            "tiles": {"threads": r.threads, "persistent": r.persistent, "grid": r.grid, "tiles_per_step": r.tiles_per_step,
                      "autotune_ms_step1": {f"{t}{'p' if pm == 0 else '1'}": round(first.tune_ms[i * 2 + pm], 3)
                                            for i, t in enumerate((32, 64, 128)) for pm in (0, 1)}},
            "graph_nodes": r.graph_nodes, "n_plans": r.n_plans, "setup_s": setup_s, "first_run_s": first_s,
            "direct_launches_ms": direct.kernel_ms if direct else None}
    if not args.no_sequential and world == 1:
        dev = Device(int(os.environ.get("LOCAL_RANK", "0")))
        seq_s, worst = 0.0, 0.0
        for i, p in enumerate(specs):
            e = mk(p)
            init = [P_s.data.copy() for P_s in e.P]
            inchworm(e, range(0, p["kmax"] + 1), range(0, p["kmax"] + 1), p["N"], dev=dev, precision=prec, n_steps=1)
            for P_s, d in zip(e.P, init):   # the short run above only planned the groups
                P_s.data[...] = d
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            inchworm(e, range(0, p["kmax"] + 1), range(0, p["kmax"] + 1), p["N"], dev=dev, precision=prec)
            torch.cuda.synchronize()
            seq_s += time.perf_counter() - t0
            ref = np.concatenate([np.transpose(P_s.data, (0, 2, 1)).ravel() for P_s in e.P])
            worst = max(worst, float(np.abs(P_batch[i] - ref).max() / np.abs(ref).max()))
        line["sequential"] = {"value": r.topology_samples / seq_s, "unit": "topology-samples/s", "seconds": seq_s,
                              "what": "the same solves one at a time: host loop, one qiw_integrate launch per step"}
        line["speedup_vs_sequential"] = seq_s / wall
        line["max_rel_diff_vs_sequential"] = worst
    print(json.dumps(line))


if __name__ == "__main__":
    a = parse()
    if a.steps is None:
        a.steps = 1 if (a.mode == "batch" and a.impl != "reference") else 8
    if a.impl == "reference":
        run_reference(a)
    elif a.mode == "accuracy":
        run_accuracy(a)
    elif a.mode == "batch":
        run_batch(a)
    elif a.mode == "warp":
        run_warp(a)
    elif a.mode == "correlators":
        run_correlators(a)
    else:
        run_ours(a)
