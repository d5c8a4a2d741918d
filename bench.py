"""Benchmark of the 2D-BZ tau / CPA path: (E,k) points per second.

Workload: the relativistic (kappa,mu) bcc(001) interface, lmax=3 (32x32 per
site), 4 layers per principal layer (128x128 blocks), 12 interface layers,
24 semicircle-contour energies with uneven adaptive IBZ meshes of 210..12090
k points, square wells with j = l +- 1/2 split depths (seeded synthetic
inputs, see skkr_budapest_gb300/workloads.py).

One step = one contour energy, all of its k points carried through the CPA
pass: G_scr(k) transform, L and R decimation, tau2d, k-sum with point-group
rotation, CPA update.  Steps cycle through the 24 contour energies; the
default run times each of them once (38 145 (E,k) points).

  value   (E,k)/s with inputs resident in HBM (every step's energy staged
          before the timed region), device time from CUDA events on the
          library stream.
  e2e     the same metric through the reference-facing call
          skkr_gpu_cpacoord with host buffers (H2D of inputs, D2H of results
          inside the timed region).

`--impl reference` times the reference's CPU algorithm (the oracle port of
the Fortran routines) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "(E,k) points/s: mixed+batched vs FP64 GPU at <=1e-9 rel err in k-summed tau"
UNIT = "(E,k)/s"
WORKLOAD = "rel_bcc001_lmax3_pl4_12layers_24E"
# contour energies visited by the steps, in order (adaptive k: 210 .. 12090):
# the default 3 warm-up steps take the largest energy (all buffers at full
# size) and the first two; the default 24 timed steps are the whole contour
STEP_ENERGIES = [23] + list(range(23))


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=24)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--energies", default="", help="comma list overriding the step energies")
    ap.add_argument("--split", default="energies", choices=["energies", "k"],
                    help="N > 1: each rank its own contour energies (weak scaling), or every energy's k points "
                         "split round-robin over the ranks with one in-place NCCL allreduce of the k-summed tau "
                         "per CPA iteration (strong scaling)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="only the device loop of the timed steps (for ncu captures); prints a short line")
    ap.add_argument("--slab", type=int, default=12, help="gk workload: layers of the screening slab")
    ap.add_argument("--slices", type=int, default=0, help="BF16 slices per product operand (0: the library's 6)")
    ap.add_argument("--newton", type=int, default=2, help="standard Newton steps of the split-precision inverse")
    ap.add_argument("--fp64-ref", default="", help="file of the FP64 pass (tau per energy, timing): written when "
                                                   "absent, read instead of rerunning the FP64 pass when present")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "gk", "tauij"],
                    help="c1: the plain non-relativistic interface, the whole contour per step, FP64 and split "
                         "precision; "
                         "c3: one energy of each of three systems per step through skkr_gpu_cpacoord_many; "
                         "c4: CPA alloy interfaces from the ATA and from the learned start; "
                         "c5: the BdG interface (n_PL = 256, Im E = 1e-4 Ry), FP64 and split precision; "
                         "gk: the C2 path on the reference's k-space G_scr(k) (Kambe sums + slab screening) "
                         "beside the table transform; "
                         "tauij: the off-diagonal tau of the interface (skkr_gpu_tauij) per step")
    return ap.parse_args()


def dist_init(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1
    import torch
    import torch.distributed as dist
    dist.init_process_group("nccl")
    r = dist.get_rank()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", r)))
    return r, dist.get_world_size()


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, ws):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-i", os.environ.get("LOCAL_RANK", "0"), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except Exception:
            self.p.kill()
            out = ""
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def l2_flush(buf):
    if buf is not None:
        buf.add_(1.0)


def fp64_peak_tflops():
    """cuBLAS ZGEMM (complex128) burst rate on this GPU, TFLOP/s."""
    import torch
    n = 2048
    a = torch.randn(n, n, dtype=torch.complex128, device="cuda")
    b = torch.randn(n, n, dtype=torch.complex128, device="cuda")
    a @ b
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e))
    return 8.0 * n ** 3 / (best * 1e-3) / 1e12


def traffic_from_profiles():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        return json.load(open(p))
    except Exception:
        return {}


def strided(ep, m):
    """m k points spread evenly over the whole mesh of ep (first to last), with
    their weights renormalised: a sample of every part of the zone, not the
    start of the IBZ list."""
    idx = np.unique(np.linspace(0, ep.nk - 1, max(1, min(m, ep.nk))).round().astype(int))
    return ep.with_k(ep.xk[idx], ep.wk[idx] / ep.wk[idx].sum())


def _oracle_rate(eps_list, per_step, nthreads):
    """(E,k)/s of the oracle's full CPA pass over strided samples of the given
    energies on nthreads host threads; returns (rate, points, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    t0 = time.perf_counter()
    pts = 0
    for ep in eps_list:
        sub = strided(ep, per_step)
        if O.cpacoord(sub, nthreads=nthreads)["status"] != 0:
            raise RuntimeError("oracle failed on the CPU sample")
        pts += sub.nk
    dt = time.perf_counter() - t0
    return pts / dt, pts, dt


def cpu_baseline(nthreads, budget_s=20.0):
    """The oracle (port of the reference's Fortran routines) on the host
    cores, on a bounded sample of the same workload: k points spread evenly
    over the mesh of contour energy 19 (2485 points), grown until about a
    third of budget_s, on all threads; then a single-core figure on a smaller
    strided sample of the same energy."""
    from skkr_budapest_gb300 import workloads as W
    ep = W.energy_problem(W.rel_bcc(), 19)
    m = nthreads
    while True:
        v, pts, t = _oracle_rate([ep], m, nthreads)
        if t > budget_s / 3 or m >= 8 * nthreads:
            break
        m *= 2
    v1, p1, t1 = _oracle_rate([ep], 6, 1)
    return {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "%d k points spread over the 2485-point mesh of contour energy 19 (full CPA pass), "
                      "%.1f s wall" % (pts, t),
            "single_core": {"value": v1, "unit": UNIT, "cores": 1,
                            "sample": "%d strided k points of energy 19, %.1f s" % (p1, t1)}}


def run_reference(args, rank, ws):
    """Reference arm: the CPU algorithm on all host threads, bounded steps.
    Each step is one contour energy of the GPU arm's cycle, sampled by one k
    point per thread spread evenly over that energy's mesh; a single-core
    figure follows on a smaller sample of the first steps."""
    if rank != 0:
        return
    nth = os.cpu_count() or 1
    from skkr_budapest_gb300 import workloads as W
    spec = W.rel_bcc()
    eps = [W.energy_problem(spec, STEP_ENERGIES[i % len(STEP_ENERGIES)]) for i in range(args.steps + args.warmup)]
    per_step = nth
    _oracle_rate(eps[:args.warmup], per_step, nth)
    v, pts, dt = _oracle_rate(eps[args.warmup:], per_step, nth)
    v1, p1, t1 = _oracle_rate(eps[args.warmup:args.warmup + 3], 2, 1)
    sample = "%d k points per step spread evenly over the energy's mesh, %d steps" % (per_step, args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "step": "one contour energy of the cycle, strided k sample (CPU)",
                       "so_split": spec.so_split, "alloy_layers": 0, "l2": "host run"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port", "sample": sample,
                             "single_core": {"value": v1, "unit": UNIT, "cores": 1,
                                             "sample": "2 strided k points of each of 3 steps, %.1f s" % t1}},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def timed_steps(ctx, order, slot_of, eps, args, flush, stats=False):
    """Run warmup + timed steps on staged slots; device time from CUDA events
    on the library stream (max over ranks done by the caller)."""
    import torch
    from skkr_budapest_gb300 import native as N
    for i in range(args.warmup):
        ctx.run_slot(slot_of[order[i]])
    torch.cuda.synchronize()
    if stats:
        N.kernel_stats_start()
    t_dev, pts, launches, dec_iters, resid, fallbacks, kfp64, refined, alg = 0.0, 0, 0, 0, 0.0, 0, 0, 0, 0.0
    host_ops = 0
    w0 = time.perf_counter()
    for i in range(args.steps):
        ie = order[args.warmup + i]
        l2_flush(flush)
        torch.cuda.synchronize()
        st = ctx.run_slot(slot_of[ie])
        t_dev += st.run_ms
        pts += eps[ie].nk
        launches += st.gpu_launches
        dec_iters += st.dec_iters_total
        resid = max(resid, st.max_refine_resid)
        fallbacks += st.inv_fallbacks
        refined += st.inv_refined
        kfp64 += st.k_fp64
        alg += st.alg_flops
        host_ops += st.gpu_launches - st.graph_kernels + st.graph_launches
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    ks = N.kernel_stats_stop() if stats else None
    return dict(t_dev=t_dev, pts=pts, launches=launches, dec_iters=dec_iters, wall=wall, ks=ks, resid=resid,
                fallbacks=fallbacks, kfp64=kfp64, refined=refined, alg=alg, host_ops=host_ops)


def roofline(ks, precision, alg_flops, t_dev_ms):
    """Roofline of the dominant kernel class (live CUDA events, taken in a
    separate pass from the timed one).  For the sliced products `achieved` is
    FP64-equivalent algorithmic FLOP/s (8 n^2 K per complex product) against
    the measured BF16 tensor peak; the BF16 rate of all slice pairs is kept
    as `tensor_pipe`.  `step` gives the whole path's FP64-equivalent rate in
    the reference's operation count over the timed device time."""
    dom = max(ks.items(), key=lambda kv: kv[1]["ms"])
    name, d = dom
    # DRAM bytes of one launch from the committed ncu capture, scaled to this
    # run's average work per launch (traffic grows with the matrices processed)
    tr = traffic_from_profiles().get(name)
    traffic = None
    if tr and d["launches"]:
        traffic = tr["dram_bytes"] * (d["work"] / d["launches"]) / tr["work"]
    peaks = {}
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    bf16 = peaks.get("bf16_tflops", 1889.5)
    fp64 = fp64_peak_tflops()
    if name in ("gk_ft", "other"):
        peak = peaks.get("hbm_gbs", 6800.0)
        ach = d["work"] / (d["ms"] * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "traffic": traffic, "kernel": name}
    elif name == "ozaki":
        ach = d["work_fp64eq"] / (d["ms"] * 1e-3) / 1e12
        pipe = d["work"] / (d["ms"] * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16,
                "traffic": traffic, "kernel": "k_ozaki (sliced complex GEMM, tcgen05)",
                "achieved_is": "FP64-equivalent algorithmic FLOP/s (8 n^2 K per complex product)",
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst); frac is of measured",
                "tensor_pipe": {"bf16_tflops": pipe, "frac": pipe / bf16,
                                "counts": "every BF16 slice-pair MMA, S(S+1)/2 per product"}}
    else:
        ach = d["work"] / (d["ms"] * 1e-3) / 1e12
        roof = {"bound": "fp64", "achieved": ach, "peak": fp64, "unit": "TFLOP/s", "frac": ach / fp64,
                "traffic": traffic, "kernel": name,
                "peak_source": "cuBLAS ZGEMM 2048^3 measured in this run (no FP64 figure in MEASURED_PEAKS.json)"}
    step = alg_flops / (t_dev_ms * 1e-3) / 1e12
    roof["step"] = {"fp64eq_tflops": step, "frac_of_bf16_peak": step / bf16, "fp64_zgemm_peak": fp64,
                    "x_fp64_peak": step / fp64,
                    "counts": "[2 (9 it_dec + 3) + (7 nprc - 6) n_cpa] 8 n^3 per (E,k) with the executed "
                              "iteration counts, over the timed device time"}
    tot = max(1e-9, sum(x["ms"] for x in ks.values()))
    roof["per_kernel"] = {k: {"launches": v["launches"], "ms": round(v["ms"], 3), "share": round(v["ms"] / tot, 4)}
                          for k, v in ks.items()}
    roof["per_kernel_source"] = "a separate pass over the same steps with per-launch CUDA events"
    return roof


def run_ours(args, rank, ws):
    import torch
    from skkr_budapest_gb300 import api, native as N
    from skkr_budapest_gb300 import workloads as W
    torch.cuda.init()
    energies = [int(x) for x in args.energies.split(",")] if args.energies else STEP_ENERGIES
    spec = W.rel_bcc()
    nsteps = args.steps + args.warmup
    split_k = args.split == "k" and ws > 1
    # energy split: rank r starts its energy cycle at offset r (weak scaling,
    # every rank its own energies); k split: every rank every energy, its own
    # k points (the reference's modulo(ik-1, nprocs) split), strong scaling
    order = [energies[((0 if split_k else rank) + i) % len(energies)] for i in range(nsteps)]
    eps = {ie: W.energy_problem(spec, ie) for ie in set(order)}
    mine = {ie: api.ksplit_problem(ep, rank, ws) for ie, ep in eps.items()} if split_k else eps

    def context(precision):
        c = api.Context.for_problem(eps[order[0]], precision=precision, slices=args.slices)
        if precision == "mixed":
            c.set_newton(args.newton)
        if split_k:
            c.set_reduce_device(api.torch_allreduce_device())
        return c

    ctx = context(args.precision)
    if args.profile:
        # launch lists under ncu: the same kernels from the host-driven loop,
        # no conditional graph nodes to step through
        ctx.set_graphs(False)
    slot_of = {}
    for ie in order:
        if ie not in slot_of:
            slot_of[ie] = len(slot_of)
            ctx.stage_slot(slot_of[ie], mine[ie])
    flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    barrier(ws)
    clocks = Clocks()
    clocks.start()
    r = timed_steps(ctx, order, slot_of, eps, args, flush)
    clk = clocks.stop()
    if args.profile:
        ctx.close()
        print(json.dumps({"profile_run": True, "points": r["pts"], "device_ms": r["t_dev"],
                          "launches": r["launches"]}))
        return
    barrier(ws)
    t_max = max_over_ranks(r["t_dev"], ws)
    # k split: the ranks share each energy's points, counted once
    pts_all = r["pts"] if split_k else sum_over_ranks(r["pts"], ws)
    value = pts_all / (t_max * 1e-3)

    # the same steps through the plain FP64 GPU path: the metric's denominator,
    # and the error of the k-summed tau against it
    fp64 = None
    if args.precision == "mixed" and not args.no_fp64_compare:
        timed = order[args.warmup:]
        if args.fp64_ref and os.path.exists(args.fp64_ref):
            z = np.load(args.fp64_ref)
            ref_tau = {int(ie): z["tau_%d" % ie] for ie in set(timed)}
            r64 = {"t_dev": float(z["t_dev"])}
        else:
            cref = context("fp64")
            for ie, sl in slot_of.items():
                cref.stage_slot(sl, mine[ie])
            r64 = timed_steps(cref, order, slot_of, eps, args, flush)
            ref_tau = {ie: cref.fetch_slot(slot_of[ie])["tauc"] for ie in set(timed)}
            cref.close()
            if args.fp64_ref:
                np.savez(args.fp64_ref, t_dev=r64["t_dev"], **{"tau_%d" % ie: v for ie, v in ref_tau.items()})
        errs = []
        for ie in set(timed):
            a = ctx.fetch_slot(slot_of[ie])["tauc"]
            b = ref_tau[ie]
            errs.append(float(np.linalg.norm(a - b) / np.linalg.norm(b)))
        t64 = max_over_ranks(r64["t_dev"], ws)
        v64 = pts_all / (t64 * 1e-3)
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": t64 / args.steps, "speedup": value / v64,
                "max_rel_err_tau_vs_fp64": max(errs) if errs else None}

    # e2e: the reference-facing call with host buffers, same steps
    barrier(ws)
    e0 = time.perf_counter()
    h2d = d2h = 0
    for i in range(args.steps):
        ie = order[args.warmup + i]
        rr = ctx.cpacoord(mine[ie])
        h2d += rr["h2d_bytes"]
        d2h += rr["d2h_bytes"]
    torch.cuda.synchronize()
    e_wall = max_over_ranks(time.perf_counter() - e0, ws)
    e2e = pts_all / e_wall

    # the G_scr(R) tables of the timed energies (the screened real-space
    # structure constants the path Fourier-transforms per k) are host work:
    # their build, in parallel over the host cores, is reported with the
    # device time it adds to
    nw = max(1, min(16, (os.cpu_count() or 1) // max(1, ws)))
    try:
        t_tab = W.table_build_seconds(spec, order[args.warmup:], nw)
    except Exception:   # a host that cannot spawn workers builds them serially
        nw = 1
        t_tab = W.table_build_seconds(spec, order[args.warmup:], 1)
    t_tab = max_over_ranks(t_tab, ws)
    tables = {"seconds": round(t_tab, 3), "workers": nw,
              "what": "G_scr(R) screened real-space tables of the timed energies, built on the host cores",
              "value_incl_tables": pts_all / (t_max * 1e-3 + t_tab)}
    if fp64 is not None:
        fp64["value_incl_tables"] = pts_all / (t64 * 1e-3 + t_tab)

    # kernel shares: the same steps again with per-launch events (not timed)
    rs = timed_steps(ctx, order, slot_of, eps, args, flush, stats=True)
    roof = roofline(rs["ks"], args.precision, r["alg"], r["t_dev"])
    roof["gj_layouts"] = N.autotune(report=True)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "strong" if split_k else "weak", "vs_baseline": None,
            "dtype": "c128" if args.precision == "fp64" else
            "c128 via BF16x%d slices + FP64 refinement" % (args.slices or 6),
            "data": "synthetic (seeded square wells, real-space screened structure constants)",
            "config": {"workload": WORKLOAD, "precision": args.precision,
                       "step": "one contour energy, all k, full CPA pass",
                       "slices": args.slices or 6, "newton_steps": args.newton,
                       "parallelism": ("k split over %d ranks, NCCL allreduce per CPA iteration" % ws) if split_k
                       else "energies over %d ranks" % ws,
                       "step_energies": order[args.warmup:], "points": r["pts"],
                       "so_split": spec.so_split, "alloy_layers": len(spec.alloy_layers),
                       "screening": "%.1f Ry in spheres of %.4f d_NN (the reference's bcc sample: "
                                    "Wigner-Seitz spheres)" % (spec.vscreen, spec.rscreen),
                       "launches_per_energy": r["launches"] / max(1, args.steps),
                       "host_launch_ops_per_energy": r["host_ops"] / max(1, args.steps),
                       "l2": "256 MB buffer written between steps; per-step working set > 1 GB",
                       "wall_s": round(r["wall"], 3), "dec_iters": r["dec_iters"],
                       "max_newton_resid": r["resid"], "inverses_redone_in_fp64": r["fallbacks"],
                       "inverses_with_further_newton_steps": r["refined"],
                       "k_points_redone_in_fp64": r["kfp64"]},
            "fp64_gpu": fp64,
            "roofline": roof, "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
                                      "d2h_bytes_per_step": d2h // args.steps},
            "gpu_launches": r["launches"], "clocks": clk, "host_tables": tables}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(os.cpu_count() or 1)
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


C3_METRIC = "(E,k) points/s of three interface systems in one call"
C3_WORKLOAD = "c3: rel_bcc lmax3 PL4 + nonrel fcc lmax2 PL2 + rel bcc lmax2 PL3"


def _c3_setup():
    from skkr_budapest_gb300 import workloads as W
    specs = [W.rel_bcc(), W.nonrel_pl2(), W.rel_pl3_l2()]
    plan = [[12, 16, 4, 14, 8], [12, 14, 6, 10, 3], [14, 17, 8, 12, 4]]
    return plan, [[W.energy_problem(sp, ie) for ie in pl] for sp, pl in zip(specs, plan)]


def run_c3_reference(args):
    """Reference arm of the three-system workload: the oracle's CPA and k loop
    of every system on all host threads, a bounded sample of k points per
    energy and system."""
    nth = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    plan, eps = _c3_setup()
    per_step = nth

    def step(i):
        pts = 0
        for e in eps:
            ep = e[i % len(e)]
            sub = strided(ep, per_step)
            if O.cpacoord(sub, nthreads=nth)["status"] != 0:
                raise RuntimeError("oracle failed")
            pts += len(sub.xk)
        return pts

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    pts = sum(step(i) for i in range(args.warmup, args.warmup + args.steps))
    dt = time.perf_counter() - t0
    v = pts / dt
    print(json.dumps({"impl": "reference", "metric": C3_METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
                      "data": "synthetic (seeded)",
                      "config": {"workload": C3_WORKLOAD, "energies": plan,
                                 "step": "%d k points spread over the mesh of one energy of each system (CPU)" % per_step},
                      "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                                       "sample": "%d k points per system and step, %d steps" % (per_step,
                                                                                              args.steps)},
                      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


def run_c3(args):
    """Three interfaces in one call per step (relativistic PL4 lmax=3,
    non-relativistic PL2 lmax=2, relativistic PL3 lmax=2), host buffers in and
    out, against the same calls made one after the other."""
    import torch
    from skkr_budapest_gb300 import api
    plan, eps = _c3_setup()
    ctxs = [api.Context.for_problem(e[0], args.precision) for e in eps]
    nsteps = args.warmup + args.steps

    def step(i, concurrent):
        group = [e[i % len(e)] for e in eps]
        if concurrent:
            return api.cpacoord_many(group, contexts=ctxs)
        return [c.cpacoord(ep) for c, ep in zip(ctxs, group)]

    out = {}
    for mode in (True, False):
        for i in range(args.warmup):
            step(i, mode)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pts = 0
        for i in range(args.warmup, nsteps):
            step(i, mode)
            pts += sum(e[i % len(e)].nk for e in eps)
        torch.cuda.synchronize()
        out[mode] = (pts, time.perf_counter() - t0)
    for c in ctxs:
        c.close()
    v = out[True][0] / out[True][1]
    seq = out[False][0] / out[False][1]
    print(json.dumps({"metric": C3_METRIC, "value": v,
                      "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * out[True][1] / args.steps, "higher_is_better": True,
                      "dtype": "c128 via BF16x6 slices" if args.precision == "mixed" else "c128",
                      "data": "synthetic", "sequential_value": seq, "concurrency_gain": v / seq,
                      "config": {"workload": C3_WORKLOAD,
                                 "precision": args.precision, "energies": plan,
                                 "timing": "host wall clock around whole calls (host buffers)"}}), flush=True)


C4_METRIC = "(E,k) points/s of CPA alloy interfaces converged to cpatol 1e-10"
C4_WORKLOAD = ("c4: relativistic bcc(001) PL4 lmax=3 interface with 4 alloy layers A_c B_(1-c), c ~ U[0.1, 0.9], "
               "depths ~ U[-1.2, -0.4] Ry drawn per step (held-out draws), contour energies cycled, IBZ mesh of "
               "the surrogate's family")


def _c4_steps(nsteps, seed=9001):
    from skkr_budapest_gb300 import cpa_warmstart as CW
    model = CW.Model()
    fam = model.family()
    rng = np.random.default_rng(seed)
    eps = [fam.problem(fam.energies[i % len(fam.energies)], fam.draw(rng)) for i in range(nsteps)]
    return model, fam, eps


def run_c4_reference(args):
    """Reference arm of the alloy workload: the oracle's CPA loop on all host
    threads, one k point per thread spread over each step's mesh."""
    nth = os.cpu_count() or 1
    _, _, eps = _c4_steps(args.warmup + args.steps)
    _oracle_rate(eps[:args.warmup], nth, nth)
    v, pts, dt = _oracle_rate(eps[args.warmup:], nth, nth)
    print(json.dumps({"impl": "reference", "metric": C4_METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
                      "data": "synthetic (seeded)",
                      "config": {"workload": C4_WORKLOAD, "start": "ATA (tata)",
                                 "step": "one alloy stack at one energy, strided k sample (CPU)"},
                      "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                                       "sample": "%d k points per step, %d steps" % (nth, args.steps)},
                      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


def run_c4(args):
    """Alloy interfaces converged to cpatol 1e-10 through the reference-facing
    call with host buffers: the FP64 path and the split-precision path from
    the ATA start, and the split-precision path from the learned start (the
    surrogate's inference and the start's assembly inside the timed region).
    value = the last; the CPA iterations of each are reported."""
    import torch
    from skkr_budapest_gb300 import api, cpa_warmstart as CW
    model, fam, eps = _c4_steps(args.warmup + args.steps)
    out = {}
    for name, prec, learned in (("fp64", "fp64", False), ("mixed", "mixed", False), ("mixed_mlp", "mixed", True)):
        ctx = api.Context.for_problem(eps[0], prec)
        for ep in eps[:args.warmup]:
            ctx.cpacoord(ep, tminv=CW.warm_start(ep, model, fam) if learned else None)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pts, its, dev, res, h2d, d2h = 0, 0, 0.0, [], 0, 0
        for ep in eps[args.warmup:]:
            r = ctx.cpacoord(ep, tminv=CW.warm_start(ep, model, fam) if learned else None)
            pts += ep.nk
            its += r["cpa_iterations"]
            dev += r["run_ms"]
            h2d += r["h2d_bytes"]
            d2h += r["d2h_bytes"]
            res.append(r["tauc"])
        torch.cuda.synchronize()
        out[name] = dict(wall=time.perf_counter() - t0, pts=pts, its=its, dev=dev, tau=res, h2d=h2d, d2h=d2h)
        ctx.close()
    ref = out["fp64"]["tau"]
    err = {k: max(float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(out[k]["tau"], ref))
           for k in ("mixed", "mixed_mlp")}
    rate = {k: v["pts"] / v["wall"] for k, v in out.items()}
    line = {"metric": C4_METRIC, "value": rate["mixed_mlp"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * out["mixed_mlp"]["wall"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128 via BF16 slices + FP64 refinement; surrogate BF16 weights, FP32 accumulation",
            "data": "synthetic (seeded, held-out alloy draws)",
            "config": {"workload": C4_WORKLOAD, "nset": fam.nset, "k_points_per_step": eps[0].nk,
                       "so_split": fam.so_split, "cpatol": eps[0].cpatol,
                       "timing": "host wall clock around whole calls (host buffers), surrogate included"},
            "paths": {k: {"value": rate[k], "cpa_iterations": out[k]["its"], "device_ms": round(out[k]["dev"], 1),
                          # the learned start converges to cpatol from another
                          # point: its difference from the ATA-started FP64 run
                          # is the spread of converged solutions, not rounding
                          ("max_rel_diff_tau_vs_fp64_from_ata" if k == "mixed_mlp" else
                           "max_rel_err_tau_vs_fp64"): err.get(k)} for k in out},
            "speedup_vs_fp64": rate["mixed_mlp"] / rate["fp64"],
            "cpa_iterations_learned_vs_ata": out["mixed_mlp"]["its"] / max(1, out["mixed"]["its"]),
            "e2e": {"value": rate["mixed_mlp"], "unit": UNIT, "h2d_bytes_per_step": out["mixed_mlp"]["h2d"] // args.steps,
                    "d2h_bytes_per_step": out["mixed_mlp"]["d2h"] // args.steps}}
    print(json.dumps(line), flush=True)


C1_METRIC = "(E,k) points/s of the plain non-relativistic interface (k-summed tau within 1e-9 of FP64)"
C1_WORKLOAD = ("c1: fcc(001) a = 6.8, lmax = 2, PL2 (n_PL = 18), 6-layer interface between identical bulks, "
               "16 contour energies, 253-point IBZ meshes (nset 22), all energies and k points every step")


def _c1_problems():
    from skkr_budapest_gb300 import workloads as W
    spec = W.plain_fcc()
    return [W.energy_problem(spec, ie) for ie in range(len(spec.energies))]


def run_c1(args):
    """The plain non-relativistic interface (the reference's own CPU-sized
    case): one step = the whole 16-energy contour with full meshes through
    skkr_gpu_cpacoord with host buffers, FP64 and split precision; the error
    of the k-summed tau of the split path against FP64."""
    import torch
    from skkr_budapest_gb300 import api
    eps = _c1_problems()
    out, tau = {}, {}
    for prec in ("fp64", "mixed"):
        ctx = api.Context.for_problem(eps[0], prec)
        for _ in range(args.warmup):
            for ep in eps:
                ctx.cpacoord(ep)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pts, dev = 0, 0.0
        for _ in range(args.steps):
            for ie, ep in enumerate(eps):
                r = ctx.cpacoord(ep)
                pts += ep.nk
                dev += r["run_ms"]
                tau[(prec, ie)] = r["tauc"]
        torch.cuda.synchronize()
        out[prec] = dict(wall=time.perf_counter() - t0, pts=pts, dev=dev)
        ctx.close()
    err = max(float(np.linalg.norm(tau[("mixed", ie)] - tau[("fp64", ie)]) / np.linalg.norm(tau[("fp64", ie)]))
              for ie in range(len(eps)))
    rate = {k: v["pts"] / (v["dev"] * 1e-3) for k, v in out.items()}
    print(json.dumps({"metric": C1_METRIC, "value": rate["mixed"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": out["mixed"]["dev"] / args.steps,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "c128 via BF16x6 slices + FP64 refinement", "data": "synthetic (seeded)",
                      "config": {"workload": C1_WORKLOAD, "points_per_step": out["mixed"]["pts"] // args.steps},
                      "fp64_value": rate["fp64"], "speedup": rate["mixed"] / rate["fp64"],
                      "max_rel_err_tau_vs_fp64": err,
                      "e2e": {"value": out["mixed"]["pts"] / out["mixed"]["wall"], "unit": UNIT,
                              "fp64_value": out["fp64"]["pts"] / out["fp64"]["wall"],
                              "h2d_bytes_per_step": None, "d2h_bytes_per_step": None}}), flush=True)


def run_c1_reference(args):
    """Reference arm of the plain interface: the oracle's CPA and k loop over
    the whole contour with full meshes (no sample: the case runs on a CPU in
    seconds), all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    nth = os.cpu_count() or 1
    eps = _c1_problems()
    for _ in range(args.warmup):
        for ep in eps:
            O.cpacoord(ep, nthreads=nth)
    t0 = time.perf_counter()
    pts = 0
    for _ in range(args.steps):
        for ep in eps:
            if O.cpacoord(ep, nthreads=nth)["status"] != 0:
                raise RuntimeError("oracle failed on the c1 workload")
            pts += ep.nk
    dt = time.perf_counter() - t0
    v = pts / dt
    print(json.dumps({"impl": "reference", "metric": C1_METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
                      "data": "synthetic (seeded)", "config": {"workload": C1_WORKLOAD},
                      "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                                       "sample": "the whole workload, %d steps" % args.steps},
                      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


C5_METRIC = "(E,k) points/s of the BdG interface (anomalous block within 1e-9 of FP64)"
C5_ENERGIES = [8, 24, 40, 56]
C5_NSET = 12


def _c5_problems():
    from skkr_budapest_gb300 import workloads as W
    spec = W.bdg_bcc()
    return spec, {ie: W.energy_problem(spec, ie, nset=C5_NSET) for ie in C5_ENERGIES}


def run_c5(args):
    """The Bogoliubov-de Gennes interface of config C5 (electron + hole
    (kappa,mu) blocks, lmax=3, PL4: n_PL = 256, 12 layers, Im E = 1e-4 Ry)
    on a bounded sample: 4 of its 64 energies, 78-point IBZ meshes.  FP64 and
    split precision (near the axis the decimation stays FP64 by policy, tau2d
    runs split), through skkr_gpu_cpacoord_bdg with host buffers; the error
    of the k-summed tau and of its electron-hole block against FP64."""
    import torch
    from skkr_budapest_gb300 import api
    spec, eps = _c5_problems()
    order = [C5_ENERGIES[i % len(C5_ENERGIES)] for i in range(args.warmup + args.steps)]
    out, tau = {}, {}
    for prec in ("fp64", "mixed"):
        ctx = api.Context.for_problem(eps[order[0]], prec)
        for ie in order[:args.warmup]:
            ctx.cpacoord(eps[ie])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pts, dev, kfp = 0, 0.0, 0
        for ie in order[args.warmup:]:
            r = ctx.cpacoord(eps[ie])
            pts += eps[ie].nk
            dev += r["run_ms"]
            kfp += r["k_fp64"]
            tau[(prec, ie)] = r["tauc"]
        torch.cuda.synchronize()
        out[prec] = dict(wall=time.perf_counter() - t0, pts=pts, dev=dev, kfp=kfp)
        ctx.close()
    km = eps[order[0]].lkmax // 2
    err = err_eh = 0.0
    for ie in set(order[args.warmup:]):
        a, b = tau[("mixed", ie)], tau[("fp64", ie)]
        err = max(err, float(np.linalg.norm(a - b) / np.linalg.norm(b)))
        e, f = a[:, :km, km:], b[:, :km, km:]
        err_eh = max(err_eh, float(np.linalg.norm(e - f) / np.linalg.norm(f)))
    rate = {k: v["pts"] / (v["dev"] * 1e-3) for k, v in out.items()}
    print(json.dumps({"metric": C5_METRIC, "value": rate["mixed"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": out["mixed"]["dev"] / args.steps,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "c128 via BF16 slices (electron and hole K halves) + FP64 refinement",
                      "data": "synthetic (seeded)",
                      "config": {"workload": "c5: BdG bcc(001) lmax=3 PL4 (n_PL = 256), 12 layers, delta = 1e-3 Ry, "
                                             "Im E = 1e-4 Ry, energies %s of 64, %d k each" %
                                             (C5_ENERGIES, eps[order[0]].nk),
                                 "sample": "4 of the 64 energies on 78-point meshes (40000 k per energy would take "
                                           "about half an hour per energy with the FP64 decimation near the axis)"},
                      "fp64_value": rate["fp64"], "speedup": rate["mixed"] / rate["fp64"],
                      "k_points_redone_in_fp64": out["mixed"]["kfp"],
                      "policy": "decimation in FP64 below Im E = 2e-4 Ry; blocks above 128 rows there: the whole "
                                "energy in FP64",
                      "max_rel_err_tau_vs_fp64": err, "max_rel_err_anomalous_block_vs_fp64": err_eh,
                      "e2e": {"value": out["mixed"]["pts"] / out["mixed"]["wall"], "unit": UNIT,
                              "h2d_bytes_per_step": None, "d2h_bytes_per_step": None}}), flush=True)


def run_c5_reference(args):
    """Reference arm of the BdG workload: the oracle's CPA and k loop on all
    host threads, one k point per thread spread over each energy's mesh."""
    nth = os.cpu_count() or 1
    _, eps = _c5_problems()
    order = [C5_ENERGIES[i % len(C5_ENERGIES)] for i in range(args.warmup + args.steps)]
    _oracle_rate([eps[ie] for ie in order[:args.warmup]], nth, nth)
    v, pts, dt = _oracle_rate([eps[ie] for ie in order[args.warmup:]], nth, nth)
    print(json.dumps({"impl": "reference", "metric": C5_METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
                      "data": "synthetic (seeded)",
                      "config": {"workload": "c5 (see the GPU arm)", "step": "strided k sample of one energy (CPU)"},
                      "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                                       "sample": "%d k points per step, %d steps" % (nth, args.steps)},
                      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


GK_METRIC = "(E,k) points/s of the C2 path with the reference's k-space G_scr(k)"


def run_gk(args):
    """The relativistic PL4 lmax=3 interface with G_scr(k) from the
    reference's own form (Kambe lattice sums of the slab's distinct layer
    separations, slab screening, skkr_gpu_stage_kambe) against the same
    energies on the table transform: (E,k)/s of each, the time of the G(k)
    build, and the relative difference of the k-summed tau between the two
    formulations (the truncation of the three-shell table, not an error)."""
    import torch
    from skkr_budapest_gb300 import api, kspace
    from skkr_budapest_gb300 import workloads as W
    spec = W.rel_bcc()
    plan = [4, 8, 12, 16, 18]
    order = [plan[i % len(plan)] for i in range(args.warmup + args.steps)]
    eps = {ie: W.energy_problem(spec, ie) for ie in set(order)}
    forms = {ie: kspace.kambe_form(ep, spec, nl=args.slab) for ie, ep in eps.items()}
    out, tau = {}, {}
    for name in ("table", "kambe"):
        ctx = api.Context.for_problem(eps[order[0]], args.precision)
        run = (lambda ie: ctx.cpacoord_kambe(eps[ie], forms[ie])) if name == "kambe" else \
            (lambda ie: ctx.cpacoord(eps[ie]))
        for ie in order[:args.warmup]:
            run(ie)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pts, dev = 0, 0.0
        for ie in order[args.warmup:]:
            r = run(ie)
            pts += eps[ie].nk
            dev += r["run_ms"]
            tau[(name, ie)] = r["tauc"]
        torch.cuda.synchronize()
        out[name] = dict(wall=time.perf_counter() - t0, pts=pts, dev=dev)
        ctx.close()
    diff = max(float(np.linalg.norm(tau[("kambe", ie)] - tau[("table", ie)]) / np.linalg.norm(tau[("kambe", ie)]))
               for ie in set(order[args.warmup:]))
    rate = {k: v["pts"] / (v["dev"] * 1e-3) for k, v in out.items()}
    print(json.dumps({"metric": GK_METRIC, "value": rate["kambe"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": out["kambe"]["dev"] / args.steps,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "c128" if args.precision == "fp64" else "c128 via BF16 slices + FP64 refinement",
                      "data": "synthetic (seeded)",
                      "config": {"workload": "rel_bcc001_lmax3_pl4 energies %s, full meshes" % plan,
                                 "slab_layers": args.slab, "slab_rows": args.slab * 16,
                                 "screening": "%.1f Ry, %.4f d_NN" % (spec.vscreen, spec.rscreen),
                                 "precision": args.precision},
                      "table_value": rate["table"], "kambe_over_table_time": out["kambe"]["dev"] / out["table"]["dev"],
                      "max_rel_diff_tau_kambe_vs_table": diff,
                      "e2e": {"value": out["kambe"]["pts"] / out["kambe"]["wall"], "unit": UNIT,
                              "h2d_bytes_per_step": None, "d2h_bytes_per_step": None}}), flush=True)


TAUIJ_METRIC = "(E,k) points/s of the off-diagonal interface tau (skkr_gpu_tauij)"
TAUIJ_WORKLOAD = ("off-diagonal tau of the relativistic bcc(001) PL4 lmax=3 interface: 144 layer pairs at R = 0 "
                  "and the 4 nearest in-plane cells of every layer (192 pairs), contour energies 12 16 14 19 13")


def _tauij_setup():
    from skkr_budapest_gb300 import synth as S
    from skkr_budapest_gb300 import workloads as W
    spec = W.rel_bcc()
    plan = [12, 16, 14, 19, 13]
    eps = {ie: W.energy_problem(spec, ie) for ie in plan}
    ep0 = eps[plan[0]]
    n, a2d, l0 = ep0.nintfc, spec.stacking.a2d, int(ep0.ninprc[0])
    cvec = np.array([[0.5 * ((l0 + l) % 2) * a2d] * 2 for l in range(n)])
    pairs = [(0, 0, a, b) for a in range(n) for b in range(n)]
    pairs += [(d1, d2, a, a) for (d1, d2) in ((1, 0), (0, 1), (-1, 0), (0, -1)) for a in range(n)]
    a0mat = [o[:2, :2].T.ravel() for o in S.c4v_ops()]
    return plan, eps, pairs, [a2d, 0.0], [0.0, a2d], cvec, a0mat


def run_tauij_reference(args):
    """Reference arm of the off-diagonal tau: the oracle's tau2d_god and pair
    sums on all host threads, a bounded sample of k points per energy."""
    nth = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    plan, eps, pairs, a1, a2, cvec, a0mat = _tauij_setup()
    order = [plan[i % len(plan)] for i in range(args.warmup + args.steps)]
    per_step = nth

    def step(ep):
        sub = ep.with_k(ep.xk[:per_step], ep.wk[:per_step] / ep.wk[:per_step].sum())
        if O.tauij(sub, pairs, a1, a2, cvec, a0mat, nthreads=nth)["status"] != 0:
            raise RuntimeError("oracle failed")
        return len(sub.xk)

    for ie in order[:args.warmup]:
        step(eps[ie])
    t0 = time.perf_counter()
    pts = sum(step(eps[ie]) for ie in order[args.warmup:])
    dt = time.perf_counter() - t0
    v = pts / dt
    print(json.dumps({"impl": "reference", "metric": TAUIJ_METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
                      "data": "synthetic (seeded)",
                      "config": {"workload": TAUIJ_WORKLOAD, "step": "%d k points of one energy (CPU)" % per_step},
                      "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                                       "sample": "%d k points per step, %d steps" % (per_step, args.steps)},
                      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


def run_tauij(args):
    """Off-diagonal tau of the relativistic PL4 lmax=3 interface for cluster
    embedding: per step one contour energy through skkr_gpu_tauij (G(k),
    decimation, full Godfrin tau, phased pair sums over all 144 layer pairs
    at R = 0 and the 4 nearest in-plane cells), split precision against FP64,
    host buffers in and out."""
    import torch
    from skkr_budapest_gb300 import api
    plan, eps, pairs, a1, a2, cvec, a0mat = _tauij_setup()
    ep0 = eps[plan[0]]
    a2d = a1[0]
    out = {}
    res = {}
    for prec in ("mixed", "fp64"):
        ctx = api.Context.for_problem(ep0, prec)
        order = [plan[i % len(plan)] for i in range(args.warmup + args.steps)]
        for ie in order[:args.warmup]:
            ctx.tauij(eps[ie], pairs, [a2d, 0.0], [0.0, a2d], cvec, a0mat)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pts = 0
        for ie in order[args.warmup:]:
            res[(prec, ie)] = ctx.tauij(eps[ie], pairs, [a2d, 0.0], [0.0, a2d], cvec, a0mat)
            pts += eps[ie].nk
        torch.cuda.synchronize()
        out[prec] = (pts, time.perf_counter() - t0)
        ctx.close()
    err = 0.0
    for ie in set(order[args.warmup:]):
        a, b = res[("mixed", ie)], res[("fp64", ie)]
        scale = np.abs(b["tau_ij"]).max()
        err = max(err, float(np.abs(a["tau_ij"] - b["tau_ij"]).max() / scale),
                  float(np.abs(a["tau_ji"] - b["tau_ji"]).max() / scale))
    v = out["mixed"][0] / out["mixed"][1]
    v64 = out["fp64"][0] / out["fp64"][1]
    print(json.dumps({"metric": TAUIJ_METRIC,
                      "value": v, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * out["mixed"][1] / args.steps, "higher_is_better": True,
                      "dtype": "c128 via BF16x6 slices + FP64 refinement", "data": "synthetic",
                      "fp64_value": v64, "speedup": v / v64,
                      "max_abs_err_vs_fp64_rel_to_largest_block": err,
                      "config": {"workload": TAUIJ_WORKLOAD, "pairs": len(pairs), "energies": order[args.warmup:],
                                 "timing": "host wall clock around whole calls (host buffers)"}}), flush=True)


def main():
    args = parse()
    if args.workload == "c1":
        if args.impl == "reference":
            run_c1_reference(args)
        else:
            run_c1(args)
        return
    if args.workload == "c3":
        if args.impl == "reference":
            run_c3_reference(args)
        else:
            run_c3(args)
        return
    if args.workload == "tauij":
        if args.impl == "reference":
            run_tauij_reference(args)
        else:
            run_tauij(args)
        return
    if args.workload == "c4":
        if args.impl == "reference":
            run_c4_reference(args)
        else:
            run_c4(args)
        return
    if args.workload == "c5":
        if args.impl == "reference":
            run_c5_reference(args)
        else:
            run_c5(args)
        return
    if args.workload == "gk":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "metric": GK_METRIC,
                              "unavailable": "the reference's Kambe G(k) has no CPU arm here: the oracle restates it "
                                             "in numpy per k point (test infrastructure, minutes per k)"}))
        else:
            run_gk(args)
        return
    rank, ws = dist_init(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, ws)
    else:
        run_ours(args, rank, ws)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
