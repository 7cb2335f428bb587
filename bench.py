#!/usr/bin/env python
"""Benchmark of the GGEM particle-side hot path on GB300.

Workload (the metric's configuration): N = 200,000 beads of radius a = 1 in a
periodic cube at volume fraction phi = 0.1 (L = 203.1), GGEM alpha = 0.5/a,
local cut-off rc = 7a, seeded random non-overlapping placement and Philox
N(0,1) noise (synthetic inputs; the reference ships none of this size).

One "step" is one Brownian step of the local mobility, the particle-side
part of Copss::fixman_integrate (copss.C:1560-1686):
  cell list + pair list build -> noise xi -> Chebyshev y ~ M^{-1/2} xi
  (FP32 pair sums, FP64 recurrence, err1 <= 1e-3, <= 50 terms) -> dw = M y.
The eigen interval is computed by Lanczos once and reused until the series
fails, the reference's policy (copss.C:1598-1671).

value      steps/s with positions and noise resident on the device
e2e        steps/s through the host-pointer C ABI (positions and xi copied
           in from pinned host memory, dw copied out, every step)
also       mobility matvecs/s, the plain FP64 GPU path (FP64 pair sweep,
           Lanczos every step, error check every term), FP32-vs-FP64
           velocity error, the pair kernel's roofline and the CPU baseline.

--impl reference times the reference algorithm on the host cores (the FP64
oracle restatement; the reference itself needs libMesh/PETSc/SLEPc) with all
host threads, on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "copss-hydrodynamics-private_gb300"))

METRIC = ("Brownian steps/s & mobility matvecs/s at N=200k vs plain FP64 GPU, "
          "rel err ≤1e-6")
N_BEADS = 200_000
PHI = 0.1
ALPHA = 0.5
RC = 7.0
CHEB_MAX = 50
CHEB_TOL = 1e-3
SEED = 20261203
# DRAM bytes (read + write) per launch of the dominant pair kernel from one
# ncu capture of this bench's workload (ncu flushes the caches before the
# launch, so this is the cold-cache figure): k_pair_cheb<1, 0, 0>, 70.60 MB
# read + 2.18 MB written (profile_cases.py pair_cheb)
PAIR_TRAFFIC = {"k_pair_cheb": 72.78e6}


def measured_peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        return {}


def workload_config(extra=None):
    cfg = {"workload": "Brownian step of the GGEM local mobility: N=200000 beads a=1, "
                       "phi=0.1 periodic cube, alpha=0.5, rc=7, Chebyshev tol 1e-3 <=50 terms",
           "n_beads": N_BEADS, "phi": PHI, "alpha": ALPHA, "rc": RC, "nrhs": 1,
           "cheb_max_terms": CHEB_MAX, "cheb_tol": CHEB_TOL,
           "l2": "flushed between timed steps (512 MB write); inputs are ~40 MB"}
    if extra:
        cfg.update(extra)
    return cfg


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0, period_ms=20):
        self.index = index
        self.period_ms = period_ms
        self.proc = None
        self.lines = []      # (host arrival time, csv line)
        self.windows = []    # timed regions (host perf_counter start, end)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)  # let the first samples arrive before the load starts
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def mark(self, t0, t1):
        self.windows.append((t0, t1))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def _parse(self, lines):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return sm, mx, reasons

    def summary(self):
        """Clocks of the samples taken inside the marked timed regions; when
        those regions are too short for three samples, all samples taken
        while the measured phases ran (the GPU is loaded throughout)."""
        inside = [x for x in self.lines
                  if any(t0 <= x[0] <= t1 + 0.05 for t0, t1 in self.windows)]
        sm, mx, reasons = self._parse(inside)
        scope = "timed regions"
        if len(sm) < 3:
            sm, mx, reasons = self._parse(self.lines)
            scope = "all measured phases (timed regions shorter than 3 samples)"
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm),
                "samples_in_timed_regions": len(inside), "period_ms": self.period_ms,
                "scope": scope}


# --------------------------------------------------------------------------
# replicas: every rank runs its own suspension, no collective on the data path
# --------------------------------------------------------------------------
def replica_throughput(ms_step, world, device="cuda"):
    """(max-over-ranks step time in ms, whole-job steps/s of `world`
    replicas); the only collective is this one scalar reduction."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(ms_step)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    return ms_step, 1e3 / ms_step * world


def replica_seed(rank):
    """each rank's suspension is an independent replica"""
    return SEED + rank


# --------------------------------------------------------------------------
# GB300 arm
# --------------------------------------------------------------------------
def run_gb300(args, rank, world):
    import torch
    import ggem_gb300 as G
    from ggem_gb300 import build as B

    B.build()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    L_lib = G.lib()
    import ctypes as C

    xyz, L = G.make_suspension(replica_seed(rank), N_BEADS, PHI)
    box = (L, L, L)

    def make_ctx(prec, div=1):
        return G.Context(alpha=ALPHA, box_hi=box, rc=RC, precision=prec, cell_div=div, device=dev)

    # pick the cell size of the FP32 pair list (a two-candidate autotune)
    d_xyz = torch.from_numpy(xyz.reshape(-1)).cuda()
    best = None
    for div in (1, 2):
        ctx = make_ctx(G.FP32, div)
        ctx.set_particles_dev(d_xyz.data_ptr(), N_BEADS)
        ctx.build_cells()
        f = torch.randn(3 * N_BEADS, dtype=torch.float64, device="cuda")
        u = torch.empty_like(f)
        for _ in range(3):
            ctx.local_matvec_dev(f.data_ptr(), u.data_ptr(), 1, G.SELF_BEAD)
        ctx.synchronize()
        t0 = time.perf_counter()
        for _ in range(20):
            ctx.set_particles_dev(d_xyz.data_ptr(), N_BEADS)
            ctx.build_cells()
            for _ in range(10):
                ctx.local_matvec_dev(f.data_ptr(), u.data_ptr(), 1, G.SELF_BEAD)
        ctx.synchronize()
        dt = time.perf_counter() - t0
        if best is None or dt < best[0]:
            best = (dt, div)
        ctx.close()
    cell_div = best[1]
    ctx = make_ctx(G.FP32, cell_div)
    # the library's autotuner picks stored or per-matvec pair tensors on this
    # configuration (about 12 matvecs per list build in a Brownian step)
    ctx.set_particles_dev(d_xyz.data_ptr(), N_BEADS)
    ctx.build_cells()
    use_stored, ms_comp, ms_store = ctx.autotune_pair_storage(reps=10, matvecs_per_build=12.0)
    tuning = {"cell_div": cell_div, "pair_tensors_stored": use_stored,
              "ms_per_matvec_computed": ms_comp, "ms_per_matvec_stored_amortised": ms_store,
              "pair_variants_computed_stored": list(ctx.pair_variants)}
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    # rebuilds return without waiting for the device; the list statistics
    # are read with the Chebyshev error check of the same step
    ctx.set_deferred_checks(True)

    d_xi = torch.empty(3 * N_BEADS, dtype=torch.float64, device="cuda")
    d_dw = torch.empty_like(d_xi)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    state = {"bounds": None, "lanczos_calls": 0, "surrogate_calls": 0, "reports": [],
             "source": None}
    from ggem_gb300 import surrogate_data as SD
    sur_loaded = None if args.no_surrogate else SD.load_default(device=dev)
    sur, sur_margins = (sur_loaded[0], sur_loaded[1]) if sur_loaded else (None, None)

    def lanczos(c):
        lo, hi = c.lanczos_bounds(k=24, seed=7)
        state["lanczos_calls"] += 1
        return lo / 1.05, hi * 1.05  # eig_factor widening, copss.C:1607

    def bounds(c, retry):
        # the network's interval first; Lanczos when the Chebyshev check
        # rejected the previous interval (the reference recomputes its
        # eigenvalues when the series fails, copss.C:1598-1671)
        if sur is not None and not retry:
            state["surrogate_calls"] += 1
            state["source"] = "surrogate"
            return c.surrogate_interval(sur, 0.0, sur_margins[0], sur_margins[1])
        state["source"] = "lanczos"
        return lanczos(c)

    # the timed step calls the C ABI directly (as a native driver would), so
    # that no Python wrapper work sits between its launches
    p_xyz, p_xi, p_dw = (C.c_void_p(t.data_ptr()) for t in (d_xyz, d_xi, d_dw))
    rep_buf = (G.ChebReport * 1)()

    def device_step(step_id, check_every=None):
        ce = args.check_every if check_every is None else check_every
        rc = L_lib.ggem_set_particles_dev(ctx.h, N_BEADS, p_xyz)
        rc |= L_lib.ggem_build_cells(ctx.h)
        rc |= L_lib.ggem_philox_normals_dev(ctx.h, SEED, step_id, 3 * N_BEADS, p_xi)
        if rc:
            raise RuntimeError(f"device step failed: {G.lib().ggem_last_error(ctx.h)}")
        if state["bounds"] is None:
            state["bounds"] = bounds(ctx, False)
        for attempt in range(2):
            lo, hi = state["bounds"]
            rc = L_lib.ggem_brownian_displacement_dev(ctx.h, 1, CHEB_MAX, lo, hi, CHEB_TOL,
                                                      ce, p_xi, p_dw, rep_buf)
            if rc == 0:
                state["reports"].append(bytes(rep_buf))  # parsed after the timing
                return
            state["bounds"] = bounds(ctx, True)  # recompute and retry once
        raise RuntimeError(f"Chebyshev failed twice: {rep_buf[0].as_dict()}")

    def timed(fn, steps, warmup, flush_l2=True):
        for s in range(warmup):
            fn(s)
        torch.cuda.synchronize()
        ts = []
        for s in range(steps):
            if flush_l2:
                flush.zero_()
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                a.record(stream)
                fn(warmup + s)
                b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return ts

    # ---- device-resident Brownian steps (value) --------------------------
    if world > 1:
        torch.distributed.barrier()
    ctx.set_kernel_timing(False)
    for s in range(args.warmup):
        device_step(s)
    torch.cuda.synchronize()
    clk = ClockSampler(dev).__enter__()
    # only the roofline's kernel is bracketed by events inside the timed
    # region (its consecutive launches share one event pair per step): an
    # event pair around every launch of every kind cost ~50 us per step
    ctx.set_kernel_timing(True, kinds=[G.KERNEL_PAIR_CHEB])
    lc0 = ctx.launch_count()
    t_wall0 = time.perf_counter()
    # an NVTX range around the timed device steps lets a profiler select
    # exactly their launches (ncu --nvtx --nvtx-include "brownian_steps/")
    torch.cuda.nvtx.range_push("brownian_steps")
    ts = timed(device_step, args.steps, 0)
    torch.cuda.nvtx.range_pop()
    t_wall = time.perf_counter() - t_wall0
    clk.mark(t_wall0, t_wall0 + t_wall)
    lc1 = ctx.launch_count()
    kt = {"pair_cheb": ctx.kernel_timing(G.KERNEL_PAIR_CHEB)}
    ctx.set_kernel_timing(False)
    ms_step, steps_per_s = replica_throughput(float(np.mean(ts)), world)
    # the bound sources of the timed steps (the legs below call Lanczos too)
    calls = {"surrogate_calls": state["surrogate_calls"], "lanczos_calls": state["lanczos_calls"]}
    n_pairs = ctx.pair_count()
    reps = [G.ChebReport.from_buffer_copy(b).as_dict() for b in state["reports"][-args.steps:]]

    # the other kernels of a step, each launch bracketed by its own events,
    # over a few further steps (outside the headline's timed region)
    kt_steps = min(5, args.steps)
    ctx.set_kernel_timing(True)
    timed(device_step, kt_steps, 0)
    kt_all = {name: ctx.kernel_timing(kind) for kind, name in
              ((G.KERNEL_PAIR_FP32, "pair_fp32"), (G.KERNEL_PAIR_CHEB, "pair_cheb"),
               (G.KERNEL_CHEB_TERM, "cheb_term"), (G.KERNEL_LIST_BUILD, "list_build"))}
    ctx.set_kernel_timing(False)
    kt_per_step = {k: {"ms_per_step": v[0] / kt_steps, "launches_per_step": v[1] / kt_steps}
                   for k, v in kt_all.items()}

    # ---- the reference's schedule: the err1 check after every term --------
    # (brownian_system.C:1089-1155: two matvecs per term), the same work per
    # step as the reference arm, which runs that schedule on the host
    faithful = None
    if args.check_every != 1:
        n_rep0 = len(state["reports"])
        ts_f = timed(lambda s_: device_step(s_, check_every=1), args.steps, 3)
        f_reps = [G.ChebReport.from_buffer_copy(b).as_dict() for b in state["reports"][n_rep0:]]
        f_reps = f_reps[-args.steps:]
        faithful = {"steps_per_s": 1e3 / float(np.mean(ts_f)) * world,
                    "ms_per_step": float(np.mean(ts_f)), "check_every": 1,
                    "cheb_terms": sorted({r["n_terms"] for r in f_reps}),
                    # the series' operator applications (the final dw = M y is
                    # the last check's M dw, so no further matvec)
                    "series_matvecs_per_step": float(np.mean([r["n_matvecs"] for r in f_reps])),
                    "adaptive_series_matvecs_per_step": float(np.mean([r["n_matvecs"]
                                                                       for r in reps]))}

    # ---- e2e through the host-pointer ABI --------------------------------
    h_xyz = torch.from_numpy(xyz.reshape(-1).copy()).pin_memory()
    h_dw = torch.empty(3 * N_BEADS, dtype=torch.float64).pin_memory()
    xi_host = [torch.from_numpy(G.make_normals(SEED + 1000 + s, 3 * N_BEADS)).pin_memory()
               for s in range(args.steps + args.warmup)]
    ctx_e = make_ctx(G.FP32, cell_div)
    ctx_e.set_pair_tensors(use_stored)
    ctx_e.set_pair_variant(*ctx.pair_variants)
    ctx_e.set_particles(xyz)
    ctx_e.build_cells()
    ctx_e.set_deferred_checks(True)
    e_bounds = state["bounds"]
    RepArr = G.ChebReport * 1
    e_stats = {"lanczos_fallbacks": 0, "terms": []}

    def e2e_step(step_id):
        nonlocal e_bounds
        h_xi = xi_host[step_id % len(xi_host)]
        rc = L_lib.ggem_set_particles(ctx_e.h, N_BEADS, C.c_void_p(h_xyz.data_ptr()))
        rc |= L_lib.ggem_build_cells(ctx_e.h)
        for attempt in range(2):
            rep = RepArr()
            rc2 = L_lib.ggem_brownian_displacement(ctx_e.h, 1, CHEB_MAX, e_bounds[0], e_bounds[1],
                                                   CHEB_TOL, args.check_every,
                                                   C.c_void_p(h_xi.data_ptr()),
                                                   C.c_void_p(h_dw.data_ptr()), rep)
            if rc2 == 0:
                e_stats["terms"].append(rep[0].n_terms)
                break
            e_stats["lanczos_fallbacks"] += 1
            lo, hi = ctx_e.lanczos_bounds(k=24, seed=7)
            e_bounds = (lo / 1.05, hi * 1.05)
        if rc or rc2:
            raise RuntimeError(f"e2e step failed rc={rc} rc2={rc2}")
        _ = float(h_dw.numpy()[0])  # host read of the step's result

    for s in range(args.warmup):
        e2e_step(s)
    e_ts = []
    for s in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step(args.warmup + s)
        t1 = time.perf_counter()
        e_ts.append((t1 - t0) * 1e3)
        clk.mark(t0, t1)
    e2e_ms = float(np.mean(e_ts))
    e_stats["ms_per_step_median"] = float(np.median(e_ts))
    e_stats["ms_per_step_max"] = float(np.max(e_ts))
    ctx_e.close()

    # ---- mobility matvec throughput (FP32, device resident) ------------
    f = torch.randn(3 * N_BEADS, dtype=torch.float64, device="cuda")
    u = torch.empty_like(f)
    for _ in range(5):
        ctx.local_matvec_dev(f.data_ptr(), u.data_ptr(), 1, G.SELF_BEAD)
    mv_ts = []
    for _ in range(max(10, args.steps)):
        flush.zero_()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.local_matvec_dev(f.data_ptr(), u.data_ptr(), 1, G.SELF_BEAD)
        b.record(stream)
        b.synchronize()
        mv_ts.append(a.elapsed_time(b))
    clk.__exit__(None, None, None)
    matvecs_per_s = 1e3 / float(np.mean(mv_ts)) * world

    # ---- accuracy: FP32 vs FP64 velocities at N=200k --------------------
    ctx64 = make_ctx(G.FP64)
    ctx64.set_particles_dev(d_xyz.data_ptr(), N_BEADS)
    ctx64.build_cells()
    fe = torch.from_numpy(G.make_normals(SEED + 5, 3 * N_BEADS)).cuda()
    u32 = torch.empty_like(fe)
    u64 = torch.empty_like(fe)
    ctx.local_matvec_dev(fe.data_ptr(), u32.data_ptr(), 1, G.SELF_BEAD)
    ctx.synchronize()
    ctx64.local_matvec_dev(fe.data_ptr(), u64.data_ptr(), 1, G.SELF_BEAD)
    ctx64.synchronize()
    rel_err = float(torch.linalg.norm(u32 - u64) / torch.linalg.norm(u64))
    comp_err = float((u32 - u64).abs().max() / u64.abs().max())

    # ---- plain FP64 GPU path (the comparison baseline) ------------------
    fp64 = None
    fp64_list = None
    if not args.skip_fp64:
        def fp64_run(c64, path, steps):
            st64 = {"reports": []}

            def fp64_step(step_id):
                c64.set_particles_dev(d_xyz.data_ptr(), N_BEADS)
                c64.build_cells()
                c64.philox_normals_dev(SEED, step_id, 3 * N_BEADS, d_xi.data_ptr())
                lo, hi = c64.lanczos_bounds(k=24, seed=7)  # every step
                rc, rep = c64.brownian_displacement_dev(d_xi.data_ptr(), d_dw.data_ptr(), 1,
                                                        CHEB_MAX, lo / 1.05, hi * 1.05,
                                                        CHEB_TOL, check_every=1)
                st64["reports"].append(rep[0])

            c64.set_stream(stream.cuda_stream)
            c64.set_kernel_timing(True)
            ts64 = timed(fp64_step, steps, 1)
            k_ms, k_n = c64.kernel_timing(G.KERNEL_PAIR_FP64)
            c64.set_kernel_timing(False)
            c64.set_stream(0)
            return {"steps_per_s": 1e3 / float(np.mean(ts64)) * world,
                    "ms_per_step": float(np.mean(ts64)), "steps": steps,
                    "cheb_terms": [r["n_terms"] for r in st64["reports"][-steps:]],
                    "pair_kernel_ms_avg": k_ms / max(k_n, 1), "pair_kernel_launches": k_n,
                    "path": path}

        fp64 = fp64_run(ctx64, "B1: FP64 cell-stencil pair sweep (27 cells per bead), "
                        "Lanczos(24) every step, err1 check every term, one RHS, no graphs",
                        args.fp64_steps)
        ctx64l = make_ctx(G.FP64)
        ctx64l.set_fp64_pair_list(True)
        fp64_list = fp64_run(ctx64l, "B1 with the FP64 pair kernel over the exact pair list "
                             "(in-cutoff pairs only, k_pair_list_f64), Lanczos(24) every step, "
                             "err1 check every term, one RHS, no graphs", max(args.fp64_steps, 3))
        # the FP64 list kernel against the FP64 pipe: flops per pair with the
        # FP64 special functions counted as the survey does (erf, exp = 1)
        fp64_list["pair_kernel_tflops"] = (n_pairs * 47 / (fp64_list["pair_kernel_ms_avg"] * 1e-3)
                                           / 1e12)
        ctx64l.close()
    ctx64.close()

    # ---- eigen bounds refreshed every step: network vs Lanczos ----------
    per_step = None
    if sur is not None:
        def refresh_step(step_id, use_sur):
            ctx.set_particles_dev(d_xyz.data_ptr(), N_BEADS)
            ctx.build_cells()
            ctx.philox_normals_dev(SEED, step_id, 3 * N_BEADS, d_xi.data_ptr())
            if use_sur:
                lo, hi = ctx.surrogate_interval(sur, 0.0, sur_margins[0], sur_margins[1])
            else:
                lo, hi = lanczos(ctx)
            rc, rep = ctx.brownian_displacement_dev(d_xi.data_ptr(), d_dw.data_ptr(), 1,
                                                    CHEB_MAX, lo, hi, CHEB_TOL,
                                                    check_every=args.check_every)
            if rc != 0:  # rejected interval: Lanczos fallback
                lo, hi = lanczos(ctx)
                rc, rep = ctx.brownian_displacement_dev(d_xi.data_ptr(), d_dw.data_ptr(), 1,
                                                        CHEB_MAX, lo, hi, CHEB_TOL,
                                                        check_every=args.check_every)
            return rc == 0, rep[0]["n_terms"]

        per_step = {}
        for name, use_sur in (("surrogate", True), ("lanczos24", False)):
            for s_ in range(2):
                refresh_step(s_, use_sur)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            oks = [refresh_step(100 + s_, use_sur) for s_ in range(max(5, args.steps))]
            ctx.synchronize()
            dt = (time.perf_counter() - t0) / len(oks)
            per_step[name] = {"steps_per_s": 1.0 / dt, "ms_per_step": dt * 1e3,
                              "converged": all(o for o, _ in oks),
                              "cheb_terms": sorted({t for _, t in oks})}
        per_step["surrogate_margins_log"] = [float(x) for x in sur_margins]

    # ---- polymer suspension, 64 batched noise right-hand sides ----------
    poly = None if args.skip_polymer else polymer_leg(G, torch, dev, flush, peak_fn=None)
    ens_res = None if args.skip_ensemble else ensemble_leg(G, torch, dev, flush, sur, sur_margins)
    spread = None if args.skip_spread else spread_leg(G, torch, dev, flush, xyz, L,
                                                     ctx.probe_fp32_peak())

    # ---- roofline of the dominant kernel --------------------------------
    # the dominant kernel of the timed steps: the fused pair-sum + Chebyshev
    # term (k_pair_cheb) or the plain pair sum (k_pair_r1), whichever took
    # more time; both do the same pair work per launch
    peak = ctx.probe_fp32_peak()
    row_width, stored = ctx.pair_storage()
    if stored:
        names = {"pair_cheb": "k_pair_cheb_tv (stored pair tensors + fused FP64 Chebyshev term)",
                 "pair_fp32": "k_pair_r1tv (stored pair tensors, one RHS)"}
    else:
        names = {"pair_cheb": "k_pair_cheb (pair list, tensors per pair + fused Chebyshev term)",
                 "pair_fp32": "k_pair_r1 (pair list, tensors per pair, one RHS)"}
    dom = "pair_cheb"  # the fused terms: 9 of the 11 pair launches of a step
    pair_ms, pair_n = kt[dom]
    avg_pair_ms = pair_ms / max(pair_n, 1)
    flops_per_launch = n_pairs * (28 + 19 * 1)
    # algorithmic bytes with stored tensors: 4 B entry + 16 B tensor per pair,
    # and per bead 16 B force + 4 B row count + the FP64 vectors the kernel
    # reads and writes (plain: f 24 + u 24; fused term: x0, x1, dw in, dw,
    # x_{k+1} out 5 x 24, next forces 16)
    per_bead = {"pair_fp32": 16 + 4 + 48, "pair_cheb": 16 + 4 + 120 + 16}
    bytes_per_launch = n_pairs * 20 + N_BEADS * per_bead[dom]
    if not stored:
        # tensors evaluated per pair: 4 B entry per pair; per bead the 32-byte
        # source record, the row count and the FP64 vectors (plain: f, u; fused
        # term: x0, x1, dw in, dw, x_{k+1} out) and the next 32-byte record
        per_bead = {"pair_fp32": 32 + 4 + 48, "pair_cheb": 32 + 4 + 120 + 32}
        bytes_per_launch = n_pairs * 4 + N_BEADS * per_bead[dom]
    achieved = flops_per_launch / (avg_pair_ms * 1e-3) / 1e12
    others = {k: {"avg_launch_ms": kt_all[k][0] / max(kt_all[k][1], 1),
                  "launches": kt_all[k][1],
                  "tflops": (flops_per_launch / (kt_all[k][0] / kt_all[k][1] * 1e-3) / 1e12)
                  if kt_all[k][1] else None} for k in names}
    ctx.close()
    if stored:
        gbs = bytes_per_launch / (avg_pair_ms * 1e-3) / 1e9
        hbm_peak = measured_peaks().get("hbm_gbs")
        roof = {"bound": "hbm", "kernel": names[dom], "achieved": gbs, "peak": hbm_peak,
                "unit": "GB/s", "frac": gbs / hbm_peak if hbm_peak else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy), of measured",
                "bytes_per_launch": bytes_per_launch, "fp32_tflops": achieved,
                "fp32_frac_of_live_peak": achieved / peak if peak else None}
    else:
        gbs = bytes_per_launch / (avg_pair_ms * 1e-3) / 1e9
        hbm_peak = measured_peaks().get("hbm_gbs")
        roof = {"bound": "fp32", "kernel": names[dom], "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                "peak_source": "measured live: FP32 FMA-chain probe on this GPU "
                               "(MEASURED_PEAKS.json has no FP32 figure)",
                "bytes_per_launch": bytes_per_launch, "hbm_gbs": gbs,
                "hbm_frac_of_measured": gbs / hbm_peak if hbm_peak else None}
    roof.update({"flops_per_launch": flops_per_launch, "pairs": n_pairs, "row_width": row_width,
                 "avg_launch_ms": avg_pair_ms, "launches_timed": pair_n,
                 "pair_kernels": others, "traffic": PAIR_TRAFFIC.get(names[dom].split()[0])})

    result = {
        "metric": METRIC, "value": steps_per_s, "unit": "Brownian steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 pair sums, f64 Chebyshev recurrence", "data": "synthetic (seeded)",
        "config": workload_config({"parallelism": f"replicas x{world}", "cell_div": cell_div,
                                   "check_every": args.check_every, "autotune": tuning}),
        "e2e": {"value": 1e3 / e2e_ms * world, "unit": "Brownian steps/s",
                "ms_per_step": e2e_ms, "detail": e_stats, "h2d_bytes_per_step": 2 * 24 * N_BEADS,
                "d2h_bytes_per_step": 24 * N_BEADS},
        "matvecs_per_s": matvecs_per_s, "matvec_ms": float(np.mean(mv_ts)),
        "plain_fp64_gpu": fp64,
        "speedup_vs_plain_fp64": (steps_per_s / fp64["steps_per_s"]) if fp64 else None,
        "plain_fp64_gpu_pair_list": fp64_list,
        "speedup_vs_plain_fp64_pair_list": (steps_per_s / fp64_list["steps_per_s"])
        if fp64_list else None,
        "velocity_rel_err_fp32_vs_fp64": rel_err, "velocity_max_component_err": comp_err,
        "cheb": {"terms": [r["n_terms"] for r in reps], "err1_max": max(r["err1"] for r in reps),
                 "converged": all(r["converged"] for r in reps),
                 "bounds_source": state["source"],
                 "surrogate_calls": calls["surrogate_calls"],
                 "lanczos_calls": calls["lanczos_calls"]},
        "bounds_every_step": per_step,
        "check_every_term": faithful,
        "roofline": roof,
        "kernel_ms_in_timed_region": {k: v[0] for k, v in kt.items()},
        "kernel_ms_per_step_separate_run": kt_per_step,
        "gpu_launches": int(lc1 - lc0),
        "clocks": clk.summary(), "wall_s_timed": t_wall,
        "polymer_64rhs": poly,
        "ensemble_512x8": ens_res,
        "spread": spread,
    }
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        result["cpu_baseline"] = cpu_baseline(xyz, L, state["bounds"], args)
    return result


# --------------------------------------------------------------------------
# polymer suspension with 64 batched right-hand sides
# --------------------------------------------------------------------------
POLY_CHAINS, POLY_BEADS, POLY_PHI, POLY_NRHS = 5000, 20, 0.05, 64


def polymer_leg(G, torch, dev, flush, peak_fn=None, reps=5):
    """5000 chains x 20 beads (N = 100k, bond 2a, self-avoiding growth) at
    phi = 0.05: the batched 64-RHS mobility matvec and one Brownian step of
    64 noise vectors (adaptive Chebyshev, tol 1e-3, <= 50 terms), device
    resident, L2 flushed before each timed call."""
    xyz, L = G.make_chains(SEED + 7, POLY_CHAINS, POLY_BEADS, 2.0, POLY_PHI)
    n = len(xyz)
    ctx = G.Context(alpha=ALPHA, box_hi=(L,) * 3, rc=RC, precision=G.FP32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    d_xyz = torch.from_numpy(xyz.reshape(-1)).cuda()
    torch.cuda.synchronize()
    ctx.set_stream(stream.cuda_stream)
    ctx.set_particles_dev(d_xyz.data_ptr(), n)
    ctx.build_cells()
    pairs = ctx.pair_count()
    R = POLY_NRHS
    f = torch.randn(R * 3 * n, dtype=torch.float64, device="cuda")
    u = torch.empty_like(f)
    torch.cuda.synchronize()
    for _ in range(3):
        ctx.local_matvec_dev(f.data_ptr(), u.data_ptr(), R, G.SELF_BEAD)
    ctx.synchronize()
    ctx.set_kernel_timing(True)
    mv = []
    for _ in range(reps):
        flush.zero_()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.local_matvec_dev(f.data_ptr(), u.data_ptr(), R, G.SELF_BEAD)
        b.record(stream)
        b.synchronize()
        mv.append(a.elapsed_time(b))
    k_ms, k_n = ctx.kernel_timing(G.KERNEL_PAIR_FP32)
    ctx.set_kernel_timing(False)
    lo, hi = ctx.lanczos_bounds(k=24, seed=7)
    lo, hi = lo / 1.05, hi * 1.05
    xi = torch.randn(R * 3 * n, dtype=torch.float64, device="cuda")
    dw = torch.empty_like(xi)
    torch.cuda.synchronize()
    terms = []
    for _ in range(2):  # the adaptive schedule learns the degree
        rc, rp = ctx.brownian_displacement_dev(xi.data_ptr(), dw.data_ptr(), R, CHEB_MAX, lo, hi,
                                               CHEB_TOL, check_every=0)
    st = []
    for _ in range(reps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc, rp = ctx.brownian_displacement_dev(xi.data_ptr(), dw.data_ptr(), R, CHEB_MAX, lo, hi,
                                               CHEB_TOL, check_every=0)
        ctx.synchronize()
        st.append((time.perf_counter() - t0) * 1e3)
        terms.append(max(r["n_terms"] for r in rp))
    ok = rc == 0 and all(r["converged"] for r in rp)
    peak = ctx.probe_fp32_peak()
    ctx.close()
    avg = k_ms / max(k_n, 1)
    flops = pairs * (28 + 19 * R)
    tf = flops / (avg * 1e-3) / 1e12
    return {"workload": f"{POLY_CHAINS} chains x {POLY_BEADS} beads (N={n}), bond 2a, "
                        f"phi={POLY_PHI}, L={L:.1f}, {R} noise right-hand sides",
            "pairs": pairs, "matvec_ms": float(np.mean(mv)),
            "matvecs_per_s": R * 1e3 / float(np.mean(mv)),
            "brownian_step_ms_64rhs": float(np.mean(st)),
            "brownian_steps_per_s_x_rhs": R * 1e3 / float(np.mean(st)),
            "cheb_terms": terms, "converged": ok,
            "kernel": "k_pair_b64 (lanes over 64 right-hand sides)",
            "kernel_avg_launch_ms": avg, "kernel_tflops": tf, "fp32_peak_tflops": peak,
            "kernel_frac_of_fp32_peak": tf / peak if peak else None,
            "flops_per_launch": flops}


# --------------------------------------------------------------------------
# Gaussian spread onto the quadrature points of the HEX20 mesh
# --------------------------------------------------------------------------
SPREAD_H_MAX = 1.414  # h <= 1/(sqrt(2) alpha), the reference tutorial's mesh rule
SPREAD_NQ = 8         # QGauss SECOND on the HEX20 velocity element (assemble_stokes.C:397)


def spread_leg(G, torch, dev, flush, xyz, L, peak, reps=5, old_fraction=16):
    """rho at the 8 Gauss points of every element of the box's HEX20 mesh
    (h = L / ceil(L / 1.414), 144^3 elements at L = 203.1), element
    neighbour lists of search_radius_e = 0.5 h + 4/alpha, for the N = 200k
    suspension: the brick kernel in FP32 and FP64, and the per-point FP64
    kernel on a 1/old_fraction slab of the elements (its per-point work is
    the same everywhere in a periodic box).  Device resident, L2 flushed
    before each timed call, CUDA events on the context's stream."""
    n = len(xyz)
    nm = int(np.ceil(L / SPREAD_H_MAX))
    h = L / nm
    sre = 0.5 * h + 4.0 / ALPHA
    ctx = G.Context(alpha=ALPHA, box_hi=(L,) * 3, nb_mode=G.NB_REFERENCE, n_mesh=(nm,) * 3,
                    search_radius_e=sre, precision=G.FP64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    d_xyz = torch.from_numpy(xyz.reshape(-1)).cuda()
    torch.cuda.synchronize()
    ctx.set_particles_dev(d_xyz.data_ptr(), n)
    ctx.build_cells()
    ne = nm ** 3
    g = [0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0)]
    loc = torch.tensor([[g[a], g[b], g[c]] for c in range(2) for b in range(2) for a in range(2)],
                       dtype=torch.float64, device="cuda")
    ar = torch.arange(nm, dtype=torch.float64, device="cuda")
    ez, ey, ex = torch.meshgrid(ar, ar, ar, indexing="ij")
    base = torch.stack([ex.reshape(-1), ey.reshape(-1), ez.reshape(-1)], dim=1)
    q = ((base[:, None, :] + loc[None, :, :]) * h).reshape(-1).contiguous()
    del base, ex, ey, ez
    nqt = ne * SPREAD_NQ
    torch.cuda.synchronize()
    ctx.set_quadrature_dev(q.data_ptr(), SPREAD_NQ, nqt)
    f = torch.from_numpy(G.make_normals(SEED + 21, 3 * n)).cuda()
    rho32 = torch.empty(3 * nqt, dtype=torch.float64, device="cuda")
    rho64 = torch.empty_like(rho32)
    torch.cuda.synchronize()
    pairs = ctx.spread_elements_dev(f.data_ptr(), rho64.data_ptr(), G.FP64, count_pairs=True)

    def time_call(fn, k):
        ts = []
        for _ in range(k):
            flush.zero_()
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.mean(ts)), ts

    for _ in range(2):
        ctx.spread_elements_dev(f.data_ptr(), rho32.data_ptr(), G.FP32)
    t32, ts32 = time_call(lambda: ctx.spread_elements_dev(f.data_ptr(), rho32.data_ptr(), G.FP32),
                          reps)
    t64, _ = time_call(lambda: ctx.spread_elements_dev(f.data_ptr(), rho64.data_ptr(), G.FP64), 2)
    # the per-point FP64 kernel (one thread per point, every stencil element
    # visited) on the first 1/old_fraction of the elements
    ne_old = ne // old_fraction
    nq_old = ne_old * SPREAD_NQ
    qe = torch.arange(ne_old, dtype=torch.int32, device="cuda").repeat_interleave(SPREAD_NQ)
    rho_old = torch.empty(3 * nq_old, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.spread_qp_dev(nq_old, q.data_ptr(), qe.data_ptr(), f.data_ptr(), rho_old.data_ptr())
    t_old, _ = time_call(lambda: ctx.spread_qp_dev(nq_old, q.data_ptr(), qe.data_ptr(),
                                                   f.data_ptr(), rho_old.data_ptr()), 1)
    same_old = float(torch.linalg.norm(rho_old - rho64[:3 * nq_old]) /
                     torch.linalg.norm(rho64[:3 * nq_old]))
    d = (rho32 - rho64).abs()
    err = float(torch.linalg.norm(rho32 - rho64) / torch.linalg.norm(rho64))
    comp = float(d.max() / rho64.abs().max())
    per = (d / rho64.abs().clamp_min(1e-300))[::7].cpu().numpy()  # a 1/7 sample
    ctx.close()
    flops = pairs * 21
    tf32 = flops / (t32 * 1e-3) / 1e12
    t_old_full = t_old * old_fraction
    # algorithmic bytes: per point its FP32 element-relative position (16 B)
    # and its FP64 rho (24 B); per particle its record (32 B) and force (24 B)
    byts = nqt * 40 + n * 56
    return {"workload": f"HEX20 mesh {nm}^3 = {ne} elements (h = {h:.4f}) x {SPREAD_NQ} Gauss "
                        f"points = {nqt} points, element lists of search_radius_e = "
                        f"{sre:.4f}, N = {n} beads (phi = {PHI})",
            "pairs": pairs, "pairs_per_point": pairs / nqt,
            "fp32_ms": t32, "fp32_ms_all": ts32, "fp64_ms": t64,
            "pairs_per_s_fp32": pairs / (t32 * 1e-3), "pairs_per_s_fp64": pairs / (t64 * 1e-3),
            "per_point_fp64_ms_scaled": t_old_full,
            "per_point_fp64_sample": f"first {ne_old} elements ({nq_old} points), "
                                    f"{t_old:.2f} ms x {old_fraction}",
            "per_point_vs_brick_fp64_rel_diff": same_old,
            "speedup_fp32_vs_per_point_fp64": t_old_full / t32,
            "speedup_fp32_vs_brick_fp64": t64 / t32,
            "fp32_vs_fp64_rel_err": err, "fp32_max_component_err": comp,
            "fp32_per_component_rel_median": float(np.median(per)),
            "fp32_per_component_rel_p99": float(np.percentile(per, 99)),
            "roofline": {"bound": "fp32", "kernel": "k_spread_brick<FP32>", "achieved": tf32,
                         "peak": peak, "unit": "TFLOP/s", "frac": tf32 / peak if peak else None,
                         "flops_per_launch": flops, "work": "20 flops + 1 exp per (point, "
                         "listed particle)", "bytes_per_launch": byts,
                         "hbm_gbs": byts / (t32 * 1e-3) / 1e9}}


# --------------------------------------------------------------------------
# uneven ensemble: 512 suspensions, 8 noise right-hand sides each
# --------------------------------------------------------------------------
ENS_K, ENS_NRHS = 512, 8


def ensemble_leg(G, torch, dev, flush, sur, margins, reps=3):
    """512 periodic suspensions, N log-uniform in [500, 20000], phi uniform
    in [0.02, 0.2], 8 noise vectors each, through one block-diagonal
    operator: build, autotune, eigen intervals (one batched forward pass of
    the network vs Lanczos(24) per suspension), and the Brownian step of
    all 4096 series (device resident, L2 flushed before each timed step)."""
    from concurrent.futures import ThreadPoolExecutor
    rng = np.random.default_rng(SEED + 11)
    ns = np.exp(rng.uniform(np.log(500), np.log(20000), ENS_K)).astype(np.int64)
    phis = rng.uniform(0.02, 0.2, ENS_K)
    with ThreadPoolExecutor(16) as ex:
        sus = list(ex.map(lambda b: G.make_suspension(SEED * 7 + b, int(ns[b]), float(phis[b])),
                          range(ENS_K)))
    t0 = time.perf_counter()
    ens = G.Ensemble([L for _, L in sus], device=dev)
    d_xyz = torch.from_numpy(np.concatenate([x for x, _ in sus]).reshape(-1)).cuda()
    torch.cuda.synchronize()
    ens.set_particles_dev(ns, d_xyz.data_ptr())
    t_build = time.perf_counter() - t0
    beads, pairs = ens.sizes()
    block, ms_term = ens.autotune(ENS_NRHS)
    t0 = time.perf_counter()
    lz = [ens.lanczos(b, 24, 7) for b in range(ENS_K)]
    t_lz = time.perf_counter() - t0
    lo = np.array([x[0] for x in lz]) / 1.05
    hi = np.array([x[1] for x in lz]) * 1.05
    t_sur = None
    if sur is not None:
        t0 = time.perf_counter()
        lo, hi = ens.intervals(sur, None, margins[0], margins[1])
        t_sur = time.perf_counter() - t0
    xi = torch.randn(beads * ENS_NRHS * 3, dtype=torch.float64, device="cuda")
    dw = torch.empty_like(xi)
    # the step's form (a persistent launch of some shape and tile size, or one
    # launch per term: shape 3), tuned on a 14-term series (about the degree
    # these intervals need); the timed steps below run the chosen form
    t0 = time.perf_counter()
    s_shape, s_slots, s_ms = ens.autotune_series(ENS_NRHS, 14, lo, hi, xi.data_ptr(),
                                                 dw.data_ptr())
    t_tune = time.perf_counter() - t0
    torch.cuda.synchronize()
    fallbacks = 0

    def step():
        nonlocal fallbacks
        rc, rp = ens.brownian_dev(ENS_NRHS, CHEB_MAX, lo, hi, CHEB_TOL, xi.data_ptr(),
                                  dw.data_ptr())
        if rc:
            for b in range(ENS_K):  # rejected intervals: Lanczos, then again
                if not all(r["converged"] for r in rp[b]):
                    fallbacks += 1
                    l_, h_ = ens.lanczos(b, 24, 7)
                    lo[b], hi[b] = l_ / 1.05, h_ * 1.05
            rc, rp = ens.brownian_dev(ENS_NRHS, CHEB_MAX, lo, hi, CHEB_TOL, xi.data_ptr(),
                                      dw.data_ptr())
        return rc, rp

    for _ in range(2):
        step()
    ts, terms, ok = [], [], True
    torch.cuda.nvtx.range_push("ensemble_steps")  # selects these launches for a profiler
    for _ in range(reps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc, rp = step()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
        ok = ok and rc == 0
        terms.append(max(r["n_terms"] for rb in rp for r in rb))
    torch.cuda.nvtx.range_pop()
    # both forms of the step: one persistent launch (device-side checks and
    # stopping decisions) and one launch per term (host-side checks)
    modes = {}
    for name, pers in (("persistent_launch", True), ("launch_per_term", False)):
        ens.set_series_mode(persistent=pers)
        for _ in range(2):
            step()
        mts = []
        for _ in range(reps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc_m, _ = step()
            torch.cuda.synchronize()
            mts.append((time.perf_counter() - t0) * 1e3)
        modes[name] = {"brownian_step_ms": float(np.mean(mts)), "converged": rc_m == 0}
    f = torch.randn(beads * ENS_NRHS * 3, dtype=torch.float64, device="cuda")
    u = torch.empty_like(f)
    ens.matvec_dev(ENS_NRHS, f.data_ptr(), u.data_ptr())
    mv = []
    for _ in range(5):
        flush.zero_()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b_ = torch.cuda.Event(enable_timing=True)
        a.record()
        ens.matvec_dev(ENS_NRHS, f.data_ptr(), u.data_ptr())
        b_.record()
        b_.synchronize()
        mv.append(a.elapsed_time(b_))
    ens.close()
    step_s = float(np.mean(ts))
    # algorithmic bytes of one fused term: 20 B per pair (entry + tensor) and
    # per bead 8 x (16 B force + 3 x 8 B x0, x1, dw in, dw, x_{k+1} out, 16 B
    # next force) + 4 B row count
    term_bytes = pairs * 20 + beads * (ENS_NRHS * (16 + 5 * 24 + 16) + 4)
    peak = measured_peaks().get("hbm_gbs")
    return {"workload": f"{ENS_K} periodic suspensions, N log-uniform in [500, 20000] "
                        f"(sum {beads}), phi uniform in [0.02, 0.2], {ENS_NRHS} noise vectors each",
            "beads": beads, "pairs": pairs, "build_s": t_build,
            "autotune": {"block_threads": block, "ms_per_term": ms_term,
                         "series_form": "persistent launch" if s_shape < 3 else "launch per term",
                         "series_shape": s_shape, "series_slots_per_tile": s_slots,
                         "series_ms_14_terms": s_ms, "series_tune_s": t_tune},
            "intervals_s": {"network_one_batch": t_sur, "lanczos24_per_suspension": t_lz},
            "lanczos_fallbacks": fallbacks,
            "brownian_step_ms": step_s * 1e3,
            "series_steps_per_s": ENS_K * ENS_NRHS / step_s,
            "cheb_terms_max": terms, "converged": ok,
            "step_forms": modes,
            "matvec_8rhs_ms": float(np.mean(mv)),
            "term_kernel": {"kernel": "k_ens_pair<true> (stored tensors, 8 lanes per slot)",
                            "bytes": term_bytes, "ms": ms_term,
                            "gbs": term_bytes / (ms_term * 1e-3) / 1e9,
                            "frac_of_hbm": (term_bytes / (ms_term * 1e-3) / 1e9 / peak)
                            if peak else None}}


# --------------------------------------------------------------------------
# CPU baseline / reference arm: the FP64 oracle on the host cores
# --------------------------------------------------------------------------
def _oracle_step(O, c, box, xyz, xi, lo, hi, nthreads):
    nb = O.neighbors_cutoff(box, xyz, RC)
    op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, nthreads))
    y, rep = O.cheb_inv_sqrt(op, xi, CHEB_MAX, lo, hi, CHEB_TOL)
    dw = O.local_matvec(c, box, xyz, nb, y, O.SELF_BEAD, nthreads)
    return rep, dw


def cpu_baseline(xyz, L, bounds, args, steps=None):
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O  # the checker, timed as the CPU baseline

    O.build_oracle(with_ref=False)
    nthreads = os.cpu_count() or 1
    c = O.constants(alpha=ALPHA)
    box = O.make_box([0] * 3, [L] * 3, [1, 1, 1])
    if bounds is None:
        nb = O.neighbors_cutoff(box, xyz, RC)
        op = O.Operator(matvec=(c, box, xyz, nb, O.SELF_BEAD, nthreads))
        lo, hi, _, _ = O.lanczos(op, np.random.default_rng(7).standard_normal(3 * len(xyz)), 24)
        bounds = (lo / 1.05, hi * 1.05)
    steps = steps or args.cpu_steps
    rng = np.random.default_rng(11)
    ts, terms = [], []
    for s in range(steps):
        xi = rng.standard_normal(3 * len(xyz))
        t0 = time.perf_counter()
        rep, _ = _oracle_step(O, c, box, xyz, xi, bounds[0], bounds[1], nthreads)
        ts.append(time.perf_counter() - t0)
        terms.append(rep.n_terms)
    v = 1.0 / float(np.mean(ts))
    return {"value": v, "unit": "Brownian steps/s", "cores": nthreads, "kind": "port",
            "sample": f"{steps} full Brownian steps at N={len(xyz)} (cut-off list build + "
                      f"reference-faithful Chebyshev, error check every term, + M y), FP64 "
                      f"oracle with {nthreads} threads; terms {terms}",
            "seconds": float(np.sum(ts))}


def run_reference(args, rank, world):
    import ggem_gb300 as G  # workload generator only (host code)
    from ggem_gb300 import build as B

    B.build()
    xyz, L = G.make_suspension(SEED, N_BEADS, PHI)
    budget_steps = max(1, min(args.steps, args.reference_max_steps))
    cb = cpu_baseline(xyz, L, None, args, steps=budget_steps)
    return {"metric": METRIC, "value": cb["value"], "unit": "Brownian steps/s", "n_gpus": world,
            "steps": budget_steps, "warmup": 0, "ms_per_step": 1e3 / cb["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference",
            "config": workload_config({"parallelism": "host threads"}),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "Brownian steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--check-every", type=int, default=0)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--reference-max-steps", type=int, default=30)
    ap.add_argument("--skip-polymer", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--skip-ensemble", action="store_true")
    ap.add_argument("--skip-spread", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args, rank, world)))
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    res = run_gb300(args, rank, world)
    if rank == 0:
        print(json.dumps(res))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
