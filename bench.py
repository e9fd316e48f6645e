#!/usr/bin/env python3
"""bench.py — throughput of the range-limited force path (pair-evals/s and ns/day).

A step is one velocity-Verlet MD step of the whole system on the GPU: kick + drift + rebin
(count, scan, scatter, in-cell sort, gather), the half-shell force kernel, kick.  Default
workload: the 92,224-atom LJ+Coulomb system (108.86 x 108.86 x 77.76 A, rc 12 A, 9x9x6 cells,
4 types, +-0.42 e) with first-order 512-bin tables and int64 fixed-point accumulation ("tuned"),
next to the FP32-atomic accumulation ("plain") at the same tables.

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference] [--workload ...]

N > 1 (one process per GPU under torch.distributed.run) runs N independent replicas (seed offset
= rank): the path has no exchange step on one node, so value = pairs of all ranks / max time.
--impl reference times the CPU implementation of the same path (the oracle's multi-threaded
cell-list port) on rank 0 with every host thread.
"""
from __future__ import annotations

import argparse
import dataclasses
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

FLOPS_PER_PAIR = 28            # algorithmic flops per in-cutoff pair, force only
L2_FLUSH_BYTES = 256 << 20     # > 129 MB L2
METRIC = "pair-evals/s & ns/day, 92k-atom RL LJ+Coulomb, tuned vs plain @1e-5 force err"


def make_system(name: str, seed_offset: int):
    from sc2019_md_gb300 import systems
    if name == "ljc92k":
        return systems.ljc92k(seed_offset=seed_offset)
    if name == "lj1728":
        return systems.lj1728(seed_offset=seed_offset)
    if name == "ljc1m":
        return systems.ljc1m(seed_offset=seed_offset)
    raise SystemExit(f"unknown workload {name}")


def workload_desc(sysm, order, bins) -> str:
    nc = "x".join(str(c) for c in sysm.ncell)
    box = "x".join(f"{b:g}" for b in sysm.box)
    kind = "LJ+Coulomb" if sysm.coulomb_k else "LJ"
    return (f"{sysm.name}: {sysm.n} atoms, {box} A periodic, rc {sysm.cutoff:g} A, {nc} cells, "
            f"{len(sysm.sigma)} types, {kind}, order-{order} {bins}-bin tables, velocity Verlet 2 fs")


class Clocks:
    """nvidia-smi samples every 200 ms while running (SM clock, max clock, throttle reasons)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.reader.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [v.strip() for v in l.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[3 + k].lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return rank, world, local, dist


def combine_ranks(dist, device, maxes, sums):
    """Max over ranks of `maxes` and sum over ranks of `sums` (each rank runs one replica)."""
    import torch
    a = torch.tensor([float(v) for v in maxes], dtype=torch.float64, device=device)
    b = torch.tensor([float(v) for v in sums], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(a, op=dist.ReduceOp.MAX)
        dist.all_reduce(b, op=dist.ReduceOp.SUM)
    return [float(v) for v in a.tolist()], [float(v) for v in b.tolist()]


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except json.JSONDecodeError:
            pass
    return {}


def committed_metric(workload: str, key: str):
    """A figure of the committed ncu summary profiles/k_force_<workload>.md ("<key>: <value> ...")."""
    f = ROOT / "profiles" / f"k_force_{workload}.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def committed_traffic(workload: str):
    """Per-launch DRAM bytes of the force kernel from the committed ncu summary, or None."""
    f = ROOT / "profiles" / f"k_force_{workload}.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def force_eval_pinned(m, ctx, bufs, n):
    """mdrl_force_eval on pinned host buffers (the C-ABI call a user makes)."""
    st = m.Stats()
    F = C.POINTER(C.c_float)
    I = C.POINTER(C.c_int)
    s = m.lib().mdrl_force_eval(ctx._h, n, bufs["x"].ctypes.data_as(F), bufs["y"].ctypes.data_as(F),
                                bufs["z"].ctypes.data_as(F), bufs["q"].ctypes.data_as(F),
                                bufs["t"].ctypes.data_as(I), bufs["fx"].ctypes.data_as(F),
                                bufs["fy"].ctypes.data_as(F), bufs["fz"].ctypes.data_as(F), None, C.byref(st))
    if s != 0:
        raise m.MdrlError(s, m.lib().mdrl_last_error().decode())
    return st


def run_ours(args, rank, world, local, dist):
    import torch

    import sc2019_md_gb300 as m
    from sc2019_md_gb300 import systems

    torch.cuda.set_device(local)
    sysm = make_system(args.workload, rank)
    params = sysm.params(table_bins=args.bins, table_order=args.order, device=local)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")

    def timed_steps(ctx, k):
        dev_ms, pairs, fms, pstep = 0.0, 0, [], []
        for _ in range(k):
            flush.zero_()
            torch.cuda.synchronize()
            st = ctx.step(1)
            dev_ms += st["device_ms"]
            pairs += st["pairs_total"]
            fms.append(st["force_ms"])
            pstep.append(st["pairs"])
        return dev_ms, pairs, fms, pstep

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # ---- tuned: int64 fixed point, autotuned tile -------------------------------------------
    ctx = m.Context(params)
    ctx.set_state(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
    if args.tile:
        ctx.set_tile(*args.tile)
        tune = {"tile": ctx.tile(), "ms": None, "default_ms": None}
    else:
        tune = ctx.autotune(retime=True) if not args.no_tune else {"tile": ctx.tile(), "ms": None, "default_ms": None}
    timed_steps(ctx, args.warmup)
    barrier()
    clocks = Clocks(local)
    clocks.start()
    t0 = time.perf_counter()
    dev_ms, pairs, fms, pstep = timed_steps(ctx, args.steps)
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    fms = []
    for _ in range(max(3, min(args.steps, 20))):      # the force kernel alone, L2 flushed
        flush.zero_()
        torch.cuda.synchronize()
        fms.append(ctx.time_force())
    ctx.close()

    # ---- the same step with smooth-PME long-range electrostatics (charged systems) -----------
    pme_out = None
    if not args.no_pme and sysm.q is not None:
        ctxl = m.Context(params)
        pme_p = ctxl.set_pme(order=args.pme_order)
        ctxl.set_state(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
        if not args.no_tune:
            ctxl.autotune(retime=True)
        timed_steps(ctxl, args.warmup)
        kl = max(3, min(args.steps, 50))
        ldev_ms, lpairs, _, _ = timed_steps(ctxl, kl)
        ctxl.close()
        pme_out = {"value": lpairs / (ldev_ms * 1e-3), "unit": "pair-evals/s", "ms_per_step": ldev_ms / kl,
                   "ns_per_day": (1000.0 / (ldev_ms / kl)) * params.dt_fs * 0.0864, "steps": kl,
                   "beta": pme_p["beta"], "grid": list(pme_p["grid"]), "order": pme_p["order"],
                   "note": "same step + PME reciprocal part (spread, 2 FFTs, gather); real space in the pair tables"}

    # ---- bonded terms: their kernels alone, on a chain topology of the same size ------------
    bonded_out = None
    if not args.no_bonded:
        nch = sysm.n // 30
        Lc = float((nch * 30 / 0.1) ** (1.0 / 3.0))
        csys, T = systems.chains(nch, 30, Lc, seed=20191117 + 6, cutoff=12.0, dmin=0.0)
        ctxb = m.Context(csys.params(table_bins=args.bins, table_order=args.order, device=local))
        ctxb.set_bonded(**T)
        ctxb.set_state(csys.pos[:, 0], csys.pos[:, 1], csys.pos[:, 2], csys.vel, None, csys.type)
        bms = []
        for _ in range(max(3, min(args.steps, 20))):
            flush.zero_()
            torch.cuda.synchronize()
            bms.append(ctxb.time_bonded())
        ctxb.close()
        nterms = sum(len(v[0]) for v in T.values())
        bmed = float(np.median(bms))
        bonded_out = {"terms": nterms, "bonds": len(T["bonds"][0]), "angles": len(T["angles"][0]),
                      "dihedrals": len(T["dihedrals"][0]), "ms": bmed, "terms_per_s": nterms / (bmed * 1e-3),
                      "workload": f"{csys.n} atoms as {nch} chains of 30 in a {Lc:.1f} A cube (density 0.1), "
                                  f"FP32 terms into the int64 accumulators; kernels alone (inverse map + terms), "
                                  f"L2 flushed"}

    # ---- plain: FP32 atomics, same tables --------------------------------------------------
    kp = max(3, min(args.steps, 50))
    pp = sysm.params(table_bins=args.bins, table_order=args.order, device=local, accum=m.ACC_FP32_ATOMIC)
    ctxp = m.Context(pp)
    ctxp.set_state(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
    timed_steps(ctxp, args.warmup)
    barrier()
    pdev_ms, ppairs, pfms, _ = timed_steps(ctxp, kp)
    barrier()
    pfms = []
    for _ in range(5):
        flush.zero_()
        torch.cuda.synchronize()
        pfms.append(ctxp.time_force())
    ctxp.close()

    # ---- e2e: mdrl_force_eval on pinned host buffers ---------------------------------------
    n = sysm.n
    pin = lambda dt: torch.empty(n, dtype=dt, pin_memory=True).numpy()
    bufs = {k: pin(torch.float32) for k in ("x", "y", "z", "q", "fx", "fy", "fz")}
    bufs["t"] = pin(torch.int32)
    for k, v in (("x", sysm.pos[:, 0]), ("y", sysm.pos[:, 1]), ("z", sysm.pos[:, 2]), ("q", sysm.q), ("t", sysm.type)):
        bufs[k][:] = v
    ctxe = m.Context(params)
    ctxe.set_tile(*tune["tile"])                       # the tile the tuned arm runs
    for _ in range(args.warmup):
        force_eval_pinned(m, ctxe, bufs, n)
    ke = max(3, min(args.steps, 30))
    e2e_s, e2e_pairs, e2e_dev = 0.0, 0, 0.0
    for _ in range(ke):
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        st = force_eval_pinned(m, ctxe, bufs, n)
        e2e_s += time.perf_counter() - t1
        e2e_pairs += st.pairs
        e2e_dev += st.device_ms
    ctxe.close()

    # ---- reduce over ranks -----------------------------------------------------------------
    mx, sm = combine_ranks(dist, f"cuda:{local}", maxes=[dev_ms, e2e_s, pdev_ms],
                           sums=[pairs, e2e_pairs, ppairs])
    if rank != 0:
        return None
    dev_ms_max = mx[0]
    tot, psum, emax = [mx[0]], sm, [mx[1], mx[2]]
    value = float(psum[0]) / (dev_ms_max * 1e-3)
    ms_per_step = dev_ms_max / args.steps
    ns_day = (1000.0 / ms_per_step) * params.dt_fs * 0.0864
    force_s = float(np.mean(fms)) * 1e-3
    pairs_launch = float(np.mean(pstep))
    achieved_tf = pairs_launch * FLOPS_PER_PAIR / force_s / 1e12
    props = torch.cuda.get_device_properties(local)
    max_mhz = clk.get("sm_max_mhz") or measured_peaks().get("sm_max_mhz") or 2070.0
    fp32_peak = props.multi_processor_count * 128 * 2 * max_mhz * 1e6 / 1e12
    hbm_peak = measured_peaks().get("hbm_gbs")
    alg_bytes = sysm.n * (16 + 4 + 24)   # pos+q, type read; int64 x3 force atomics
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "pair-evals/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "ns_per_day": ns_day,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded; shapes of the reference's ApoA1 dataset)",
        "config": {"workload": workload_desc(sysm, params.table_order, params.table_bins),
                   "accumulation": "int64 fixed point 2^-24 (tuned)", "parallelism": f"replicas x{world}",
                   "tile": {"warps_per_cta": tune["tile"][0], "steps_per_piece": tune["tile"][1],
                            "prune_steps": tune["tile"][2],
                            "autotuned": not (args.no_tune or args.tile), "force_ms_tuned": tune["ms"],
                            "force_ms_default_tile": tune["default_ms"]},
                   "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MB write)",
                   "pairs_per_step": pairs_launch},
        "plain": {"value": float(psum[2]) / (float(emax[1]) * 1e-3), "unit": "pair-evals/s",
                  "ms_per_step": float(emax[1]) / kp, "accumulation": "FP32 atomics, default tile (4 warps, 6 steps, no pruning)",
                  "steps": kp,
                  "force_ms": float(np.mean(pfms))},
        "roofline": {"bound": "fp32", "achieved": achieved_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved_tf / fp32_peak, "traffic": committed_traffic(args.workload),
                     "kernel": "k_force (half-shell pair force)", "force_ms": force_s * 1e3,
                     "flops_per_pair": FLOPS_PER_PAIR,
                     "fma_pipe_active_pct_ncu": committed_metric(args.workload, "fma_pipe_active_pct"),
                     "peak_source": f"computed: {props.multi_processor_count} SMs x 128 FP32 lanes x 2 flop x "
                                    f"{max_mhz:.0f} MHz (MEASURED_PEAKS.json has no FP32 figure)"},
        "roofline_hbm": {"achieved": alg_bytes / force_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                         "frac": (alg_bytes / force_s / 1e9 / hbm_peak) if hbm_peak else None,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                         "algorithmic_bytes_per_launch": alg_bytes},
        "e2e": {"value": float(psum[1]) / float(emax[0]), "unit": "pair-evals/s",
                "h2d_bytes_per_step": n * 20, "d2h_bytes_per_step": n * 12,
                "call": "mdrl_force_eval (pinned host x,y,z,q,type in; fx,fy,fz out)", "calls": ke,
                "ms_per_call": e2e_s / ke * 1e3, "device_ms_per_call": e2e_dev / ke,
                "host_link": "pinned buffers read and written in place by the binning and unsort kernels"},
        "with_pme": pme_out,
        "bonded": bonded_out,
        "gpu_launches": 8 * args.steps,
        "clocks": clk,
        "wall_s": wall,
    }
    if world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"], out["force_error"], out["cpu_baseline_allpairs"] = cpu_baseline(sysm, params, args)
    return out


def run_batch(args, rank, world, local, dist):
    """512 independent replicas (N log-uniform 500-20,000, rc 10 A): all of them per step in one
    graph launch, against the same replicas stepped one at a time (each its own graph)."""
    import torch

    import sc2019_md_gb300 as m
    from sc2019_md_gb300 import systems

    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    reps = systems.batch512(args.replicas)
    gen_s = time.perf_counter() - t0
    pos, vel, q, t, spec = systems.concat(reps)
    params = reps[0].params(table_bins=args.bins, table_order=args.order, device=local)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")

    b = m.Batch(params, spec)
    lay = b.layout()
    b.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, q, t)
    tune = b.autotune(retime=True) if not args.no_tune else {"tile": (4, 6, 0), "ms": None, "default_ms": None}
    b.step(args.warmup)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    dev_ms, pairs, pstep = 0.0, 0, []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        st = b.step(1)
        dev_ms += st["device_ms"]
        pairs += st["pairs_total"]
        pstep.append(st["pairs"])
    clk = clocks.stop()
    fms = []
    for _ in range(5):
        flush.zero_()
        torch.cuda.synchronize()
        fms.append(b.time_force())
    b.close()

    # the same replicas one by one: a batch of one replica each, stepped in turn
    k1 = max(3, min(args.steps, 20))
    one_ms, one_pairs = 0.0, 0
    for r, s in enumerate(reps):
        with m.Batch(params, [spec[r]]) as b1:
            b1.set_state(s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.vel, s.q, s.type)
            b1.step(1)
            st = b1.step(k1)
            one_ms += st["device_ms"]
            one_pairs += st["pairs_total"]
    value = pairs / (dev_ms * 1e-3)
    ms_step = dev_ms / args.steps
    force_s = float(np.mean(fms)) * 1e-3
    props = torch.cuda.get_device_properties(local)
    max_mhz = clk.get("sm_max_mhz") or measured_peaks().get("sm_max_mhz") or 2070.0
    fp32_peak = props.multi_processor_count * 128 * 2 * max_mhz * 1e6 / 1e12
    achieved_tf = float(np.mean(pstep)) * FLOPS_PER_PAIR / force_s / 1e12
    npath = np.bincount(lay["path"], minlength=3)
    return {
        "metric": "pair-evals/s, batched replicas (one launch per kernel per step) vs one by one",
        "value": value, "unit": "pair-evals/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded replicas)",
        "config": {"workload": f"batch{len(reps)}: {len(reps)} replicas, {int(b.n)} atoms, N log-uniform "
                               f"500-20000 at 0.1 /A^3, rc 10 A, argon-like +-0.42 e, order-{args.order} "
                               f"{args.bins}-bin tables, int64 fixed point, velocity Verlet 2 fs",
                   "paths": {"half_shell": int(npath[0]), "min_image": int(npath[1]), "all_images": int(npath[2])},
                   "work_items": int(lay["total_items"]), "pairs_per_step": float(np.mean(pstep)),
                   "tile": {"steps_per_piece": tune["tile"][1], "prune_steps": tune["tile"][2],
                            "autotuned": not args.no_tune,
                            "force_ms_tuned": tune["ms"], "force_ms_default_tile": tune["default_ms"]},
                   "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MB write)",
                   "generation_s": gen_s},
        "one_by_one": {"value": one_pairs / (one_ms * 1e-3), "unit": "pair-evals/s", "steps": k1,
                       "ms_per_step": one_ms / k1,
                       "how": "a batch of one replica each (default tile), stepped in turn, each its own graph"},
        "roofline": {"bound": "fp32", "achieved": achieved_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved_tf / fp32_peak, "traffic": committed_traffic("batch512"),
                     "kernel": "k_force (batched work list)",
                     "force_ms": force_s * 1e3, "flops_per_pair": FLOPS_PER_PAIR,
                     "fma_pipe_active_pct_ncu": committed_metric("batch512", "fma_pipe_active_pct")},
        "gpu_launches": 9 * args.steps,
        "clocks": clk,
    }


def oracle_system(sysm, order, bins, arith=0):
    import oracle
    T = len(sysm.sigma)
    pc64 = oracle.lb_coefficients(sysm.sigma, sysm.epsilon)
    m0 = -2
    rc2 = np.float32(np.float32(sysm.cutoff) * np.float32(sysm.cutoff))
    nseg = int(np.floor(np.log2(rc2))) - m0 + 1
    tab = oracle.fit_tables(order, nseg, bins, m0)
    return oracle.System(sysm.pos, sysm.box, sysm.ncell, sysm.cutoff, pc64.astype(np.float32), q=sysm.q,
                         type=sysm.type, ke=sysm.coulomb_k, tab=tab, order=order, nseg=nseg, bins=bins,
                         min_log2=m0, arith=arith, pcoef64=pc64, ke64=sysm.coulomb_k)


def _force_error(F, Fref, vs):
    d = np.linalg.norm(F - Fref, axis=1)
    nrm = np.linalg.norm(Fref, axis=1)
    return {"vs": vs, "max_over_rms": float(d.max() / np.sqrt((nrm ** 2).mean())),
            "median_rel": float(np.median(d / np.maximum(nrm, 1e-30)))}


def cpu_baseline(sysm, params, args):
    """The oracle's multi-threaded cell-list port on the host cores (bounded sample), a bounded
    sample of the C model's all-pairs restatement, and the force error of the GPU's first
    evaluation (tuned and plain) against the FP64 direct oracle and the FP64 evaluation of the
    same tables."""
    import sc2019_md_gb300 as m
    o = oracle_system(sysm, params.table_order, params.table_bins)
    cores = os.cpu_count() or 1
    o.force_cells_mt(cores)                                   # warm
    t0 = time.perf_counter()
    pairs, calls = 0, 0
    while calls < 3 or (time.perf_counter() - t0 < 10.0 and calls < 40):
        _, p = o.force_cells_mt(cores)
        pairs += p
        calls += 1
    el = time.perf_counter() - t0
    base = {"value": pairs / el, "unit": "pair-evals/s", "cores": cores, "kind": "port",
            "sample": f"{calls} full force evaluations of the same system (half-shell cell list, "
                      f"FP32, OpenMP over home cells)", "seconds": el}
    # the C model's all-pairs O(N^2) form: every ordered pair of the first n_ap particles tested,
    # the test rate extrapolated to the full system's N^2 tests and set against the pairs one
    # cell-list evaluation of the full system finds
    n_ap = min(sysm.n, 24000)
    prefix = dataclasses.replace(sysm, pos=sysm.pos[:n_ap], vel=sysm.vel[:n_ap], type=sysm.type[:n_ap],
                                 q=None if sysm.q is None else sysm.q[:n_ap])
    sub = oracle_system(prefix, params.table_order, params.table_bins)
    t1 = time.perf_counter()
    sub.force_allpairs_mt(cores)
    el_ap = time.perf_counter() - t1
    tests_per_s = n_ap * n_ap / el_ap
    full_s = float(sysm.n) ** 2 / tests_per_s
    base_ap = {"value": (pairs / calls) / full_s, "unit": "pair-evals/s", "cores": cores, "kind": "port",
               "sample": f"all {n_ap}^2 ordered pair tests of the first {n_ap} particles (C-model all-pairs "
                         f"form, FP32, OpenMP over i), extrapolated to {sysm.n}^2 tests",
               "pair_tests_per_s": tests_per_s, "full_eval_s": full_s, "seconds": el_ap}
    with m.Context(params) as ctx:
        F, _, _ = ctx.force(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q, sysm.type)
    pp = sysm.params(table_bins=params.table_bins, table_order=params.table_order, device=params.device,
                     accum=m.ACC_FP32_ATOMIC)
    with m.Context(pp) as ctx:
        Fp, _, _ = ctx.force(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q, sysm.type)
    F64, _ = o.force_direct64()
    Ft, _ = o.force_tables64()
    err = {"tuned": [_force_error(F, F64, "FP64 direct oracle, same pair set"),
                     _force_error(F, Ft, "FP64 evaluation of the same tables")],
           "plain": [_force_error(Fp, F64, "FP64 direct oracle, same pair set"),
                     _force_error(Fp, Ft, "FP64 evaluation of the same tables")]}
    return base, err, base_ap


def run_reference(args, rank, world):
    """The CPU implementation of the path (oracle port), every host thread, rank 0 only."""
    if rank != 0:
        return None
    import oracle
    sysm = make_system(args.workload, 0)
    o = oracle_system(sysm, args.order, args.bins)
    cores = os.cpu_count() or 1
    ncells = int(np.prod(sysm.ncell))
    t0 = time.perf_counter()
    o.force_cells_mt(cores)
    full = time.perf_counter() - t0
    # bound the whole run to about two minutes: each step covers a prefix of the home cells
    budget = 120.0 / max(1, args.steps + args.warmup)
    hend = ncells if full <= budget else max(1, int(ncells * budget / full))
    for _ in range(args.warmup):
        o.force_cells_mt(cores, 0, hend)
    pairs, el = 0, 0.0
    for _ in range(args.steps):
        t1 = time.perf_counter()
        _, p = o.force_cells_mt(cores, 0, hend)
        el += time.perf_counter() - t1
        pairs += p
    value = pairs / el
    sample = (f"{hend} of {ncells} home cells per step (half-shell cell-list port of the reference's "
              f"algorithm, FP32, OpenMP)")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pair-evals/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": workload_desc(sysm, args.order, args.bins), "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": "pair-evals/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "pair-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="ljc92k", choices=["ljc92k", "lj1728", "ljc1m", "batch512"])
    ap.add_argument("--no-bonded", action="store_true", help="skip the bonded-term kernel timing")
    ap.add_argument("--replicas", type=int, default=512, help="batch512: number of replicas")
    ap.add_argument("--bins", type=int, default=512)
    ap.add_argument("--order", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default tile (no autotuning)")
    ap.add_argument("--tile", type=lambda v: tuple(int(x) for x in v.split(",")), default=None,
                    help="fixed tile warps,steps,prune instead of autotuning (e.g. 4,6,1)")
    ap.add_argument("--no-pme", action="store_true", help="skip timing the step with smooth-PME electrostatics")
    ap.add_argument("--pme-order", type=int, default=4)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local, dist = dist_setup(args)
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload == "batch512":
        out = run_batch(args, rank, world, local, dist)
    else:
        out = run_ours(args, rank, world, local, dist)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
