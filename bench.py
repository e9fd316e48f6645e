#!/usr/bin/env python3
"""bench.py — throughput of the range-limited force path (pair-evals/s and ns/day).

A step is one velocity-Verlet MD step of the whole system on the GPU: kick + drift + rebin
(count, scan, scatter, in-cell sort, gather), the half-shell force kernel, kick.  Default
workload: the 92,224-atom LJ+Coulomb system (108.86 x 108.86 x 77.76 A, rc 12 A, 9x9x6 cells,
4 types, +-0.42 e).  "tuned" = int64 fixed-point accumulation, autotuned tile, the exact-difference
rule and bin-local order-2 512-bin tables (within 1e-5 of the FP64 oracle in max |dF| / rms |F|);
"plain" = FP32-atomic accumulation and the default tile with the same datapath and tables;
"reference_datapath" = the reference's difference rule and order-1 tables (pair list bit-equal to
the reference's).  The same run also measures the 1,048,576-atom system and the 512-replica batch
(sub-objects "ljc1m" and "batch512"), smooth PME and the bonded terms.

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference] [--workload ...]

N > 1 (one process per GPU under torch.distributed.run) runs N independent replicas (seed offset
= rank): the path has no exchange step on one node, so value = pairs of all ranks / max time.
--impl reference times the CPU implementation of the same path (the oracle's multi-threaded
cell-list port) on rank 0 with every host thread.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes as C
import json
import multiprocessing as mp
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
BYTES_PER_PARTICLE = 16 + 4 + 24   # pos+q and type read, int64 x3 force atomics, per force launch
L2_FLUSH_BYTES = 256 << 20     # > 129 MB L2
METRIC = "pair-evals/s & ns/day, 92k-atom RL LJ+Coulomb, tuned vs plain @1e-5 force err"
CAPTURES = ROOT / "profiles" / "ncu_captures.json"   # per-capture ncu figures (workload, tile, datapath)


def make_system(name: str, seed_offset: int = 0):
    from sc2019_md_gb300 import systems
    if name == "ljc92k":
        return systems.ljc92k(seed_offset=seed_offset)
    if name == "lj1728":
        return systems.lj1728(seed_offset=seed_offset)
    if name == "ljc1m":
        return systems.ljc1m(seed_offset=seed_offset)
    if name == "batch512":
        return systems.batch512()
    raise SystemExit(f"unknown workload {name}")


def workload_desc(sysm) -> str:
    nc = "x".join(str(c) for c in sysm.ncell)
    box = "x".join(f"{b:g}" for b in sysm.box)
    kind = "LJ+Coulomb" if sysm.coulomb_k else "LJ"
    return (f"{sysm.name}: {sysm.n} atoms, {box} A periodic, rc {sysm.cutoff:g} A, {nc} cells, "
            f"{len(sysm.sigma)} types, {kind}, velocity Verlet 2 fs")


def method_desc(order: int, bins: int, exact: bool) -> str:
    form = "bin-local" if order >= 2 else "monomial"
    return (f"order-{order} {bins}-bin {form} tables, "
            + ("exact minimum-image differences" if exact else "reference difference rule fl(fl(xi-xj)+-L)"))


def tile_str(t) -> str:
    return f"{t[0]}x{t[1]}x{t[2]} (warps per CTA x j-steps per piece x pruning)"


class Clocks:
    """nvidia-smi samples every 20 ms while running (SM clock, max clock, throttle reasons)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self, window: str = "0.3 s of back-to-back warm-up steps right before the timed steps, then the timed steps"):
        self.window = window
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

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
        sm, mx, busy, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [v.strip() for v in l.split(",")]
            if len(f) < 8:
                continue
            try:
                s, mxv = float(f[0]), float(f[1])
            except ValueError:
                continue
            try:
                u = float(f[7])
            except ValueError:
                u = 1.0
            sm.append(s)
            mx.append(mxv)
            busy.append(u)
            for k, nm in enumerate(names):
                if f[3 + k].lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        loaded = [s for s, u in zip(sm, busy) if u > 0] or sm
        return {"sm_mhz": float(np.median(loaded)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm), "samples_under_load": len([u for u in busy if u > 0]),
                "window": self.window, "interval_ms": 20}


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


def ncu_capture(workload: str, tile, order: int, bins: int, exact: bool, min_log2: int) -> dict:
    """The committed ncu figures for this kernel configuration, or a record saying none matches.
    Each capture names the tile, tables and datapath it was taken with; figures of another
    configuration are not reported for this one."""
    want = {"workload": workload, "tile": list(tile), "order": order, "bins": bins, "exact": bool(exact),
            "table_min_log2": min_log2}
    try:
        caps = json.loads(CAPTURES.read_text())
    except (OSError, json.JSONDecodeError):
        caps = []
    for c in caps:
        if all(c.get(k) == v for k, v in want.items()):
            return {"matched": True, "source": f"profiles/{CAPTURES.name}", **c}
    near = [c for c in caps if c.get("workload") == workload]
    return {"matched": False, "source": f"profiles/{CAPTURES.name}", "wanted": want,
            "captured": [{k: c.get(k) for k in want if k != "workload"} for c in near]}


def fp32_peak_tflops(props, mhz: float) -> float:
    return props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12


def _generate(name: str):
    """Worker of the spawned generation pool (no CUDA in this process)."""
    return make_system(name)


class Flush:
    def __init__(self, device):
        import torch
        self.buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)

    def __call__(self):
        import torch
        self.buf.zero_()
        torch.cuda.synchronize()


def md_leg(m, obj, steps: int, warmup: int, flush, nkernel: int = 12):
    """Warm-up steps, then `steps` timed steps one graph launch each (L2 flushed before each);
    then the force kernel alone nkernel times.  obj is a Context or Batch with state set."""
    obj.step(warmup)
    dev_ms, pairs, pstep = 0.0, 0, []
    for _ in range(steps):
        flush()
        st = obj.step(1)
        dev_ms += st["device_ms"]
        pairs += st["pairs_total"]
        pstep.append(st["pairs"])
    fms = []
    for _ in range(nkernel):
        flush()
        fms.append(obj.time_force())
    return {"dev_ms": dev_ms, "pairs": pairs, "pairs_per_step": float(np.mean(pstep)) if pstep else 0.0,
            "force_ms": float(np.median(fms)), "steps": steps}


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


def e2e_leg(m, params, sysm, tile, warmup: int, calls: int, flush):
    """mdrl_force_eval end to end on pinned host buffers, host-timed per call."""
    import torch
    n = sysm.n
    pin = lambda dt: torch.empty(n, dtype=dt, pin_memory=True).numpy()
    bufs = {k: pin(torch.float32) for k in ("x", "y", "z", "q", "fx", "fy", "fz")}
    bufs["t"] = pin(torch.int32)
    for k, v in (("x", sysm.pos[:, 0]), ("y", sysm.pos[:, 1]), ("z", sysm.pos[:, 2]), ("q", sysm.q),
                 ("t", sysm.type)):
        bufs[k][:] = v
    with m.Context(params) as ctx:
        ctx.set_tile(*tile)
        for _ in range(warmup):
            force_eval_pinned(m, ctx, bufs, n)
        secs, pairs, dev = 0.0, 0, 0.0
        for _ in range(calls):
            flush()
            t1 = time.perf_counter()
            st = force_eval_pinned(m, ctx, bufs, n)
            secs += time.perf_counter() - t1
            pairs += st.pairs
            dev += st.device_ms
    return {"secs": secs, "pairs": pairs, "calls": calls, "dev_ms": dev, "n": n}


def force_kernel_name(tile, batch: bool = False) -> str:
    if tile and tile[0] == 1:
        return ("k_force_warp (half-shell pair force, one warp per unit x i-tile group)" if not batch else
                "k_force_warp for the half-shell replicas + k_force for the small ones (one force evaluation)")
    return "k_force (half-shell pair force, one CTA per unit)"


def roofline(pairs_per_launch: float, force_ms: float, n: int, props, mhz: float, capture: dict,
             kernel: str = "k_force (half-shell pair force)") -> dict:
    achieved = pairs_per_launch * FLOPS_PER_PAIR / (force_ms * 1e-3) / 1e12
    peak = fp32_peak_tflops(props, mhz)
    alg_bytes = n * BYTES_PER_PARTICLE
    hbm = measured_peaks().get("hbm_gbs")
    return {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "traffic": capture.get("dram_bytes_per_launch") if capture.get("matched") else None,
            "kernel": kernel, "force_ms": force_ms, "flops_per_pair": FLOPS_PER_PAIR,
            "algorithmic_bytes_per_launch": alg_bytes,
            "hbm_achieved_gbs": alg_bytes / (force_ms * 1e-3) / 1e9, "hbm_peak_gbs": hbm,
            "peak_source": f"computed: {props.multi_processor_count} SMs x 128 FP32 lanes x 2 flop x {mhz:.0f} MHz "
                           f"(MEASURED_PEAKS.json has no FP32 figure); hbm_peak_gbs of measured",
            "ncu_summary": capture}


def _force_error(F, Fref, vs):
    d = np.linalg.norm(F - Fref, axis=1)
    nrm = np.linalg.norm(Fref, axis=1)
    return {"vs": vs, "max_over_rms": float(d.max() / np.sqrt((nrm ** 2).mean())),
            "median_rel": float(np.median(d / np.maximum(nrm, 1e-30)))}


def oracle_system(sysm, order, bins, arith=0, exact=False):
    import oracle
    pc64 = oracle.lb_coefficients(sysm.sigma, sysm.epsilon)
    m0 = sysm.table_min_log2
    rc2 = np.float32(np.float32(sysm.cutoff) * np.float32(sysm.cutoff))
    nseg = int(np.floor(np.log2(rc2))) - m0 + 1
    tab = oracle.fit_tables(order, nseg, bins, m0, local=order >= 2)
    return oracle.System(sysm.pos, sysm.box, sysm.ncell, sysm.cutoff, pc64.astype(np.float32), q=sysm.q,
                         type=sysm.type, ke=sysm.coulomb_k, tab=tab, order=order, nseg=nseg, bins=bins,
                         min_log2=m0, arith=arith, pcoef64=pc64, ke64=sysm.coulomb_k, local=order >= 2,
                         exact=exact)


def cpu_port_rate(o, cores: int, budget_s: float = 10.0):
    """The oracle's OpenMP half-shell port: full force evaluations for about budget_s seconds."""
    o.force_cells_mt(cores)
    t0 = time.perf_counter()
    pairs, calls = 0, 0
    while calls < 3 or (time.perf_counter() - t0 < budget_s and calls < 40):
        _, p = o.force_cells_mt(cores)
        pairs += p
        calls += 1
    el = time.perf_counter() - t0
    return pairs / el, calls, el


def accuracy(m, sysm, legs: dict) -> dict:
    """Force error of each leg's first evaluation against the FP64 direct oracle (and the FP64
    evaluation of the same tables), both stated norms."""
    out, cache = {}, {}
    for name, (params, order, bins, exact) in legs.items():
        with m.Context(params) as ctx:
            F, _, _ = ctx.force(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q, sysm.type)
        key = (order, bins, exact)
        if key not in cache:
            o = oracle_system(sysm, order, bins, exact=exact)
            cache[key] = (o.force_direct64()[0], o.force_tables64()[0])
        F64, Ft = cache[key]
        out[name] = [_force_error(F, F64, "FP64 direct oracle, same pair set"),
                     _force_error(F, Ft, "FP64 evaluation of the same tables")]
    return out


def single_system(m, sysm, args, local, flush, clocks=None, barrier=lambda: None):
    """Tuned (timed, autotuned), plain and reference-datapath legs of one system."""
    base = dict(table_bins=args.bins, device=local)
    exact = args.datapath == "exact"
    fl = m.FLAG_EXACT_DIFF if exact else 0
    p_tuned = sysm.params(table_order=args.order, flags=fl, **base)
    p_plain = sysm.params(table_order=args.order, flags=fl, accum=m.ACC_FP32_ATOMIC, **base)
    p_ref = sysm.params(table_order=1, **base)
    st_args = (sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
    out = {"params": {"tuned": p_tuned, "plain": p_plain, "reference_datapath": p_ref}}

    with m.Context(p_tuned) as ctx:
        ctx.set_state(*st_args)
        if args.tile:
            ctx.set_tile(*args.tile)
            tune = {"tile": ctx.tile(), "ms": None, "default_ms": None}
        elif args.no_tune:
            tune = {"tile": ctx.tile(), "ms": None, "default_ms": None}
        else:
            tune = ctx.autotune(retime=True)
        ctx.step(args.warmup)
        if clocks is not None:
            clocks.start()     # sample the clocks under sustained load: warm-up steps back to back, then the timed steps
            t_soak = time.perf_counter()
            while time.perf_counter() - t_soak < 0.3:
                ctx.step(20)
        barrier()
        t0 = time.perf_counter()
        leg = md_leg(m, ctx, args.steps, 0, flush, nkernel=max(3, min(args.steps, 20)))
        barrier()
        out["wall_s"] = time.perf_counter() - t0
        out["clocks"] = clocks.stop() if clocks is not None else None
    out["tuned"] = {**leg, "tile": tune["tile"], "tune": tune}

    kp = max(3, min(args.steps, 50))
    with m.Context(p_plain) as ctx:
        ctx.set_state(*st_args)
        out["plain"] = md_leg(m, ctx, kp, args.warmup, flush, nkernel=5)
        out["plain"]["tile"] = ctx.tile()

    with m.Context(p_ref) as ctx:
        ctx.set_state(*st_args)
        rtune = ctx.autotune(retime=True) if not args.no_tune else {"tile": ctx.tile()}
        out["reference_datapath"] = md_leg(m, ctx, kp, args.warmup, flush, nkernel=5)
        out["reference_datapath"]["tile"] = rtune["tile"]

    out["e2e"] = e2e_leg(m, p_tuned, sysm, tune["tile"], args.warmup, max(3, min(args.steps, 30)), flush)
    return out


def sub_workload_single(m, sysm, args, local, flush, props):
    """Tuned vs plain MD steps, kernel timing and e2e of a second single system (the 1M-atom one)."""
    exact = args.datapath == "exact"
    fl = m.FLAG_EXACT_DIFF if exact else 0
    k = max(3, min(args.steps, 10))
    p_t = sysm.params(table_order=args.order, table_bins=args.bins, device=local, flags=fl)
    p_p = sysm.params(table_order=args.order, table_bins=args.bins, device=local, flags=fl,
                      accum=m.ACC_FP32_ATOMIC)
    st_args = (sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
    with m.Context(p_t) as ctx:
        ctx.set_state(*st_args)
        tune = ctx.autotune(retime=True) if not args.no_tune else {"tile": ctx.tile(), "ms": None, "default_ms": None}
        tuned = md_leg(m, ctx, k, args.warmup, flush, nkernel=5)
    with m.Context(p_p) as ctx:
        ctx.set_state(*st_args)
        plain = md_leg(m, ctx, k, args.warmup, flush, nkernel=5)
    e2e = e2e_leg(m, p_t, sysm, tune["tile"], 2, 3, flush)
    mhz = measured_peaks().get("sm_max_mhz") or 2070.0
    ms = tuned["dev_ms"] / k
    return {
        "workload": workload_desc(sysm) + "; " + method_desc(args.order, args.bins, exact),
        "value": tuned["pairs"] / (tuned["dev_ms"] * 1e-3), "unit": "pair-evals/s", "steps": k,
        "warmup": args.warmup, "ms_per_step": ms, "ns_per_day": (1000.0 / ms) * 2.0 * 0.0864,
        "tile": tile_str(tune["tile"]), "force_ms_tuned_tile": tune.get("ms"),
        "force_ms_default_tile": tune.get("default_ms"),
        "plain": {"value": plain["pairs"] / (plain["dev_ms"] * 1e-3), "ms_per_step": plain["dev_ms"] / k,
                  "force_ms": plain["force_ms"], "accumulation": "FP32 atomics, default tile, same datapath"},
        "tuned_over_plain": (plain["dev_ms"] / tuned["dev_ms"]) if tuned["dev_ms"] else None,
        "roofline": roofline(tuned["pairs_per_step"], tuned["force_ms"], sysm.n, props, mhz,
                             ncu_capture(sysm.name, tune["tile"], args.order, args.bins, exact, sysm.table_min_log2),
                             force_kernel_name(tune["tile"])),
        "e2e": {"value": e2e["pairs"] / e2e["secs"], "unit": "pair-evals/s", "h2d_bytes_per_step": sysm.n * 20,
                "d2h_bytes_per_step": sysm.n * 12, "calls": e2e["calls"],
                "ms_per_call": e2e["secs"] / e2e["calls"] * 1e3},
        "pairs_per_step": tuned["pairs_per_step"],
        "gpu_launches": 8 * k,
    }


def sub_workload_batch(m, reps, args, local, flush, props):
    """The batched replicas: one graph launch per step for all of them, against the same replicas
    stepped one at a time; kernel timing and e2e (host buffers through mdrl_batch_force_eval)."""
    from sc2019_md_gb300 import systems
    pos, vel, q, t, spec = systems.concat(reps)
    params = reps[0].params(table_bins=args.bins, table_order=1, device=local)
    k = max(3, min(args.steps, 10))
    with m.Batch(params, spec) as b:
        lay = b.layout()
        b.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, q, t)
        if args.tile:
            b.set_tile(*args.tile)
            tune = {"tile": tuple(args.tile), "ms": None, "default_ms": None}
        elif args.no_tune:
            tune = {"tile": (4, 6, 0), "ms": None, "default_ms": None}
        else:
            tune = b.autotune(retime=True)
        leg = md_leg(m, b, k, args.warmup, flush, nkernel=5)
    with m.Batch(params, spec) as b:       # e2e: host arrays in and out (copies inside the call)
        b.set_tile(*tune["tile"])
        b.force(pos[:, 0], pos[:, 1], pos[:, 2], q, t)
        e_secs, e_pairs = 0.0, 0
        for _ in range(3):
            flush()
            t1 = time.perf_counter()
            _, st, _ = b.force(pos[:, 0], pos[:, 1], pos[:, 2], q, t)
            e_secs += time.perf_counter() - t1
            e_pairs += st["pairs"]
    k1 = 3
    one_ms, one_pairs = 0.0, 0
    for r, s in enumerate(reps):
        with m.Batch(params, [spec[r]]) as b1:
            b1.set_state(s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.vel, s.q, s.type)
            b1.step(1)
            st = b1.step(k1)
            one_ms += st["device_ms"]
            one_pairs += st["pairs_total"]
    ntot = len(pos)
    mhz = measured_peaks().get("sm_max_mhz") or 2070.0
    npath = np.bincount(lay["path"], minlength=3)
    value = leg["pairs"] / (leg["dev_ms"] * 1e-3)
    one = one_pairs / (one_ms * 1e-3)
    return {
        "workload": (f"batch{len(reps)}: {len(reps)} replicas, {ntot} atoms, N log-uniform 500-20000 at 0.1 /A^3, "
                     f"rc 10 A, argon-like +-0.42 e; order-1 {args.bins}-bin tables, reference difference rule, "
                     f"int64 fixed point"),
        "value": value, "unit": "pair-evals/s", "steps": k, "warmup": args.warmup,
        "ms_per_step": leg["dev_ms"] / k, "tile": tile_str(tune["tile"]),
        "paths": {"half_shell": int(npath[0]), "min_image": int(npath[1]), "all_images": int(npath[2])},
        "work_items": int(lay["total_items"]),
        "one_by_one": {"value": one, "unit": "pair-evals/s", "steps": k1, "ms_per_step": one_ms / k1,
                       "how": "a batch of one replica each (default tile), stepped in turn, each its own graph"},
        "batched_over_one_by_one": value / one if one else None,
        "roofline": roofline(leg["pairs_per_step"], leg["force_ms"], ntot, props, mhz,
                             ncu_capture("batch512", tune["tile"], 1, args.bins, False, reps[0].table_min_log2),
                             force_kernel_name(tune["tile"], batch=True)),
        "e2e": {"value": e_pairs / e_secs, "unit": "pair-evals/s", "h2d_bytes_per_step": ntot * 20,
                "d2h_bytes_per_step": ntot * 12, "calls": 3, "ms_per_call": e_secs / 3 * 1e3,
                "call": "mdrl_batch_force_eval (host x,y,z,q,type in; fx,fy,fz out)"},
        "pairs_per_step": leg["pairs_per_step"],
        "gpu_launches": 9 * k,
    }


def run_ours(args, rank, world, local, dist):
    import torch

    import sc2019_md_gb300 as m
    from sc2019_md_gb300 import systems

    # the larger workloads are generated on the host while the GPU measures the first one
    extra = world == 1 and not args.no_extra and args.workload == "ljc92k"
    pool = futs = None
    if extra:
        pool = cf.ProcessPoolExecutor(max_workers=2, mp_context=mp.get_context("spawn"))
        futs = {name: pool.submit(_generate, name) for name in ("ljc1m", "batch512")}

    torch.cuda.set_device(local)
    sysm = make_system(args.workload, rank)
    flush = Flush(f"cuda:{local}")
    props = torch.cuda.get_device_properties(local)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    exact = args.datapath == "exact"
    res = single_system(m, sysm, args, local, flush, Clocks(local), barrier)
    tuned, plain, refd, e2e = res["tuned"], res["plain"], res["reference_datapath"], res["e2e"]
    clk = res["clocks"]

    # ---- the same step with smooth-PME long-range electrostatics (charged systems) -----------
    pme_out = None
    if not args.no_pme and sysm.q is not None:
        with m.Context(res["params"]["tuned"]) as ctxl:
            pme_p = ctxl.set_pme(order=args.pme_order)
            ctxl.set_state(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
            ctxl.set_tile(*tuned["tile"])
            kl = max(3, min(args.steps, 50))
            leg = md_leg(m, ctxl, kl, args.warmup, flush, nkernel=1)
        pme_out = {"value": leg["pairs"] / (leg["dev_ms"] * 1e-3), "unit": "pair-evals/s",
                   "ms_per_step": leg["dev_ms"] / kl, "ns_per_day": (1000.0 / (leg["dev_ms"] / kl)) * 2.0 * 0.0864,
                   "steps": kl, "beta": pme_p["beta"], "grid": list(pme_p["grid"]), "order": pme_p["order"],
                   "note": "same step + PME reciprocal part (spread, 2 FFTs, gather); real space in the pair tables"}

    # ---- bonded terms: their kernels alone, on a chain topology of the same size ------------
    bonded_out = None
    if not args.no_bonded:
        nch = sysm.n // 30
        Lc = float((nch * 30 / 0.1) ** (1.0 / 3.0))
        csys, T = systems.chains(nch, 30, Lc, seed=20191117 + 6, cutoff=12.0, dmin=0.0)
        with m.Context(csys.params(table_bins=args.bins, device=local)) as ctxb:
            ctxb.set_bonded(**T)
            ctxb.set_state(csys.pos[:, 0], csys.pos[:, 1], csys.pos[:, 2], csys.vel, None, csys.type)
            bms = []
            for _ in range(max(3, min(args.steps, 20))):
                flush()
                bms.append(ctxb.time_bonded())
        nterms = sum(len(v[0]) for v in T.values())
        bmed = float(np.median(bms))
        bonded_out = {"terms": nterms, "bonds": len(T["bonds"][0]), "angles": len(T["angles"][0]),
                      "dihedrals": len(T["dihedrals"][0]), "ms": bmed, "terms_per_s": nterms / (bmed * 1e-3),
                      "workload": f"{csys.n} atoms as {nch} chains of 30 in a {Lc:.1f} A cube (density 0.1), "
                                  f"FP32 terms into the int64 accumulators; kernels alone (inverse map + terms), "
                                  f"L2 flushed"}

    # ---- reduce over ranks -----------------------------------------------------------------
    mx, sm = combine_ranks(dist, f"cuda:{local}", maxes=[tuned["dev_ms"], e2e["secs"], plain["dev_ms"]],
                           sums=[tuned["pairs"], e2e["pairs"], plain["pairs"]])
    if rank != 0:
        if pool:
            pool.shutdown(cancel_futures=True)
        return None
    value = sm[0] / (mx[0] * 1e-3)
    ms_per_step = mx[0] / args.steps
    mhz = (clk or {}).get("sm_max_mhz") or measured_peaks().get("sm_max_mhz") or 2070.0
    cap = ncu_capture(args.workload, tuned["tile"], args.order, args.bins, exact, sysm.table_min_log2)
    kp = plain["steps"]
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "pair-evals/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "ns_per_day": (1000.0 / ms_per_step) * 2.0 * 0.0864,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded; shapes of the reference's ApoA1 dataset)",
        "config": {"workload": workload_desc(sysm), "method": method_desc(args.order, args.bins, exact),
                   "accumulation": "int64 fixed point 2^-24 (tuned)", "parallelism": f"replicas x{world}",
                   "tile": tile_str(tuned["tile"]), "autotuned": not (args.no_tune or args.tile),
                   "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MB write)",
                   "pairs_per_step": tuned["pairs_per_step"]},
        "plain": {"value": sm[2] / (mx[2] * 1e-3), "unit": "pair-evals/s", "ms_per_step": mx[2] / kp,
                  "steps": kp, "force_ms": plain["force_ms"], "tile": tile_str(plain["tile"]),
                  "accumulation": "FP32 atomics, default tile, same datapath and tables"},
        "tuned_over_plain": mx[2] / kp / ms_per_step,
        "reference_datapath": {"value": refd["pairs"] / (refd["dev_ms"] * 1e-3), "unit": "pair-evals/s",
                               "ms_per_step": refd["dev_ms"] / refd["steps"], "force_ms": refd["force_ms"],
                               "tile": tile_str(refd["tile"]), "method": method_desc(1, args.bins, False),
                               "pairs_per_step": refd["pairs_per_step"],
                               "note": "int64 fixed point, autotuned; pair list bit-equal to the reference's datapath"},
        "roofline": roofline(tuned["pairs_per_step"], tuned["force_ms"], sysm.n, props, mhz, cap,
                             force_kernel_name(tuned["tile"])),
        "e2e": {"value": sm[1] / mx[1], "unit": "pair-evals/s", "h2d_bytes_per_step": sysm.n * 20,
                "d2h_bytes_per_step": sysm.n * 12,
                "call": "mdrl_force_eval (pinned host x,y,z,q,type in; fx,fy,fz out)", "calls": e2e["calls"],
                "ms_per_call": e2e["secs"] / e2e["calls"] * 1e3, "device_ms_per_call": e2e["dev_ms"] / e2e["calls"],
                "host_link": "pinned buffers read and written in place by the binning and unsort kernels"},
        "with_pme": pme_out,
        "bonded": bonded_out,
        "gpu_launches": 8 * args.steps,
        "clocks": clk,
        "wall_s": res["wall_s"],
    }
    if world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        o = oracle_system(sysm, args.order, args.bins, exact=exact)
        rate, calls, el = cpu_port_rate(o, cores)
        out["cpu_baseline"] = {"value": rate, "unit": "pair-evals/s", "cores": cores, "kind": "port",
                               "sample": f"{calls} full force evaluations of the same system and datapath "
                                         f"(half-shell cell list, FP32, OpenMP over home cells)", "seconds": el}
        out["force_error"] = accuracy(m, sysm, {
            "tuned": (res["params"]["tuned"], args.order, args.bins, exact),
            "plain": (res["params"]["plain"], args.order, args.bins, exact),
            "reference_datapath": (res["params"]["reference_datapath"], 1, args.bins, False)})
        out["force_error"]["norm"] = "max_i |dF_i| / rms_j |F_j| (primary); median_i |dF_i| / |F_i|"
    if extra:
        try:
            out["ljc1m"] = sub_workload_single(m, futs["ljc1m"].result(), args, local, flush, props)
            out["batch512"] = sub_workload_batch(m, futs["batch512"].result(), args, local, flush, props)
        finally:
            pool.shutdown()
    return out


def run_batch(args, rank, world, local, dist):
    """The batched workload as the headline (--workload batch512)."""
    import torch

    import sc2019_md_gb300 as m

    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    reps = make_system("batch512")
    gen_s = time.perf_counter() - t0
    flush = Flush(f"cuda:{local}")
    props = torch.cuda.get_device_properties(local)
    clocks = Clocks(local).start("the whole batch run: tuning, timed steps, e2e calls, the replicas one by one")
    sub = sub_workload_batch(m, reps, args, local, flush, props)
    clk = clocks.stop()
    return {"metric": "pair-evals/s, batched replicas (one launch per kernel per step) vs one by one",
            "n_gpus": world, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded replicas)", "clocks": clk, "generation_s": gen_s,
            "config": {"workload": sub["workload"], "tile": sub["tile"],
                       "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MB write)"},
            **{k: v for k, v in sub.items() if k not in ("workload", "tile")}}


def run_reference(args, rank, world):
    """The CPU implementation of the path (oracle port) on the same workload, datapath and tables,
    every host thread, rank 0 only; each step is a bounded sample of the home cells."""
    if rank != 0:
        return None
    sysm = make_system(args.workload, 0)
    exact = args.datapath == "exact"
    o = oracle_system(sysm, args.order, args.bins, exact=exact)
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
        "data": "synthetic (seeded; shapes of the reference's ApoA1 dataset)",
        "config": {"workload": workload_desc(sysm), "method": method_desc(args.order, args.bins, exact),
                   "accumulation": "FP32 per-pair forces, FP64 sums (CPU port)",
                   "parallelism": f"{cores} host threads", "tile": "none (CPU: OpenMP over home cells)",
                   "autotuned": False, "l2": "host caches (CPU)", "pairs_per_step": pairs / args.steps},
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
    ap.add_argument("--datapath", choices=["exact", "reference"], default="exact",
                    help="difference rule of the tuned and plain arms (MDRL_FLAG_EXACT_DIFF or the reference's)")
    ap.add_argument("--no-bonded", action="store_true", help="skip the bonded-term kernel timing")
    ap.add_argument("--no-extra", action="store_true", help="skip the 1M-atom and 512-replica sub-workloads")
    ap.add_argument("--bins", type=int, default=512)
    ap.add_argument("--order", type=int, default=2)
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
