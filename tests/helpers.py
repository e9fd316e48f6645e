"""Shared helpers of the test suite: golden fixtures and oracle systems built from a context."""
from __future__ import annotations

from pathlib import Path

import numpy as np

import oracle
import sc2019_md_gb300 as m

GOLDEN = Path(__file__).resolve().parent / "golden"


def kat1():
    d = np.load(GOLDEN / "kat1_pairs.npz")
    tab = np.zeros((2, 2, 14 * 256), np.float32)
    tab[0, 0] = d["c0_14"].view(np.float32)
    tab[0, 1] = d["c1_14"].view(np.float32)
    tab[1, 0] = d["c0_8"].view(np.float32)
    tab[1, 1] = d["c1_8"].view(np.float32)
    return d["pos"].view(np.float32), d["expect"], tab


def kat2_positions():
    """The LJArgon 20k positions as GenInputCellList_LJArgon.m prepares them: parsed in double,
    shifted by the per-axis minimum in double, then cast to single (:64-86)."""
    d = np.load(GOLDEN / "kat2_cells.npz")
    raw = d["micro"].astype(np.float64) / 1e6
    return (raw - raw.min(0)).astype(np.float32), d


def oracle_from_ctx(ctx: m.Context, sysm, arith=None, eval_mode=None):
    """An oracle system with exactly the tables and multipliers the context uses."""
    tab, meta = ctx.tables()
    pc = ctx.pair_coefficients()
    p = ctx.params
    T = p.ntypes
    pc64 = np.zeros((T * T, 4))
    for a in range(T):
        for b in range(T):
            sig = 0.5 * (p.sigma[a] + p.sigma[b])
            eps = np.sqrt(p.epsilon[a] * p.epsilon[b])
            pc64[a * T + b] = [48 * eps * sig ** 12, -24 * eps * sig ** 6, 4 * eps * sig ** 12, -4 * eps * sig ** 6]
    return oracle.System(sysm.pos, sysm.box, sysm.ncell, sysm.cutoff, pc, q=sysm.q, type=sysm.type,
                         ke=p.coulomb_k, tab=tab, order=meta["order"], nseg=meta["nseg"], bins=meta["bins"],
                         min_log2=meta["min_log2"], eval=p.eval if eval_mode is None else eval_mode,
                         arith=p.arith if arith is None else arith, pcoef64=pc64, ke64=p.coulomb_k)


def force_err(F, Fref):
    """(max_i |dF_i| / rms_j |F_ref_j|, median_i |dF_i| / |F_ref_i|) — the two stated norms."""
    d = np.linalg.norm(F - Fref, axis=1)
    n = np.linalg.norm(Fref, axis=1)
    rms = np.sqrt((n ** 2).mean())
    return float(d.max() / rms), float(np.median(d / np.maximum(n, 1e-30)))
