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
                         arith=p.arith if arith is None else arith, pcoef64=pc64, ke64=p.coulomb_k,
                         local=meta["local"], exact=bool(p.flags & m.FLAG_EXACT_DIFF))


def liquid_argon(seed: int = 3):
    """A liquid-argon state point (1,728 atoms in a 36 A box, 120 K, rc 8.5 A, 4x4x4 cells): a
    jittered lattice that melts without exploding, for energy-conservation checks."""
    from sc2019_md_gb300 import systems
    rng = np.random.default_rng(seed)
    L = 36.0
    nside = 12
    g = (np.arange(nside) + 0.5) * (L / nside)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) + rng.uniform(-0.05, 0.05, (nside ** 3, 3))
    pos = systems.wrap_into_box(pos, (L, L, L))
    vel = systems.maxwell(len(pos), np.full(len(pos), 39.95), 120.0, rng)
    return systems.System("argon", (L, L, L), 8.5, (4, 4, 4), pos, vel, None, np.zeros(len(pos), np.int32),
                          [3.4], [0.238], [39.95], 0.0)


def force_err(F, Fref):
    """(max_i |dF_i| / rms_j |F_ref_j|, median_i |dF_i| / |F_ref_i|) — the two stated norms."""
    d = np.linalg.norm(F - Fref, axis=1)
    n = np.linalg.norm(Fref, axis=1)
    rms = np.sqrt((n ** 2).mean())
    return float(d.max() / rms), float(np.median(d / np.maximum(n, 1e-30)))


# ---- the RTL pair generator's input stream (SC/Particle_Pair_Gen_HalfShell.v) -----------------
# Its 8 filters take the half-shell cells in groups of 1, 1, 2, 2, 2, 2, 2, 2 (home first); a line
# per reference particle of the home cell and cycle c holds, for filters 7..0, the c-th particle of
# the filter's concatenated cell lists: "<cell digits><index %2X>" (digits 1/2/3 = -1/0/+1 about
# the home cell, index 1-based in the cell), a valid bit, and positions as FP32 hex in z, y, x order.

def _f32hex(v):
    import struct
    return "%08X" % struct.unpack(">I", struct.pack(">f", float(v)))[0]


def pair_stream_canon_from_text(text):
    """Canonical lines of VERIFICATION_PARTICLE_PAIR_INPUT.txt: every field but the positions of
    invalid slots (which print stale reservoir data)."""
    out = []
    for line in text.replace("\r\n", "\n").split("\n")[1:]:
        if not line:
            continue
        f = line.split("\t")
        ids = [f[1][5 * s:5 * s + 5] for s in range(8)]
        valid = f[2]
        npos = [f[4][24 * s:24 * s + 24] if valid[s] == "1" else "-" for s in range(8)]
        out.append("|".join([f[0]] + ids + [valid, f[3]] + npos))
    return out


def pair_stream_canon_from_cells(pos, cell_list, home, offsets):
    """The same stream rebuilt from cell lists: cell_list(cx, cy, cz) (1-based) returns the particle
    ids of a cell in cell order; offsets = the 14 half-shell offsets, home cell first."""
    groups = [[0], [1], [2, 3], [4, 5], [6, 7], [8, 9], [10, 11], [12, 13]]
    hexpos = lambda i: "".join(_f32hex(v) for v in pos[i][::-1])
    filt = []
    for g in groups:
        lst = []
        for o in g:
            off = offsets[o]
            code = "%d%d%d" % tuple(2 + int(off[d]) for d in range(3))
            ids = cell_list(*(home[d] + int(off[d]) for d in range(3)))
            lst += [(code + "%2X" % (k + 1), i) for k, i in enumerate(ids)]
        filt.append(lst)
    ncyc = max(len(l) for l in filt)
    out = []
    for k, a in enumerate(cell_list(*home)):
        rid = "%d%d%d" % (2, 2, 2) + "%2X" % (k + 1)
        for c in range(ncyc):
            ids, valid, npos = [], "", []
            for s in range(8):
                lst = filt[7 - s]
                if c < len(lst):
                    ids.append(lst[c][0]); valid += "1"; npos.append(hexpos(lst[c][1]))
                else:
                    ids.append("000 0"); valid += "0"; npos.append("-")
            out.append("|".join([rid] + ids + [valid, hexpos(a)] + npos))
    return out


def dhfr_bonded():
    """The DHFR (23,558 atoms) bonded terms and FP32 positions in the box, from the fixture:
    (pos (n, 3) float32, box (3,), {"bonds": (atoms, params), "angles": ..., "dihedrals": ...})."""
    d = np.load(GOLDEN / "dhfr_bonded.npz")
    terms = {k: (d[f"{k}_atoms"], d[f"{k}_table"][d[f"{k}_type"]]) for k in ("bonds", "angles", "dihedrals")}
    return d["pos"], tuple(float(v) for v in d["box"]), terms


def _fma32(a, b, c):
    """float32 fma emulated through float64 (a*b exact; one rounding of the sum, then to float32:
    close enough to choose test positions, which the oracle then checks exactly)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def boundary_dimers(ndimers: int, L: float, rc: float, seed: int, dmin: float = 1.5):
    """Particles in a periodic cube of edge L, in dimers whose r2 under the reference's rounding
    (d = fl(xi - xj) with one +-L wrap, r2 = fl(fl(dx^2 + dy^2) + dz^2)) lies exactly on rc2 or
    one ulp either side of it, and for which r2 computed with a fused multiply-add (fma(dz, dz,
    dx^2 + dy^2) or fma(dy, dy, dx^2) + dz^2) falls on the other side of the cutoff: a kernel that
    lets its compiler contract the r2 arithmetic gets these pairs wrong.  No two particles are
    closer than dmin.  Returns float32 positions (2 ndimers, 3)."""
    f32 = np.float32
    rng = np.random.default_rng(seed)
    Lf, rc2 = f32(L), f32(rc) * f32(rc)
    h = Lf / f32(2)
    steps = np.arange(-6, 7)
    grid = np.stack(np.meshgrid(steps, steps, steps, indexing="ij"), -1).reshape(-1, 3)
    pts = []
    tries = 0
    while len(pts) < 2 * ndimers and tries < 200 * ndimers:
        tries += 1
        xi = (rng.random(3) * L).astype(f32)
        u = rng.standard_normal(3)
        u /= np.linalg.norm(u)
        base = np.mod(xi.astype(np.float64) + rc * u, L).astype(f32)
        # nudge each coordinate of the partner by up to 6 ulps
        xj = base[None, :].copy().repeat(len(grid), 0)
        for a in range(3):
            up = np.nextafter(base[a], f32(np.inf)) - base[a]
            xj[:, a] = (base[a] + grid[:, a].astype(f32) * up).astype(f32)
        if (xj < 0).any() or (xj >= Lf).any():
            continue
        d = (xi[None, :] - xj).astype(f32)
        d = np.where(d > h, (d - Lf).astype(f32), np.where(d < -h, (d + Lf).astype(f32), d)).astype(f32)
        sq = (d * d).astype(f32)
        ref = ((sq[:, 0] + sq[:, 1]).astype(f32) + sq[:, 2]).astype(f32)
        fz = _fma32(d[:, 2], d[:, 2], (sq[:, 0] + sq[:, 1]).astype(f32))
        fy = (_fma32(d[:, 1], d[:, 1], sq[:, 0]) + sq[:, 2]).astype(f32)
        keep_ref = ref <= rc2
        flip = (keep_ref != (fz <= rc2)) | (keep_ref != (fy <= rc2))
        near = np.abs(ref.view(np.int32).astype(np.int64) - int(rc2.view(np.int32))) <= 1
        cand = np.where(flip & near)[0]
        if len(cand) == 0:
            continue
        pj = xj[rng.choice(cand)]
        if pts:
            P = np.asarray(pts, dtype=np.float64)
            for q in (xi, pj):
                dd = np.abs(P - q.astype(np.float64))
                dd = np.minimum(dd, L - dd)
                if (np.sqrt((dd ** 2).sum(1)) < dmin).any():
                    break
            else:
                pts += [xi, pj]
        else:
            pts += [xi, pj]
    if len(pts) < 2 * ndimers:
        raise RuntimeError("could not place the dimers")
    return np.asarray(pts, dtype=f32)
