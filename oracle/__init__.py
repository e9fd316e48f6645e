"""ctypes wrapper of the CPU oracle (oracle.cpp, bonded.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm, as the checker or the timed CPU baseline.  The product package
(sc2019_md_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


class OrcSys(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("x", _F), ("y", _F), ("z", _F), ("q", _F), ("type", _I),
        ("box", C.c_float * 3), ("ncell", C.c_int * 3), ("rc2", C.c_float), ("ntypes", C.c_int),
        ("pcoef", _F), ("ke", C.c_float), ("eval", C.c_int), ("arith", C.c_int),
        ("order", C.c_int), ("nseg", C.c_int), ("bins", C.c_int), ("min_log2", C.c_int),
        ("tab", _F), ("pcoef64", _D), ("ke64", C.c_double), ("local", C.c_int), ("exact", C.c_int),
    ]


class OrcBonded(C.Structure):
    _fields_ = [("nb", C.c_int), ("bond_atoms", _I), ("bond_par", _D), ("na", C.c_int), ("angle_atoms", _I),
                ("angle_par", _D), ("nd", C.c_int), ("dih_atoms", _I), ("dih_par", _D)]


class OrcStats(C.Structure):
    _fields_ = [("pairs", C.c_int64), ("candidates", C.c_int64), ("below_table", C.c_int64),
                ("e_lj", C.c_double), ("e_coul", C.c_double), ("virial", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        from .build import build
        L = C.CDLL(str(build()))
        L.orc_bin.argtypes = [C.c_int, _F, _F, _F, _F, _I, _I, _I, _I]
        L.orc_pair_f32.argtypes = [C.POINTER(OrcSys), C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                   C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, _F]
        L.orc_force_cells.argtypes = [C.POINTER(OrcSys), _D, _D, _I, C.POINTER(OrcStats)]
        L.orc_force_direct64.argtypes = [C.POINTER(OrcSys), _D, C.POINTER(OrcStats)]
        L.orc_force_tables64.argtypes = [C.POINTER(OrcSys), _D, C.POINTER(OrcStats)]
        L.orc_force_split64.argtypes = [C.POINTER(OrcSys), C.c_int, C.c_int, _D, C.POINTER(OrcStats)]
        L.orc_force_cells_fixed.argtypes = [C.POINTER(OrcSys), C.c_int, C.c_int, C.POINTER(C.c_int64)]
        L.orc_force_cells_fixed.restype = C.c_int64
        L.orc_force_cells_mt.argtypes = [C.POINTER(OrcSys), C.c_int, C.c_int, C.c_int, _F]
        L.orc_force_cells_mt.restype = C.c_int64
        L.orc_force_allpairs_mt.argtypes = [C.POINTER(OrcSys), C.c_int, _F]
        L.orc_force_allpairs_mt.restype = C.c_int64
        L.orc_force_allimage.argtypes = [C.POINTER(OrcSys), _D, _D, _D, _I, C.POINTER(OrcStats)]
        L.orc_force_allimage.restype = C.c_int64
        L.orc_ewald64.argtypes = [C.POINTER(OrcSys), C.c_double, C.c_int, _D, _D]
        L.orc_cmodel_run.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, _F, _F, _F, _I]
        L.orc_bonded64.argtypes = [C.c_int, _D, _D, _D, _D, C.POINTER(OrcBonded), _D, _D]
        _lib = L
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


class System:
    """Arrays + parameters of one system, kept alive for the C structure that points at them."""

    def __init__(self, pos, box, ncell, cutoff, pcoef, q=None, type=None, ke=0.0, tab=None,
                 order=1, nseg=0, bins=256, min_log2=-2, eval=0, arith=0, pcoef64=None, ke64=0.0,
                 local=False, exact=False):
        pos = np.asarray(pos, np.float32)
        self.x = np.ascontiguousarray(pos[:, 0])
        self.y = np.ascontiguousarray(pos[:, 1])
        self.z = np.ascontiguousarray(pos[:, 2])
        n = len(self.x)
        self.q = None if q is None else np.ascontiguousarray(q, np.float32)
        self.type = np.zeros(n, np.int32) if type is None else np.ascontiguousarray(type, np.int32)
        self.pcoef = np.ascontiguousarray(pcoef, np.float32).ravel()
        self.pcoef64 = None if pcoef64 is None else np.ascontiguousarray(pcoef64, np.float64).ravel()
        self.tab = None if tab is None else np.ascontiguousarray(tab, np.float32)
        s = OrcSys()
        s.n = n
        s.x, s.y, s.z = _p(self.x, _F), _p(self.y, _F), _p(self.z, _F)
        s.q, s.type = _p(self.q, _F), _p(self.type, _I)
        for d in range(3):
            s.box[d] = np.float32(box[d])
            s.ncell[d] = int(ncell[d])
        rcf = np.float32(cutoff)
        s.rc2 = np.float32(rcf * rcf)
        s.ntypes = int(round(np.sqrt(len(self.pcoef) // 4)))
        s.pcoef = _p(self.pcoef, _F)
        s.ke = np.float32(ke)
        s.eval, s.arith = eval, arith
        s.order, s.nseg, s.bins, s.min_log2 = order, nseg, bins, min_log2
        s.tab = _p(self.tab, _F)
        s.pcoef64 = _p(self.pcoef64, _D)
        s.ke64 = ke64
        s.local = int(bool(local))
        s.exact = int(bool(exact))
        self.s = s
        self.n = n

    def force_cells(self):
        """Exact-sum FP32 half-shell force: (F (n,3) f64, Fabs (n,3) f64, counts (n,), stats)."""
        F = np.zeros((self.n, 3)); A = np.zeros((self.n, 3)); cnt = np.zeros(self.n, np.int32)
        st = OrcStats()
        r = lib().orc_force_cells(C.byref(self.s), _p(F, _D), _p(A, _D), _p(cnt, _I), C.byref(st))
        assert r >= 0
        return F, A, cnt, st.as_dict()

    def force_direct64(self):
        F = np.zeros((self.n, 3)); st = OrcStats()
        assert lib().orc_force_direct64(C.byref(self.s), _p(F, _D), C.byref(st)) >= 0
        return F, st.as_dict()

    def force_tables64(self):
        F = np.zeros((self.n, 3)); st = OrcStats()
        assert lib().orc_force_tables64(C.byref(self.s), _p(F, _D), C.byref(st)) >= 0
        return F, st.as_dict()

    def force_split64(self, f32_diff: bool, tables: bool):
        """FP64 forces on the accepted pairs with the datapath's rounded differences or exact
        ones, and tables (evaluated in FP64) or direct powers: the error decomposition."""
        F = np.zeros((self.n, 3)); st = OrcStats()
        assert lib().orc_force_split64(C.byref(self.s), int(f32_diff), int(tables), _p(F, _D), C.byref(st)) >= 0
        return F, st.as_dict()

    def force_cells_fixed(self, hbegin=0, hend=-1):
        """Half-shell forces of the home cells [hbegin, hend) as int64 2^-24 fixed point, summed per
        pair ((n, 3) int64, pair count)."""
        F = np.zeros((self.n, 3), np.int64)
        pairs = lib().orc_force_cells_fixed(C.byref(self.s), hbegin, hend, F.ctypes.data_as(C.POINTER(C.c_int64)))
        assert pairs >= 0
        return F, int(pairs)

    def force_cells_mt(self, nthreads=0, hbegin=0, hend=-1):
        F = np.zeros((self.n, 3), np.float32)
        pairs = lib().orc_force_cells_mt(C.byref(self.s), nthreads, hbegin, hend, _p(F, _F))
        return F, pairs

    def force_allpairs_mt(self, nthreads=0):
        F = np.zeros((self.n, 3), np.float32)
        pairs = lib().orc_force_allpairs_mt(C.byref(self.s), nthreads, _p(F, _F))
        return F, pairs

    def force_allimage(self):
        """Every periodic image within rc (boxes with edge in (rc, 3 rc)): (F (n,3) FP64 table
        evaluation, F32sum (n,3) FP64 sum of the ordered pairs' FP32 forces, Fabs (n,3),
        counts (n,), stats)."""
        F = np.zeros((self.n, 3)); F32 = np.zeros((self.n, 3)); A = np.zeros((self.n, 3))
        cnt = np.zeros(self.n, np.int32); st = OrcStats()
        r = lib().orc_force_allimage(C.byref(self.s), _p(F, _D), _p(F32, _D), _p(A, _D), _p(cnt, _I),
                                     C.byref(st))
        assert r >= 0
        return F, F32, A, cnt, st.as_dict()

    def ewald64(self, beta, nmax, forces=True):
        """FP64 Ewald sum (see oracle.h): (F (n,3) or None, {'real', 'recip', 'self', 'background',
        'total'})."""
        F = np.zeros((self.n, 3)) if forces else None
        e = np.zeros(4)
        assert lib().orc_ewald64(C.byref(self.s), float(beta), int(nmax), _p(F, _D), _p(e, _D)) == 0
        return F, {"real": e[0], "recip": e[1], "self": e[2], "background": e[3], "total": float(e.sum())}

    def pair(self, xi, xj, qi=0.0, qj=0.0, ti=0, tj=0):
        out = np.zeros(8, np.float32)
        ok = lib().orc_pair_f32(C.byref(self.s), *[np.float32(v) for v in xi], np.float32(qi), int(ti),
                                *[np.float32(v) for v in xj], np.float32(qj), int(tj), _p(out, _F))
        return ok, out


def bin_cells(pos, box, ncell):
    pos = np.asarray(pos, np.float32)
    x, y, z = (np.ascontiguousarray(pos[:, k]) for k in range(3))
    n = len(x)
    b = np.asarray(box, np.float32)
    nc = np.asarray(ncell, np.int32)
    cell_of = np.zeros(n, np.int32)
    start = np.zeros(int(np.prod(nc)) + 1, np.int32)
    order = np.zeros(n, np.int32)
    mx = lib().orc_bin(n, _p(x, _F), _p(y, _F), _p(z, _F), _p(b, _F), _p(nc, _I), _p(cell_of, _I),
                       _p(start, _I), _p(order, _I))
    return cell_of, start, order, mx


def cmodel_run(pos, vel, iters, box=24.0, cutoff=8.0):
    pos = np.ascontiguousarray(pos, np.float32).copy()
    vel = np.ascontiguousarray(vel, np.float32).copy()
    n = len(pos)
    energy = np.zeros((max(iters, 1), 2), np.float32)
    cnt = np.zeros(n, np.int32)
    lib().orc_cmodel_run(n, iters, C.c_float(box), C.c_float(cutoff), _p(pos, _F), _p(vel, _F),
                         _p(energy, _F), _p(cnt, _I))
    return pos, vel, energy[:iters], cnt


def read_pdb_like_reference(path, n):
    """Positions as the reference C model reads them: skip 5 lines, then fields 7-9 via %f."""
    lines = Path(path).read_text().splitlines()[5:5 + n]
    return np.asarray([[np.float32(v) for v in l.split()[6:9]] for l in lines], np.float32)


def fit_tables(order, nseg, bins, min_log2, samples=8, local=False):
    """Independent numpy restatement of the table fit of
    MatlabScripts/LJ_no_smooth_poly_interpolation_function.m:182-378: per power-of-two segment and
    bin, a least-squares polynomial through `samples` points x_i = bin_start + i*width/samples of
    the unit functions x^-7, x^-4, x^-1.5, x^-6, x^-3, x^-0.5 (x = r2).  FP64 normal-equation fit
    in the bin-local variable, returned as FP32 monomial coefficients (6, order+1, nseg*bins), or
    with local=True as coefficients of u = r2 - bin start (the library's order-2/3 form)."""
    expo = np.array([-7.0, -4.0, -1.5, -6.0, -3.0, -0.5])
    seg = np.repeat(np.arange(nseg), bins)
    b = np.tile(np.arange(bins), nseg)
    lo = np.ldexp(1.0, min_log2 + seg)
    w = lo / bins
    x0 = lo + b * w
    t = np.arange(samples) / samples
    V = np.vander(t, order + 1, increasing=True)           # (samples, order+1)
    pinv = np.linalg.pinv(V)                                # least squares in t
    out = np.zeros((6, order + 1, nseg * bins), np.float32)
    from math import comb
    for f, e in enumerate(expo):
        y = (x0[:, None] + t[None, :] * w[:, None]) ** e     # (nidx, samples)
        a = y @ pinv.T                                       # (nidx, order+1) in t
        if local:
            out[f] = (a / w[:, None] ** np.arange(order + 1)[None, :]).T.astype(np.float32)
            continue
        c = np.zeros_like(a)
        for mm in range(order + 1):
            am = a[:, mm] / w ** mm
            for k in range(mm + 1):
                c[:, k] += am * comb(mm, k) * (-x0) ** (mm - k)
        out[f] = c.T.astype(np.float32)
    return out


def lb_coefficients(sigma, epsilon):
    """Lorentz-Berthelot per-type-pair multipliers (T*T, 4): A14, B8, A12, B6 (FP64)."""
    T = len(sigma)
    pc = np.zeros((T * T, 4))
    for a in range(T):
        for b in range(T):
            sig = 0.5 * (sigma[a] + sigma[b])
            eps = np.sqrt(epsilon[a] * epsilon[b])
            pc[a * T + b] = [48 * eps * sig ** 12, -24 * eps * sig ** 6, 4 * eps * sig ** 12, -4 * eps * sig ** 6]
    return pc


def bonded64(pos, box=None, bonds=None, angles=None, dihedrals=None):
    """FP64 bonded forces (n, 3) and energies {bond, angle, dihedral} (bonded.cpp).  Each term
    set is (atoms (m, 2|3|4) int, params (m, 2|4|3) float): bonds {k, r0}; angles {k_theta,
    theta0, k_ub, s0}; dihedrals {k, n, delta}.  box: periodic edges (None or 0: no wrap)."""
    pos = np.asarray(pos, np.float64)
    n = len(pos)
    x, y, z = (np.ascontiguousarray(pos[:, k]) for k in range(3))
    keep = []

    def arr(t, w_atoms, w_par):
        if t is None or len(t[0]) == 0:
            return 0, None, None
        a = np.ascontiguousarray(np.asarray(t[0], np.int32).reshape(-1, w_atoms))
        p = np.ascontiguousarray(np.asarray(t[1], np.float64).reshape(-1, w_par))
        assert len(a) == len(p)
        keep.extend((a, p))
        return len(a), _p(a, _I), _p(p, _D)

    b = OrcBonded()
    b.nb, b.bond_atoms, b.bond_par = arr(bonds, 2, 2)
    b.na, b.angle_atoms, b.angle_par = arr(angles, 3, 4)
    b.nd, b.dih_atoms, b.dih_par = arr(dihedrals, 4, 3)
    bx = np.zeros(3) if box is None else np.asarray(box, np.float64)
    F = np.zeros((n, 3))
    E = np.zeros(3)
    r = lib().orc_bonded64(n, _p(x, _D), _p(y, _D), _p(z, _D), _p(bx, _D), C.byref(b), _p(F, _D), _p(E, _D))
    if r != 0:
        raise ValueError(f"orc_bonded64: bad arguments ({r})")
    return F, {"bond": E[0], "angle": E[1], "dihedral": E[2]}
