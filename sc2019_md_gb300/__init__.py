"""sc2019_md_gb300 — Python mirror of libmdrl's C ABI (include/mdrl.h).

libmdrl is a GB300 (sm_103a) implementation of the SC2019-MD range-limited force path: cell
binning, half-shell pairs, the 0 < r2 <= rc2 filter, tabulated LJ r^-14 / r^-8 plus Coulomb r^-3,
Newton's-third-law accumulation in int64 fixed point and the motion update.  This module only
marshals numpy arrays through ctypes; every computation runs in the CUDA library, and importing
it fails loudly when the library has not been built (``python -m sc2019_md_gb300.build``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

__all__ = [
    "Params", "Stats", "Context", "MdrlError", "lib", "library_path", "fit_tables", "halfshell_offsets",
    "cmodel_run", "md_evaluation_model", "Batch", "Replica", "Tile", "TUNE_RETIME", "PmeParams", "PATH_HALF_SHELL", "PATH_MIN_IMAGE",
    "PATH_ALL_IMAGES", "ACC_FIXED64", "ACC_FP32_ATOMIC", "ACC_KAHAN",
    "ARITH_FMA", "ARITH_SEPARATE", "EVAL_TABLE", "EVAL_DIRECT", "INT_VELOCITY_VERLET",
    "Slab", "slab_plan", "slab_select", "INT_EULER", "FLAG_ENERGY", "FLAG_PAIR_COUNTS", "FLAG_NO_PBC", "FLAG_EXACT_DIFF", "TABLE_RAW",
    "TABLE_BIN_LOCAL", "MAX_TYPES", "STATUS",
]

MAX_TYPES = 16
ACC_FIXED64, ACC_FP32_ATOMIC, ACC_KAHAN = 0, 1, 2
ARITH_FMA, ARITH_SEPARATE = 0, 1
EVAL_TABLE, EVAL_DIRECT = 0, 1
INT_VELOCITY_VERLET, INT_EULER = 0, 1
FLAG_ENERGY, FLAG_PAIR_COUNTS, FLAG_NO_PBC, FLAG_EXACT_DIFF = 0x1, 0x2, 0x4, 0x8
TABLE_RAW, TABLE_BIN_LOCAL = 0x1, 0x2
STATUS = {0: "OK", 1: "INVALID_ARG", 2: "CELL_OVERFLOW", 3: "RANGE", 4: "CUDA_ERROR",
          5: "TIMEOUT", 6: "STATE"}

_HERE = Path(__file__).resolve().parent


def library_path() -> Path:
    """The in-tree libmdrl.so, or the file named by MDRL_LIBRARY (a build variant)."""
    import os
    env = os.environ.get("MDRL_LIBRARY")
    return Path(env) if env else _HERE / "_build" / "libmdrl.so"


class MdrlError(RuntimeError):
    """A libmdrl call returned a status other than MDRL_OK."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}")


class Params(C.Structure):
    _fields_ = [
        ("box", C.c_double * 3), ("cutoff", C.c_double), ("ncell", C.c_int * 3),
        ("ntypes", C.c_int), ("sigma", C.c_double * MAX_TYPES),
        ("epsilon", C.c_double * MAX_TYPES), ("mass", C.c_double * MAX_TYPES),
        ("coulomb_k", C.c_double), ("table_order", C.c_int), ("table_bins", C.c_int),
        ("table_min_log2", C.c_int), ("eval", C.c_int), ("arith", C.c_int), ("accum", C.c_int),
        ("integrator", C.c_int), ("dt_fs", C.c_double), ("flags", C.c_uint32), ("device", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("pairs", C.c_int64), ("candidates", C.c_int64), ("below_table", C.c_int64),
        ("max_cell_occupancy", C.c_int), ("ncells", C.c_int), ("e_lj", C.c_double),
        ("e_coul", C.c_double), ("virial", C.c_double), ("kinetic", C.c_double),
        ("device_ms", C.c_double), ("pairs_total", C.c_int64), ("force_ms", C.c_double),
        ("e_bond", C.c_double), ("e_angle", C.c_double), ("e_dihedral", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int)
_D = C.POINTER(C.c_double)
_lib = None


class PmeParams(C.Structure):
    _fields_ = [("beta", C.c_double), ("tolerance", C.c_double), ("spacing", C.c_double),
                ("grid", C.c_int * 3), ("order", C.c_int)]

    def as_dict(self):
        return {"beta": self.beta, "tolerance": self.tolerance, "spacing": self.spacing,
                "grid": tuple(self.grid), "order": self.order}


class Tile(C.Structure):
    _fields_ = [("warps_per_cta", C.c_int), ("steps_per_piece", C.c_int), ("prune_steps", C.c_int)]

    def as_tuple(self):
        return (self.warps_per_cta, self.steps_per_piece, self.prune_steps)


TUNE_RETIME = 1


class Replica(C.Structure):
    _fields_ = [("n", C.c_int), ("box", C.c_double * 3)]


PATH_HALF_SHELL, PATH_MIN_IMAGE, PATH_ALL_IMAGES = 0, 1, 2


class Slab(C.Structure):
    _fields_ = [("nranks", C.c_int), ("rank", C.c_int), ("x0", C.c_int), ("x1", C.c_int), ("halo_x", C.c_int),
                ("import_from", C.c_int), ("export_to", C.c_int), ("ncell", C.c_int * 3)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "ncell"}
        d["ncell"] = tuple(self.ncell)
        return d


def slab_plan(params: "Params", nranks: int, rank: int) -> Slab:
    """The slab of cell layers along x that `rank` owns (mdrl_slab_plan; host only)."""
    s = Slab()
    _check(lib().mdrl_slab_plan(C.byref(params), nranks, rank, C.byref(s)))
    return s


def slab_select(params: "Params", slab: Slab, x) -> tuple:
    """(owned indices, exported indices) of the particles with x coordinates `x` (host only)."""
    x = _f32(x)
    n = x.shape[0]
    owned, exported = np.zeros(n, np.int32), np.zeros(n, np.int32)
    no, ne = C.c_int(), C.c_int()
    _check(lib().mdrl_slab_select(C.byref(params), C.byref(slab), n, _fp(x), _ip(owned), C.byref(no),
                                  _ip(exported), C.byref(ne)))
    return owned[:no.value], exported[:ne.value]


def lib() -> C.CDLL:
    """The loaded libmdrl (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise ImportError(f"libmdrl is not built ({path}); run python -m sc2019_md_gb300.build")
    L = C.CDLL(str(path))
    st = C.c_int
    vp = C.c_void_p
    L.mdrl_version.restype = C.c_char_p
    L.mdrl_last_error.restype = C.c_char_p
    L.mdrl_default_params.argtypes = [C.POINTER(Params)]
    L.mdrl_default_params.restype = None
    L.mdrl_fit_tables.argtypes = [st, st, st, st, st, _F]
    L.mdrl_fit_tables_bin_local.argtypes = [st, st, st, st, st, _F]
    L.mdrl_get_table_form.argtypes = [vp, _I]
    L.mdrl_slab_plan.argtypes = [C.POINTER(Params), st, st, C.POINTER(Slab)]
    L.mdrl_slab_select.argtypes = [C.POINTER(Params), C.POINTER(Slab), st, _F, _I, _I, _I, _I]
    L.mdrl_force_eval_fixed.argtypes = [vp, st, _F, _F, _F, _F, _I, st, st, C.POINTER(C.c_int64), C.POINTER(Stats)]
    L.mdrl_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    L.mdrl_destroy.argtypes = [vp]
    L.mdrl_set_tables.argtypes = [vp, st, st, st, st, st, _F, st]
    L.mdrl_get_tables.argtypes = [vp, _I, _I, _I, _I, _F]
    L.mdrl_get_pair_coefficients.argtypes = [vp, _F]
    L.mdrl_bin.argtypes = [vp, st, _F, _F, _F, _I, _I, _I]
    L.mdrl_force_eval.argtypes = [vp, st, _F, _F, _F, _F, _I, _F, _F, _F, _I, C.POINTER(Stats)]
    L.mdrl_force_eval_device.argtypes = [vp, st, vp, vp, vp, vp, vp, vp, vp, vp, vp, C.POINTER(Stats)]
    L.mdrl_pair_eval.argtypes = [vp, st, _F, _F, _I, _I, _F, _F]
    L.mdrl_set_state.argtypes = [vp, st, _F, _F, _F, _F, _F, _F, _F, _I]
    L.mdrl_step.argtypes = [vp, st, C.POINTER(Stats)]
    L.mdrl_get_state.argtypes = [vp, _F, _F, _F, _F, _F, _F, _F, _F, _F]
    L.mdrl_time_force.argtypes = [vp, _F]
    L.mdrl_force_eval_static.argtypes = [C.POINTER(Params), st, vp, vp, vp, vp, vp, vp, vp, vp,
                                         C.POINTER(C.c_int64), vp]
    L.MD_Evaluation_Model.argtypes = []
    L.MD_Evaluation_Model.restype = C.c_int
    L.mdrl_cmodel_run.argtypes = [st, st, C.c_float, C.c_float, _F, _F, _F, _I]
    L.mdrl_batch_create.argtypes = [C.POINTER(Params), st, C.POINTER(Replica), C.POINTER(vp)]
    L.mdrl_batch_destroy.argtypes = [vp]
    L.mdrl_batch_layout.argtypes = [vp, _I, _I, _I, _I]
    L.mdrl_batch_force_eval.argtypes = [vp, _F, _F, _F, _F, _I, _F, _F, _F, _I, C.POINTER(Stats)]
    L.mdrl_batch_set_state.argtypes = [vp, _F, _F, _F, _F, _F, _F, _F, _I]
    L.mdrl_batch_step.argtypes = [vp, st, C.POINTER(Stats)]
    L.mdrl_batch_get_state.argtypes = [vp, _F, _F, _F, _F, _F, _F, _F, _F, _F]
    L.mdrl_batch_replica_stats.argtypes = [vp, C.POINTER(Stats)]
    L.mdrl_batch_time_force.argtypes = [vp, _F]
    L.mdrl_halfshell_offsets.argtypes = [_I]
    L.mdrl_halfshell_offsets.restype = None
    L.mdrl_default_pme_params.argtypes = [C.POINTER(PmeParams)]
    L.mdrl_default_pme_params.restype = None
    L.mdrl_set_pme.argtypes = [vp, C.POINTER(PmeParams)]
    L.mdrl_get_pme.argtypes = [vp, C.POINTER(PmeParams), _I]
    L.mdrl_set_pair_coefficients.argtypes = [vp, _D]
    L.mdrl_batch_set_pair_coefficients.argtypes = [vp, _D]
    L.mdrl_set_tile.argtypes = [vp, C.POINTER(Tile)]
    L.mdrl_get_tile.argtypes = [vp, C.POINTER(Tile)]
    L.mdrl_autotune.argtypes = [vp, st, C.POINTER(Tile), _F, _F]
    L.mdrl_batch_set_tile.argtypes = [vp, C.POINTER(Tile)]
    L.mdrl_batch_autotune.argtypes = [vp, st, C.POINTER(Tile), _F, _F]
    for name in ("mdrl_set_pme", "mdrl_get_pme", "mdrl_set_pair_coefficients", "mdrl_batch_set_pair_coefficients", "mdrl_set_tile", "mdrl_get_tile", "mdrl_autotune", "mdrl_batch_set_tile", "mdrl_batch_autotune",
                 "mdrl_batch_create", "mdrl_batch_destroy", "mdrl_batch_layout", "mdrl_batch_force_eval",
                 "mdrl_batch_set_state", "mdrl_batch_step", "mdrl_batch_get_state",
                 "mdrl_batch_replica_stats", "mdrl_batch_time_force"):
        getattr(L, name).restype = st
    for name in ("mdrl_fit_tables", "mdrl_fit_tables_bin_local", "mdrl_get_table_form", "mdrl_slab_plan",
                 "mdrl_slab_select", "mdrl_force_eval_fixed", "mdrl_create", "mdrl_destroy", "mdrl_set_tables",
                 "mdrl_get_tables", "mdrl_get_pair_coefficients", "mdrl_bin", "mdrl_force_eval",
                 "mdrl_force_eval_device", "mdrl_pair_eval", "mdrl_set_state", "mdrl_step",
                 "mdrl_get_state", "mdrl_cmodel_run", "mdrl_time_force", "mdrl_force_eval_static"):
        getattr(L, name).restype = st
    _lib = L
    return L


def _check(status: int) -> None:
    if status != 0:
        raise MdrlError(status, lib().mdrl_last_error().decode())


def _fp(a):
    return None if a is None else a.ctypes.data_as(_F)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_I)


def _f32(a, n=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float32)
    if n is not None and a.shape[0] != n:
        raise ValueError("array length mismatch")
    return a


def _i32(a, n=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.int32)
    if n is not None and a.shape[0] != n:
        raise ValueError("array length mismatch")
    return a


def default_params(**kw) -> Params:
    """Params filled by mdrl_default_params, then overridden by keyword (sequences for the
    per-type arrays and the box)."""
    p = Params()
    lib().mdrl_default_params(C.byref(p))
    for k, v in kw.items():
        if k in ("box", "ncell", "sigma", "epsilon", "mass"):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, k, v)
    return p


def halfshell_offsets() -> np.ndarray:
    """The 14 (dx, dy, dz) cell offsets of the half-shell traversal, home cell first (host only)."""
    out = np.zeros((14, 3), dtype=np.int32)
    lib().mdrl_halfshell_offsets(_ip(out))
    return out


def fit_tables(order: int, nseg: int, bins: int, min_log2: int, samples: int = 8,
               local: bool = False) -> np.ndarray:
    """FP64-fitted unit tables, shape (6, order+1, nseg*bins) (host only, no GPU): monomial in r2,
    or with local=True coefficients of u = r2 - bin start (orders 2-3)."""
    out = np.zeros((6, order + 1, nseg * bins), dtype=np.float32)
    fn = lib().mdrl_fit_tables_bin_local if local else lib().mdrl_fit_tables
    _check(fn(order, nseg, bins, min_log2, samples, _fp(out)))
    return out


class Context:
    """One libmdrl context (a CUDA stream, device buffers and tables)."""

    def __init__(self, params: Params | None = None, **kw):
        self.params = params if params is not None else default_params(**kw)
        self._h = C.c_void_p()
        _check(lib().mdrl_create(C.byref(self.params), C.byref(self._h)))

    def close(self) -> None:
        if self._h:
            lib().mdrl_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # tables ------------------------------------------------------------------------------
    def tables(self) -> tuple[np.ndarray, dict]:
        o, s, b, m = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        _check(lib().mdrl_get_tables(self._h, C.byref(o), C.byref(s), C.byref(b), C.byref(m), None))
        out = np.zeros((6, o.value + 1, s.value * b.value), dtype=np.float32)
        _check(lib().mdrl_get_tables(self._h, None, None, None, None, _fp(out)))
        form = C.c_int()
        _check(lib().mdrl_get_table_form(self._h, C.byref(form)))
        return out, {"order": o.value, "nseg": s.value, "bins": b.value, "min_log2": m.value,
                     "raw": bool(form.value & TABLE_RAW), "local": bool(form.value & TABLE_BIN_LOCAL)}

    def set_tables(self, coef: np.ndarray, order: int, nseg: int, bins: int, min_log2: int,
                   raw: bool = False, local: bool = False) -> None:
        coef = np.ascontiguousarray(coef, dtype=np.float32)
        nfunc = coef.shape[0]
        flags = (TABLE_RAW if raw else 0) | (TABLE_BIN_LOCAL if local else 0)
        _check(lib().mdrl_set_tables(self._h, order, nseg, bins, min_log2, nfunc, _fp(coef), flags))

    def set_pme(self, enable: bool = True, **kw) -> dict:
        """Switch smooth-PME long-range electrostatics on (keywords: beta, tolerance, spacing,
        grid, order) or off; returns the resolved parameters (or {} when off)."""
        if not enable:
            _check(lib().mdrl_set_pme(self._h, None))
            return {}
        p = PmeParams()
        lib().mdrl_default_pme_params(C.byref(p))
        for k, v in kw.items():
            if k == "grid":
                for d in range(3):
                    p.grid[d] = int(v[d])
            else:
                setattr(p, k, v)
        _check(lib().mdrl_set_pme(self._h, C.byref(p)))
        return self.pme()

    def pme(self) -> dict:
        p, on = PmeParams(), C.c_int()
        _check(lib().mdrl_get_pme(self._h, C.byref(p), C.byref(on)))
        return p.as_dict() if on.value else {}

    def set_pair_coefficients(self, coef) -> None:
        """Per-type-pair multipliers (ntypes*ntypes, 4): A14, B8, A12, B6 (FP64)."""
        c = np.ascontiguousarray(coef, dtype=np.float64).reshape(-1)
        if c.size != self.params.ntypes ** 2 * 4:
            raise ValueError("coef must hold ntypes*ntypes*4 values")
        _check(lib().mdrl_set_pair_coefficients(self._h, c.ctypes.data_as(_D)))

    def set_bonded(self, bonds=None, angles=None, dihedrals=None) -> None:
        """Bonded terms (mdrl_set_bonded).  Each set is (atoms, params): bonds ((m, 2), (m, 2)
        {k, r0}); angles ((m, 3), (m, 4) {k_theta, theta0, k_ub, s0}, the middle atom the vertex);
        dihedrals ((m, 4), (m, 3) {k, n, delta}).  None everywhere removes the terms."""
        keep = []

        def arr(t, wa, wp):
            if t is None or len(t[0]) == 0:
                return 0, None, None
            a = np.ascontiguousarray(np.asarray(t[0], dtype=np.int32).reshape(-1, wa))
            p = np.ascontiguousarray(np.asarray(t[1], dtype=np.float64).reshape(-1, wp))
            if len(a) != len(p):
                raise ValueError("atoms and params differ in length")
            keep.extend((a, p))
            return len(a), _ip(a), p.ctypes.data_as(_D)

        nb, ba, bp = arr(bonds, 2, 2)
        na, aa, ap = arr(angles, 3, 4)
        nd, da, dp = arr(dihedrals, 4, 3)
        _check(lib().mdrl_set_bonded(self._h, nb, ba, bp, na, aa, ap, nd, da, dp))

    def time_bonded(self) -> float:
        """Device time (ms) of one launch of the bonded-term kernels on the current state."""
        ms = C.c_float()
        _check(lib().mdrl_time_bonded(self._h, C.byref(ms)))
        return ms.value

    def bonded_counts(self) -> tuple:
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _check(lib().mdrl_get_bonded_counts(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def pair_coefficients(self) -> np.ndarray:
        T = self.params.ntypes
        out = np.zeros((T * T, 4), dtype=np.float32)
        _check(lib().mdrl_get_pair_coefficients(self._h, _fp(out)))
        return out

    # evaluation --------------------------------------------------------------------------
    def bin(self, x, y, z):
        x, y, z = _f32(x), _f32(y), _f32(z)
        n = x.shape[0]
        nc = self.params.ncell
        cell_of = np.zeros(n, np.int32)
        order = np.zeros(n, np.int32)
        ncells = self._ncells()
        count = np.zeros(ncells, np.int32)
        _check(lib().mdrl_bin(self._h, n, _fp(x), _fp(y), _fp(z), _ip(cell_of), _ip(count), _ip(order)))
        return cell_of, count, order

    def _ncells(self) -> int:
        p = self.params
        tot = 1
        for d in range(3):
            nc = p.ncell[d] if p.ncell[d] > 0 else int(np.floor(np.float64(np.float32(p.box[d])) /
                                                               np.float64(np.float32(p.cutoff))))
            tot *= nc
        return tot

    def force(self, x, y, z, q=None, type=None, counts: bool = False):
        """One force evaluation; returns (F (n,3) float32, stats dict, counts or None)."""
        x = _f32(x)
        n = x.shape[0]
        y, z, q, t = _f32(y, n), _f32(z, n), _f32(q, n), _i32(type, n)
        fx, fy, fz = (np.zeros(n, np.float32) for _ in range(3))
        cnt = np.zeros(n, np.int32) if counts else None
        st = Stats()
        _check(lib().mdrl_force_eval(self._h, n, _fp(x), _fp(y), _fp(z), _fp(q), _ip(t), _fp(fx),
                                     _fp(fy), _fp(fz), _ip(cnt), C.byref(st)))
        return np.stack([fx, fy, fz], axis=1), st.as_dict(), cnt

    def force_fixed(self, x, y, z, q=None, type=None, home=None):
        """Forces of the units whose home cell layer lies in home = (x0, x1) (None: all) as raw int64
        2^-24 fixed point (mdrl_force_eval_fixed); returns ((n,3) int64, stats dict)."""
        x = _f32(x)
        n = x.shape[0]
        y, z, q, t = _f32(y, n), _f32(z, n), _f32(q, n), _i32(type, n)
        F = np.zeros((3, n), np.int64)
        h0, h1 = home if home is not None else (0, self._ncell_x())
        st = Stats()
        _check(lib().mdrl_force_eval_fixed(self._h, n, _fp(x), _fp(y), _fp(z), _fp(q), _ip(t), h0, h1,
                                           F.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(st)))
        return np.ascontiguousarray(F.T), st.as_dict()

    def _ncell_x(self) -> int:
        p = self.params
        return p.ncell[0] if p.ncell[0] > 0 else int(np.floor(np.float64(np.float32(p.box[0])) /
                                                              np.float64(np.float32(p.cutoff))))

    def pair_eval(self, ref, nbr, type_ref=None, type_nbr=None):
        """Per-pair plugin: ref/nbr (n,4) float32 (x,y,z,q); returns (out (n,4), aux (n,2))."""
        ref = np.ascontiguousarray(ref, dtype=np.float32)
        nbr = np.ascontiguousarray(nbr, dtype=np.float32)
        n = ref.shape[0]
        out = np.zeros((n, 4), np.float32)
        aux = np.zeros((n, 2), np.float32)
        _check(lib().mdrl_pair_eval(self._h, n, _fp(ref), _fp(nbr), _ip(_i32(type_ref, n)),
                                    _ip(_i32(type_nbr, n)), _fp(out), _fp(aux)))
        return out, aux

    # molecular dynamics ------------------------------------------------------------------
    def set_state(self, x, y, z, v=None, q=None, type=None) -> None:
        x = _f32(x)
        n = x.shape[0]
        y, z = _f32(y, n), _f32(z, n)
        self._n = n
        vx = vy = vz = None
        if v is not None:
            v = np.asarray(v, dtype=np.float32)
            vx, vy, vz = (np.ascontiguousarray(v[:, k]) for k in range(3))
        self._keep = (x, y, z, vx, vy, vz, _f32(q, n), _i32(type, n))
        k = self._keep
        _check(lib().mdrl_set_state(self._h, n, _fp(k[0]), _fp(k[1]), _fp(k[2]), _fp(k[3]),
                                    _fp(k[4]), _fp(k[5]), _fp(k[6]), _ip(k[7])))

    def step(self, nsteps: int = 1) -> dict:
        st = Stats()
        _check(lib().mdrl_step(self._h, nsteps, C.byref(st)))
        return st.as_dict()

    def time_force(self) -> float:
        """Device time (ms) of one launch of the force kernel on the current state."""
        ms = C.c_float()
        _check(lib().mdrl_time_force(self._h, C.byref(ms)))
        return ms.value

    def set_tile(self, warps_per_cta: int, steps_per_piece: int, prune_steps: int = 0) -> None:
        t = Tile(warps_per_cta, steps_per_piece, prune_steps)
        _check(lib().mdrl_set_tile(self._h, C.byref(t)))

    def tile(self) -> tuple:
        t = Tile()
        _check(lib().mdrl_get_tile(self._h, C.byref(t)))
        return t.as_tuple()

    def autotune(self, retime: bool = False) -> dict:
        """Time every candidate tile on the current state and keep the fastest."""
        t, b, d = Tile(), C.c_float(), C.c_float()
        _check(lib().mdrl_autotune(self._h, TUNE_RETIME if retime else 0, C.byref(t), C.byref(b), C.byref(d)))
        return {"tile": t.as_tuple(), "ms": b.value, "default_ms": d.value}

    def state(self):
        n = self._n
        a = [np.zeros(n, np.float32) for _ in range(9)]
        _check(lib().mdrl_get_state(self._h, *[_fp(v) for v in a]))
        return (np.stack(a[0:3], 1), np.stack(a[3:6], 1), np.stack(a[6:9], 1))


class Batch:
    """Independent periodic replicas sharing one force field (mdrl_batch_*).  `replicas` is a
    sequence of (n, (Lx, Ly, Lz)); arrays are the replicas' particles concatenated in order."""

    def __init__(self, params: Params, replicas):
        self.params = params
        reps = (Replica * len(replicas))()
        for k, (n, box) in enumerate(replicas):
            reps[k].n = int(n)
            for d in range(3):
                reps[k].box[d] = float(box[d])
        self.nrep = len(replicas)
        self.sizes = np.array([int(n) for n, _ in replicas], np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)])
        self.n = int(self.offsets[-1])
        self._h = C.c_void_p()
        _check(lib().mdrl_batch_create(C.byref(params), self.nrep, reps, C.byref(self._h)))

    def close(self) -> None:
        if self._h:
            lib().mdrl_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def layout(self) -> dict:
        path = np.zeros(self.nrep, np.int32)
        ncell = np.zeros((self.nrep, 3), np.int32)
        items = np.zeros(self.nrep, np.int32)
        tot = C.c_int()
        _check(lib().mdrl_batch_layout(self._h, _ip(path), _ip(ncell), _ip(items), C.byref(tot)))
        return {"path": path, "ncell": ncell, "items": items, "total_items": tot.value}

    def force(self, x, y, z, q=None, type=None, counts: bool = False):
        n = self.n
        x, y, z, q, t = _f32(x, n), _f32(y, n), _f32(z, n), _f32(q, n), _i32(type, n)
        fx, fy, fz = (np.zeros(n, np.float32) for _ in range(3))
        cnt = np.zeros(n, np.int32) if counts else None
        st = Stats()
        _check(lib().mdrl_batch_force_eval(self._h, _fp(x), _fp(y), _fp(z), _fp(q), _ip(t), _fp(fx), _fp(fy),
                                           _fp(fz), _ip(cnt), C.byref(st)))
        return np.stack([fx, fy, fz], axis=1), st.as_dict(), cnt

    def set_state(self, x, y, z, v=None, q=None, type=None) -> None:
        n = self.n
        vx = vy = vz = None
        if v is not None:
            v = np.asarray(v, dtype=np.float32)
            vx, vy, vz = (np.ascontiguousarray(v[:, k]) for k in range(3))
        self._keep = (_f32(x, n), _f32(y, n), _f32(z, n), vx, vy, vz, _f32(q, n), _i32(type, n))
        k = self._keep
        _check(lib().mdrl_batch_set_state(self._h, _fp(k[0]), _fp(k[1]), _fp(k[2]), _fp(k[3]), _fp(k[4]),
                                          _fp(k[5]), _fp(k[6]), _ip(k[7])))

    def step(self, nsteps: int = 1) -> dict:
        st = Stats()
        _check(lib().mdrl_batch_step(self._h, nsteps, C.byref(st)))
        return st.as_dict()

    def state(self):
        a = [np.zeros(self.n, np.float32) for _ in range(9)]
        _check(lib().mdrl_batch_get_state(self._h, *[_fp(v) for v in a]))
        return (np.stack(a[0:3], 1), np.stack(a[3:6], 1), np.stack(a[6:9], 1))

    def replica_stats(self) -> list:
        out = (Stats * self.nrep)()
        _check(lib().mdrl_batch_replica_stats(self._h, out))
        return [out[k].as_dict() for k in range(self.nrep)]

    def time_force(self) -> float:
        ms = C.c_float()
        _check(lib().mdrl_batch_time_force(self._h, C.byref(ms)))
        return ms.value

    def set_tile(self, warps_per_cta: int, steps_per_piece: int, prune_steps: int = 0) -> None:
        t = Tile(warps_per_cta, steps_per_piece, prune_steps)
        _check(lib().mdrl_batch_set_tile(self._h, C.byref(t)))

    def set_pair_coefficients(self, coef) -> None:
        c = np.ascontiguousarray(coef, dtype=np.float64).reshape(-1)
        if c.size != self.params.ntypes ** 2 * 4:
            raise ValueError("coef must hold ntypes*ntypes*4 values")
        _check(lib().mdrl_batch_set_pair_coefficients(self._h, c.ctypes.data_as(_D)))

    def autotune(self, retime: bool = False) -> dict:
        t, b, d = Tile(), C.c_float(), C.c_float()
        _check(lib().mdrl_batch_autotune(self._h, TUNE_RETIME if retime else 0, C.byref(t), C.byref(b), C.byref(d)))
        return {"tile": t.as_tuple(), "ms": b.value, "default_ms": d.value}


def force_eval_static(params: Params, n: int, x, y, z, q, type, fx, fy, fz, stream=None) -> int:
    """mdrl_force_eval_static: a force evaluation that allocates no device memory.  Every array
    argument is a device address (an int, e.g. a torch tensor's data_ptr(), or None for q/type);
    returns the number of pairs."""
    pairs = C.c_int64()
    _check(lib().mdrl_force_eval_static(C.byref(params), n, x, y, z, q, type, fx, fy, fz,
                                        C.byref(pairs), stream))
    return pairs.value


def cmodel_run(pos: np.ndarray, vel: np.ndarray, iters: int, box: float = 24.0,
               cutoff: float = 8.0, counts: bool = False):
    """The reference C model's run on the GPU (mdrl_cmodel_run); returns (pos, vel, energy
    (iters,2), counts or None)."""
    pos = np.ascontiguousarray(pos, dtype=np.float32).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float32).copy()
    n = pos.shape[0]
    energy = np.zeros((max(iters, 1), 2), np.float32)
    cnt = np.zeros(n, np.int32) if counts else None
    _check(lib().mdrl_cmodel_run(n, iters, C.c_float(box), C.c_float(cutoff), _fp(pos), _fp(vel),
                                 _fp(energy), _ip(cnt)))
    return pos, vel, energy[:iters], cnt


def md_evaluation_model() -> int:
    """Call the drop-in int MD_Evaluation_Model() (reads MDRL_INPUT, prints to stdout)."""
    return lib().MD_Evaluation_Model()
