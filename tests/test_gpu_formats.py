"""Formats through the GPU path.

* The GPU binning (mdrl_bin, the reference's in-cell input order) of the 20k LJArgon positions,
  written with write_cell_mif / write_cell_hex, reproduces the reference's 64 RTL cell images
  byte for byte (SHA-256 fixture).
* Per-type-pair multipliers from Amber-style A/B (16 types, mdrl_set_pair_coefficients): pair
  lists and forces at parity with the oracle given the same multipliers, during MD too.
"""
import hashlib
import json

import numpy as np
import pytest

import oracle
import sc2019_md_gb300 as m
from sc2019_md_gb300 import formats as F
from sc2019_md_gb300 import systems
from helpers import GOLDEN, kat2_positions

pytestmark = pytest.mark.gpu

SUM_TOL = 2e-6
FIX_ABS = 64 * 2.0 ** -24


def test_gpu_binning_writes_reference_cell_images():
    pos, _ = kat2_positions()
    p = m.default_params(box=(7 * 8.5, 6 * 8.5, 6 * 8.5), cutoff=8.5, ncell=(7, 6, 6))
    with m.Context(p) as ctx:
        cell_of, count, order = ctx.bin(pos[:, 0], pos[:, 1], pos[:, 2])
    start = np.concatenate([[0], np.cumsum(count)])
    expect = json.loads((GOLDEN / "cell_images_20k.json").read_text())
    for key, e in expect.items():
        x, y, z = (int(v) for v in key.split("_"))
        c = ((x - 1) * 6 + (y - 1)) * 6 + (z - 1)
        cell = pos[order[start[c]:start[c + 1]]]
        assert len(cell) == e["count"], key
        assert hashlib.sha256(F.write_cell_mif(None, cell).encode()).hexdigest() == e["mif"], key
        assert hashlib.sha256(F.write_cell_hex(None, cell).encode()).hexdigest() == e["hex"], key


def _amber_like(T=16, seed=7):
    """Symmetric Amber-style A, B for T types (sigma 2.4-3.8 A, eps 0.02-0.25, geometric-style
    mixing with per-pair jitter, so the matrix is not Lorentz-Berthelot)."""
    rng = np.random.default_rng(seed)
    sig = rng.uniform(2.4, 3.8, T)
    eps = rng.uniform(0.02, 0.25, T)
    s = np.sqrt(np.outer(sig, sig)) * (1 + 0.05 * rng.uniform(-1, 1, (T, T)))
    e = np.sqrt(np.outer(eps, eps)) * (1 + 0.2 * rng.uniform(-1, 1, (T, T)))
    s, e = 0.5 * (s + s.T), 0.5 * (e + e.T)
    return 4 * e * s ** 12, 4 * e * s ** 6


def test_pair_coefficient_override_parity():
    T = 16
    A, B = _amber_like(T)
    coef = F.pair_coefficients_from_AB(A, B)
    s0 = systems.small_ljc(4000, 40.0, 10.0, seed=13)
    rng = np.random.default_rng(3)
    types = rng.integers(0, T, s0.n).astype(np.int32)
    p = m.default_params(box=s0.box, cutoff=10.0, ntypes=T, sigma=[3.0] * T, epsilon=[0.1] * T, mass=[20.0] * T,
                         coulomb_k=systems.COULOMB_K, table_bins=512, flags=m.FLAG_ENERGY)
    x, y, z = (np.ascontiguousarray(s0.pos[:, k]) for k in range(3))
    with m.Context(p) as ctx:
        ctx.set_pair_coefficients(coef)
        pc32 = ctx.pair_coefficients()
        assert np.array_equal(pc32, coef.astype(np.float32))
        F1, st, cnt = ctx.force(x, y, z, s0.q, types, counts=True)
        tab, meta = ctx.tables()
        ctx.set_state(x, y, z, s0.vel, s0.q, types)       # MD with the override (graph captured after)
        ctx.step(3)
    o = oracle.System(s0.pos, s0.box, s0.ncell, 10.0, pc32, q=s0.q, type=types, ke=systems.COULOMB_K, tab=tab,
                      order=1, nseg=meta["nseg"], bins=meta["bins"], min_log2=meta["min_log2"], eval=0, arith=0,
                      pcoef64=coef, ke64=systems.COULOMB_K)
    Fo, Fabs, cnto, sto = o.force_cells()
    assert np.array_equal(cnt, cnto)
    assert st["pairs"] == sto["pairs"]
    err = np.abs(F1 - Fo) / (SUM_TOL * Fabs + FIX_ABS)
    assert err.max() <= 1.0, err.max()
    assert abs(st["e_lj"] - sto["e_lj"]) <= 1e-5 * abs(sto["e_lj"])
    with m.Context(p) as ctx:
        with pytest.raises(m.MdrlError):
            ctx.set_pair_coefficients(np.full(T * T * 4, np.nan))


def test_gpu_binning_reproduces_reference_pair_stream():
    """The RTL pair generator's stream for home cell (2,2,2), rebuilt from the GPU binning
    (mdrl_bin) and the library's half-shell offsets, equals the reference's."""
    from helpers import pair_stream_canon_from_cells
    pos, _ = kat2_positions()
    p = m.default_params(box=(7 * 8.5, 6 * 8.5, 6 * 8.5), cutoff=8.5, ncell=(7, 6, 6))
    with m.Context(p) as ctx:
        cell_of, count, order = ctx.bin(pos[:, 0], pos[:, 1], pos[:, 2])
    start = np.concatenate([[0], np.cumsum(count)])

    def cell_list(cx, cy, cz):
        c = ((cx - 1) * 6 + (cy - 1)) * 6 + (cz - 1)
        return order[start[c]:start[c + 1]]

    canon = pair_stream_canon_from_cells(pos, cell_list, (2, 2, 2), m.halfshell_offsets())
    expect = json.loads((GOLDEN / "pair_stream_222.json").read_text())
    assert hashlib.sha256("\n".join(canon).encode()).hexdigest() == expect["sha256"]


@pytest.mark.parametrize("mode", ["direct", "tables"])
def test_gpu_energy_matches_reference_golden_model_20k(mode):
    """The GPU path's LJ energy of the 20k LJArgon positions against the step-1 potential energy of
    the reference's double-precision golden model: within 2e-6 with direct FP32 evaluation, 2e-5
    with second-order 1024-bin tables."""
    pos, _ = kat2_positions()
    e = json.loads((GOLDEN / "energy_20k.json").read_text())
    p = m.default_params(box=(7 * 8.5, 6 * 8.5, 6 * 8.5), cutoff=8.5, ncell=(7, 6, 6), sigma=[2.1],
                         epsilon=[1.995996 ** 2], table_bins=1024, table_order=2, flags=m.FLAG_ENERGY,
                         eval=m.EVAL_DIRECT if mode == "direct" else m.EVAL_TABLE)
    with m.Context(p) as ctx:
        _, st, _ = ctx.force(pos[:, 0], pos[:, 1], pos[:, 2])
    ref = e["Double"]["potential"]
    tol = 2e-6 if mode == "direct" else 2e-5
    assert abs(st["e_lj"] - ref) <= tol * abs(ref), (st["e_lj"], ref)
    assert st["pairs"] == 3315997
