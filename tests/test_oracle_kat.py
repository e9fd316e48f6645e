"""The oracle pinned to the reference's own known answers (CPU only).

KAT-1  VERIFICATION_REFERENCE_OUTPUT.txt: per-pair r2, F, Fx, Fy, Fz of 10,000 ApoA1 pairs with
       the ROM tables c{0,1}_{14,8}.hex -- bit-exact with separately rounded mul/add.
KAT-2  cell_ini_file_*: binning of the 20k LJArgon positions -- counts, order and FP32 bits.
KAT-3  c{0,1}_{14,8,12,6,3,1}.txt: the table fit (product fitter and the oracle's own numpy fitter)
       evaluates within 2e-6 of the reference's tables (relative to the function value).
C model  the oracle's restatement of MD_Evaluation_Model.cpp prints, line for line, what the
       unmodified reference binary printed (fixture), and matches a fresh run of the binary.
"""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
import sc2019_md_gb300 as m
from helpers import GOLDEN, kat1, kat2_positions

ROOT = Path(__file__).resolve().parent.parent


def _kat1_system(arith):
    pos, expect, tab2 = kat1()
    tab = np.zeros((6, 2, 14 * 256), np.float32)
    tab[:2] = tab2
    pc = np.array([[1, -1, 1, -1]], np.float32)
    return pos, expect, oracle.System(pos, (0, 0, 0), (1, 1, 1), 14.0, pc, tab=tab, order=1, nseg=14,
                                      bins=256, min_log2=-6, arith=arith)


def test_kat1_pairs_bit_exact():
    pos, expect, s = _kat1_system(arith=1)
    got = np.zeros((10000, 5), np.float32)
    for k in range(10000):
        i, j = divmod(k, 100)
        _, out = s.pair(pos[i], pos[j])
        got[k] = [out[3], out[0], out[1], out[2], out[4]]
    assert np.array_equal(got.view(np.uint32), expect[:, :5])
    d = (pos[:, None, :] - pos[None, :, :]).reshape(-1, 3).astype(np.float32)
    assert np.array_equal(d.view(np.uint32), expect[:, 5:8])


def test_kat1_fused_rounding_differs():
    """With fused multiply-adds only a minority of the golden forces match: the golden vectors
    were produced with separately rounded products (MATLAB polyval in single precision)."""
    pos, expect, s = _kat1_system(arith=0)
    same = 0
    for k in range(10000):
        i, j = divmod(k, 100)
        _, out = s.pair(pos[i], pos[j])
        same += int(np.float32(out[3]).view(np.uint32) == expect[k, 0])
    assert 106 <= same < 5000


def test_kat2_binning_bit_exact():
    pos, d = kat2_positions()
    cell_of, start, order, mx = oracle.bin_cells(pos, (7 * 8.5, 6 * 8.5, 6 * 8.5), (7, 6, 6))
    for cx in range(3):
        for cy in range(3):
            for cz in range(3):
                c = (cx * 6 + cy) * 6 + cz
                ids = order[start[c]:start[c + 1]]
                assert len(ids) == d["counts"][cx, cy, cz]
                assert np.array_equal(pos[ids].view(np.uint32), d[f"c{cx + 1}{cy + 1}{cz + 1}"])
    assert start[-1] == 20000 and mx < 100     # the reference's CELL_PARTICLE_MAX is 100


@pytest.mark.parametrize("fitter", ["product", "oracle"])
def test_kat3_tables(fitter):
    t = (m.fit_tables(1, 9, 256, -2) if fitter == "product" else oracle.fit_tables(1, 9, 256, -2)).astype(np.float64)
    k = np.load(GOLDEN / "kat3_tables.npz")
    eps = 1.995996 * 1.995996
    sig = 2.1
    kq = 1.0 / (4 * 3.14 * eps)   # the reference's Coulomb prefactor (pi = 3.14, LJ eps)
    pref = {"14": 48 * eps * sig ** 12, "8": 24 * eps * sig ** 6, "3": kq,
            "12": 4 * eps * sig ** 12, "6": 4 * eps * sig ** 6, "1": kq}
    expo = {"14": -7, "8": -4, "3": -1.5, "12": -6, "6": -3, "1": -0.5}
    fi = {"14": 0, "8": 1, "3": 2, "12": 3, "6": 4, "1": 5}
    seg = np.repeat(np.arange(9), 256)
    b = np.tile(np.arange(256), 9)
    lo = 2.0 ** (seg - 2)
    w = lo / 256
    for frac in (0.0, 0.25, 0.5, 0.75, 0.999):
        x = lo + (b + frac) * w
        for f in fi:
            ref = k[f"c1_{f}"] * x + k[f"c0_{f}"]
            mine = (t[fi[f], 1] * x + t[fi[f], 0]) * pref[f]
            exact = pref[f] * x ** expo[f]
            assert np.max(np.abs(mine - ref) / exact) < 2e-6, (f, frac)


def test_fitters_agree():
    for order, bins in ((1, 256), (1, 512), (2, 256), (3, 128)):
        a = oracle.fit_tables(order, 8, bins, -2)
        b = m.fit_tables(order, 8, bins, -2)
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30)) < 1e-5
    for order, bins in ((2, 256), (3, 128), (2, 1024)):           # the bin-local form
        a = oracle.fit_tables(order, 8, bins, -2, local=True)
        b = m.fit_tables(order, 8, bins, -2, local=True)
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30)) < 1e-5


def test_bin_local_form_evaluates_like_the_monomial_form():
    """The same least-squares polynomial in either form: evaluated in FP64 at points across each
    bin, the bin-local and the monomial coefficients agree to the monomial form's FP32 coefficient
    rounding (which cancellation amplifies) -- and the local form is the closer one to the
    function itself."""
    order, nseg, bins, m0 = 2, 8, 256, -2
    mono = m.fit_tables(order, nseg, bins, m0).astype(np.float64)
    loc = m.fit_tables(order, nseg, bins, m0, local=True).astype(np.float64)
    idx = np.arange(nseg * bins)
    seg, b = np.divmod(idx, bins)
    x0 = np.ldexp(1.0 + b / bins, m0 + seg)
    w = np.ldexp(1.0, m0 + seg) / bins
    expo = np.array([-7.0, -4.0, -1.5, -6.0, -3.0, -0.5])
    for frac in (0.1, 0.5, 0.9):
        x = x0 + frac * w
        u = x - x0
        for f in range(6):
            pm = mono[f, 0] + x * (mono[f, 1] + x * mono[f, 2])
            pl = loc[f, 0] + u * (loc[f, 1] + u * loc[f, 2])
            exact = x ** expo[f]
            em, el = np.abs(pm - exact) / exact, np.abs(pl - exact) / exact
            assert el.max() < 2e-7, (f, frac, el.max())
            assert el.max() <= em.max(), (f, frac)


def _ref_lines():
    return (GOLDEN / "cmodel_ref_output.txt").read_text().splitlines()


def test_cmodel_restatement_matches_reference_output():
    pos = oracle.read_pdb_like_reference(GOLDEN / "cmodel_input.pdb", 500)
    _, _, e, _ = oracle.cmodel_run(pos, np.zeros_like(pos), 100)
    lines = [f"Iteration {i}, System energy is {e[i, 0]:f}, Kinetic Energy is {e[i, 1]:f}" for i in range(100)]
    assert lines == _ref_lines()


def test_cmodel_reference_binary_rerun():
    exe = ROOT / "oracle" / "_ref" / "cmodel_ref"
    if not exe.exists():
        pytest.skip("reference C model not built here (the reference tree is not mounted)")
    r = subprocess.run([str(exe)], env=dict(os.environ, MDRL_REF_PDB=str(GOLDEN / "cmodel_input.pdb")),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.splitlines() == _ref_lines()


def _brute_counts(pos, box, rc):
    """All-pairs FP32 partner counts with the reference's datapath (numpy float32, no fusion)."""
    pos = pos.astype(np.float32)
    L = np.asarray(box, np.float32)
    h = np.float32(0.5) * L
    rc2 = np.float32(rc) * np.float32(rc)
    counts = np.zeros(len(pos), np.int64)
    for i in range(len(pos)):
        d = (pos[i] - pos).astype(np.float32)
        d = np.where(d > h, d - L, np.where(d < -h, d + L, d)).astype(np.float32)
        r2 = ((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]).astype(np.float32)
        counts[i] = int(((r2 > 0) & (r2 <= rc2)).sum())
    return counts


@pytest.mark.parametrize("box,ncell", [((30.0, 30.0, 30.0), (3, 3, 3)), ((40.0, 52.0, 31.0), (4, 5, 3))])
def test_halfshell_visits_every_pair_once(box, ncell):
    rng = np.random.default_rng(17)
    n = 1500
    pos = (rng.random((n, 3)) * np.asarray(box)).astype(np.float32)
    pos = np.minimum(pos, np.nextafter(np.asarray(box, np.float32), 0))
    rc = 10.0
    pc = np.array([[1.0, -1.0, 1.0, -1.0]], np.float32)
    s = oracle.System(pos, box, ncell, rc, pc, eval=1)
    _, _, cnt, st = s.force_cells()
    bc = _brute_counts(pos, box, rc)
    assert np.array_equal(cnt, bc)
    assert st["pairs"] * 2 == bc.sum()
    nc = np.asarray([len(np.where(np.floor(pos[:, d] / np.float32(box[d] / ncell[d])) >= 0)[0]) for d in range(3)])
    assert (nc == n).all()


def test_oracle_tables64_close_to_direct64():
    from sc2019_md_gb300 import systems
    s = systems.small_ljc(1500, 37.5, 12.0, seed=2)
    pc64 = oracle.lb_coefficients(s.sigma, s.epsilon)
    tab = oracle.fit_tables(1, 10, 1024, -2)        # 2^-2 .. 2^8 covers rc^2 = 144
    o = oracle.System(s.pos, s.box, s.ncell, s.cutoff, pc64.astype(np.float32), q=s.q, type=s.type,
                      ke=s.coulomb_k, tab=tab, order=1, nseg=10, bins=1024, min_log2=-2, pcoef64=pc64,
                      ke64=s.coulomb_k)
    Ft, _ = o.force_tables64()
    Fd, _ = o.force_direct64()
    rel = np.linalg.norm(Ft - Fd, axis=1) / np.linalg.norm(Fd, axis=1)
    assert np.median(rel) < 2e-6
