"""GPU parity of the range-limited force path against the oracle and the reference's fixtures.

Bit-exact: per-pair r2 / fscal / force components (KAT-1 and random pairs), cell assignment and
in-cell order (KAT-2), per-particle partner counts and pair totals.  Tolerance-checked: summed
forces (FP32 partial sums in a fixed order vs the oracle's order-free sum of the same FP32
per-pair forces: |dF| <= 2e-6 * sum_j |f_ij| per component) and energies (1e-6 relative).
"""
import numpy as np
import pytest

import oracle
import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems
from helpers import boundary_dimers, force_err, kat1, kat2_positions, oracle_from_ctx

pytestmark = pytest.mark.gpu

SUM_TOL = 2e-6     # |F_gpu - F_oracle| <= SUM_TOL * sum_j |f_ij| + FIX_ABS, per particle and component
FIX_ABS = 64 * 2.0 ** -24   # int64 fixed point: each of a particle's per-unit flushes rounds to 2^-24


def test_pair_eval_kat1_bit_exact():
    """The 100 x 100 ApoA1 pairs of VERIFICATION_REFERENCE_OUTPUT.txt through mdrl_pair_eval with
    the reference's ROM tables: r2, F, Fx, Fy, Fz bit-identical for all 10,000 pairs."""
    pos, expect, tab = kat1()
    p = m.default_params(box=(1000.0, 1000.0, 1000.0), cutoff=14.0, table_min_log2=-6,
                         arith=m.ARITH_SEPARATE, flags=m.FLAG_NO_PBC)
    with m.Context(p) as ctx:
        ctx.set_tables(tab, order=1, nseg=14, bins=256, min_log2=-6, raw=True)
        i, j = np.divmod(np.arange(10000), 100)
        ref = np.concatenate([pos[i], np.zeros((10000, 1), np.float32)], 1)
        nbr = np.concatenate([pos[j], np.zeros((10000, 1), np.float32)], 1)
        out, aux = ctx.pair_eval(ref, nbr)
    got = np.stack([aux[:, 1], out[:, 0], out[:, 1], out[:, 2], aux[:, 0]], 1).view(np.uint32)
    exp = expect[:, :5]
    assert np.array_equal(got, exp), f"{int((got != exp).any(1).sum())} of 10000 pairs differ"
    assert int((exp[:, 0] != 0).sum()) == 9894


@pytest.mark.parametrize("order,bins", [(0, 256), (1, 256), (1, 512), (2, 256), (3, 256)])
@pytest.mark.parametrize("arith,exact", [(m.ARITH_FMA, False), (m.ARITH_SEPARATE, False), (m.ARITH_FMA, True)])
def test_pair_eval_random_vs_oracle(order, bins, arith, exact):
    """Random periodic pairs of 4 types with charges: bit-identical to the oracle's datapath (both
    difference rules; orders 2-3 with the library's bin-local tables)."""
    rng = np.random.default_rng(100 + order * 7 + arith)
    n = 4000
    L = 40.0
    sysm = systems.small_ljc(64, L, 12.0, seed=3)
    p = sysm.params(table_order=max(order, 1), table_bins=bins, arith=arith,
                    eval=m.EVAL_DIRECT if order == 0 else m.EVAL_TABLE,
                    flags=m.FLAG_EXACT_DIFF if exact else 0)
    a = rng.uniform(0, L, (n, 3)).astype(np.float32)
    b = (a + rng.uniform(-13, 13, (n, 3))).astype(np.float32) % np.float32(L)
    b[:50] = a[:50]                                   # r2 = 0 pairs are filtered
    qa = rng.choice([-0.42, 0.42], n).astype(np.float32)
    qb = rng.choice([-0.42, 0.42], n).astype(np.float32)
    ta = rng.integers(0, 4, n).astype(np.int32)
    tb = rng.integers(0, 4, n).astype(np.int32)
    with m.Context(p) as ctx:
        out, aux = ctx.pair_eval(np.column_stack([a, qa]), np.column_stack([b, qb]), ta, tb)
        o = oracle_from_ctx(ctx, sysm)
    exp = np.zeros((n, 5), np.float32)
    for k in range(n):
        ok, r = o.pair(a[k], b[k], qa[k], qb[k], ta[k], tb[k])
        exp[k] = [r[0], r[1], r[2], r[3], r[4]]
    got = np.column_stack([out[:, :3], aux[:, 1], aux[:, 0]])
    assert np.array_equal(got.view(np.uint32), exp.view(np.uint32))


def test_bin_kat2_bit_exact():
    """The LJArgon 20k binning (7x6x6 cells of 8.5 A): the 27 cell_ini files' counts, order and
    FP32 bits, and the whole assignment equal to the oracle's."""
    pos, d = kat2_positions()
    p = m.default_params(box=(7 * 8.5, 6 * 8.5, 6 * 8.5), cutoff=8.5, ncell=(7, 6, 6))
    with m.Context(p) as ctx:
        cell_of, count, order = ctx.bin(pos[:, 0], pos[:, 1], pos[:, 2])
    start = np.concatenate([[0], np.cumsum(count)])
    for cx in range(3):
        for cy in range(3):
            for cz in range(3):
                c = (cx * 6 + cy) * 6 + cz
                ids = order[start[c]:start[c + 1]]
                assert len(ids) == d["counts"][cx, cy, cz]
                assert np.array_equal(pos[ids].view(np.uint32), d[f"c{cx + 1}{cy + 1}{cz + 1}"])
    oc, ostart, oorder, _ = oracle.bin_cells(pos, p.box, (7, 6, 6))
    assert np.array_equal(cell_of, oc)
    assert np.array_equal(order, oorder)


def _check_force(sysm, params, tol=SUM_TOL, tile=None):
    with m.Context(params) as ctx:
        if tile is not None:
            ctx.set_tile(*tile)
        x, y, z = (np.ascontiguousarray(sysm.pos[:, k]) for k in range(3))
        F, st, cnt = ctx.force(x, y, z, sysm.q, sysm.type, counts=True)
        F2, st2, _ = ctx.force(x, y, z, sysm.q, sysm.type)
        o = oracle_from_ctx(ctx, sysm)
    Fo, Fabs, cnto, sto = o.force_cells()
    assert np.array_equal(cnt, cnto), "partner counts differ"
    assert st["pairs"] == sto["pairs"]
    assert st["below_table"] == sto["below_table"]
    err = np.abs(F - Fo) / (tol * Fabs + FIX_ABS)
    assert err.max() <= 1.0, f"max |dF| / (tol*sum|f| + fixed-point quantum) = {err.max():.3e}"
    if params.accum == m.ACC_FIXED64:
        assert np.array_equal(F.view(np.uint32), F2.view(np.uint32)), "not bit-reproducible"
    for key in ("e_lj", "e_coul", "virial"):
        ref = sto[key]
        assert abs(st[key] - ref) <= 1e-5 * max(abs(ref), 1.0), (key, st[key], ref)
    return F, Fo, o


@pytest.mark.parametrize("order,bins", [(0, 256), (1, 256), (1, 512), (2, 256), (3, 128)])
@pytest.mark.parametrize("arith,exact", [(m.ARITH_FMA, False), (m.ARITH_SEPARATE, False), (m.ARITH_FMA, True)])
def test_force_small_ljc(order, bins, arith, exact):
    sysm = systems.small_ljc(3000, 37.5, 12.0, seed=21)          # 3x3x3 cells, ~110 per cell
    p = sysm.params(table_order=max(order, 1), table_bins=bins, arith=arith,
                    eval=m.EVAL_DIRECT if order == 0 else m.EVAL_TABLE,
                    flags=m.FLAG_ENERGY | (m.FLAG_EXACT_DIFF if exact else 0))
    _check_force(sysm, p)


@pytest.mark.parametrize("accum,tile", [(m.ACC_FIXED64, None), (m.ACC_FIXED64, (1, 2, 1)), (m.ACC_FP32_ATOMIC, None)])
@pytest.mark.parametrize("which", ["lj1728", "ljc92k"])
def test_force_error_bound(which, accum, tile):
    """The stated accuracy: with the exact-difference rule and the library's bin-local order-2
    tables (512 bins), the GPU forces are within 1e-5 of the FP64 direct oracle in the primary
    norm, max_i |dF_i| / rms_j |F_j| (median per-particle relative error within 1e-6), for the
    fixed-point ("tuned") and the FP32-atomic ("plain") accumulation alike; partner counts
    bit-equal to the oracle's exact-rule datapath."""
    sysm = getattr(systems, which)()
    p = sysm.params(table_order=2, table_bins=512, flags=m.FLAG_EXACT_DIFF, accum=accum)
    F, Fo, o = _check_force(sysm, p, tile=tile)
    F64, _ = o.force_direct64()
    emax, emed = force_err(F, F64)
    assert emax <= 1e-5, emax
    assert emed <= 1e-6, emed


def test_force_lj1728_and_fp64_error():
    """The 1,728-atom LJ argon cube (3x3x3 cells): parity with the oracle, and the stated force
    error of 1st-order 1024-bin tables against the FP64 direct oracle (median per-particle
    relative error <= 1e-5; max error over the rms force <= 2e-5)."""
    sysm = systems.lj1728()
    p = sysm.params(table_bins=1024, flags=m.FLAG_ENERGY)
    F, Fo, o = _check_force(sysm, p)
    F64, _ = o.force_direct64()
    emax, emed = force_err(F, F64)
    assert emed <= 1e-5, emed
    assert emax <= 2e-5, emax


@pytest.mark.parametrize("bins", [512, 1024])
def test_force_ljc_fp64_error(bins):
    """LJ+Coulomb, 4 types: median per-particle relative error against FP64 direct <= 1e-5 with
    1st-order 512- and 1024-bin tables (the benchmark's setting is 512)."""
    sysm = systems.small_ljc(6000, 49.6, 12.0, seed=5)
    p = sysm.params(table_bins=bins)
    with m.Context(p) as ctx:
        F, st, _ = ctx.force(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q, sysm.type)
        o = oracle_from_ctx(ctx, sysm)
    F64, _ = o.force_direct64()
    emax, emed = force_err(F, F64)
    assert emed <= 1e-5, emed


def test_force_fp32_atomic_plain():
    sysm = systems.small_ljc(3000, 37.5, 12.0, seed=22)
    p = sysm.params(accum=m.ACC_FP32_ATOMIC, table_bins=512)
    _check_force(sysm, p, tol=1e-5)


def test_force_kahan_compensated():
    """Compensated FP32 accumulation: FP32 partial sums in a fixed order plus a TwoSum-compensated
    global sum -- within the FP32 summation bound of the oracle's exact sum."""
    sysm = systems.small_ljc(3000, 37.5, 12.0, seed=23)
    p = sysm.params(accum=m.ACC_KAHAN, table_bins=512)
    _check_force(sysm, p)


def test_force_large_cell_chunks():
    """A cell holding more particles than one shared-memory chunk (256) is processed in chunks."""
    rng = np.random.default_rng(8)
    L = 30.0
    dense = systems.uniform_min_sep(700, (9.9, 9.9, 9.9), 0.45, rng)          # 700 in cell (0,0,0)
    rest = systems.uniform_min_sep(800, (19.0, 30.0, 30.0), 0.45, rng) + np.array([10.5, 0.0, 0.0])
    pos = systems.wrap_into_box(np.concatenate([dense, rest]), (L, L, L))
    sysm = systems.System("dense", (L, L, L), 10.0, (3, 3, 3), pos, np.zeros_like(pos), None,
                          np.zeros(1500, np.int32), [0.5], [0.01], [39.95], 0.0)
    p = sysm.params(table_min_log2=-8)
    with m.Context(p) as ctx:
        F, st, cnt = ctx.force(pos[:, 0], pos[:, 1], pos[:, 2], None, None, counts=True)
        o = oracle_from_ctx(ctx, sysm)
    Fo, Fabs, cnto, sto = o.force_cells()
    assert np.array_equal(cnt, cnto)
    assert (np.abs(F - Fo) / (SUM_TOL * Fabs + FIX_ABS)).max() <= 1.0


def test_edge_cases():
    p = m.default_params()
    with m.Context(p) as ctx:
        F, st, _ = ctx.force(np.zeros(0), np.zeros(0), np.zeros(0))
        assert F.shape == (0, 3) and st["pairs"] == 0
        F, st, _ = ctx.force([1.0], [2.0], [3.0])
        assert np.all(F == 0) and st["pairs"] == 0
        # a particle exactly at 0 and one just below L
        L = np.float32(25.5)
        x = np.array([0.0, np.nextafter(L, np.float32(0))], np.float32)
        F, st, _ = ctx.force(x, np.array([1.0, 1.0], np.float32), np.array([1.0, 1.0], np.float32))
        assert st["pairs"] == 1
        with pytest.raises(m.MdrlError) as e:
            ctx.force([26.0], [1.0], [1.0])
        assert e.value.status == 1
        with pytest.raises(m.MdrlError):
            ctx.force([np.nan], [1.0], [1.0])
        with pytest.raises(m.MdrlError) as e:
            ctx.force([1.0], [1.0], [1.0], type=[5])
        assert e.value.status == 1 and "types" in str(e.value)
    with pytest.raises(m.MdrlError) as e:
        with m.Context(m.default_params(box=(16.0, 25.5, 25.5))) as ctx:   # 1 cell of 16 A on x
            ctx.force([1.0], [1.0], [1.0])
    assert e.value.status == 3
    with pytest.raises(m.MdrlError):
        m.Context(m.default_params(table_bins=300))


@pytest.mark.parametrize("ncell,L,ndimers,seed", [(5, 50.5, 600, 5), (3, 31.5, 300, 6)])
@pytest.mark.parametrize("tile", [None, (4, 6, 1), (1, 1, 1)])
def test_cutoff_boundary_pairs(ncell, L, ndimers, seed, tile):
    """Dimers whose r2 lies exactly on rc2 or one ulp either side under the reference's rounding,
    chosen so that a fused multiply-add in r2 would decide them the other way (hundreds of such
    pairs per system): partner counts and the pair total bit-equal to the oracle, with the
    per-unit shift (5 cells per axis) and the per-pair wrap (3 cells), unpruned and pruned."""
    pos = boundary_dimers(ndimers, L, 10.0, seed=seed)
    n = len(pos)
    rng = np.random.default_rng(seed)
    q = np.where(rng.permutation(n) < n // 2, -0.42, 0.42).astype(np.float32)
    sysm = systems.System(name="boundary", box=(L, L, L), cutoff=10.0, ncell=(ncell,) * 3, pos=pos,
                          vel=np.zeros_like(pos), q=q, type=np.zeros(n, np.int32), sigma=[2.0],
                          epsilon=[0.1], mass=[39.95], coulomb_k=systems.COULOMB_K)
    _check_force(sysm, sysm.params(table_bins=512, flags=m.FLAG_ENERGY), tile=tile)


@pytest.mark.parametrize("tile", [None, (4, 6, 1), (8, 4, 1), (1, 1, 1), (1, 2, 1)])
@pytest.mark.parametrize("exact", [False, True])
def test_full_size_ljc92k_counts_and_forces(tile, exact):
    """The 92,224-atom LJ+Coulomb system at full size, with the default tile and with pruned
    (survivor-list) tiles, the reference's difference rule (order-1 tables) and the exact rule
    (bin-local order-2 tables): partner counts and pair total bit-equal to the oracle, forces within
    the summation tolerance."""
    sysm = systems.ljc92k()
    p = sysm.params(table_bins=512, table_order=2 if exact else 1, flags=m.FLAG_EXACT_DIFF if exact else 0)
    F, Fo, o = _check_force(sysm, p, tile=tile)


def test_full_size_ljc1m_pairs_and_reproducibility():
    """1,048,576 atoms, 16 types, 22^3 cells: the pair total equals the oracle's (multi-threaded
    half-shell count), and the fixed-point forces are bit-identical on a second evaluation."""
    sysm = systems.ljc1m()
    p = sysm.params(table_bins=512)
    x, y, z = (np.ascontiguousarray(sysm.pos[:, k]) for k in range(3))
    with m.Context(p) as ctx:
        F1, st, _ = ctx.force(x, y, z, sysm.q, sysm.type)
        F2, _, _ = ctx.force(x, y, z, sysm.q, sysm.type)
        ctx.set_tile(4, 6, 1)
        _, st_pruned, _ = ctx.force(x, y, z, sysm.q, sysm.type)
        ctx.set_tile(1, 1, 1)
        Fw1, st_warp, _ = ctx.force(x, y, z, sysm.q, sysm.type)
        Fw2, _, _ = ctx.force(x, y, z, sysm.q, sysm.type)
        o = oracle_from_ctx(ctx, sysm)
    _, pairs = o.force_cells_mt(0)
    assert st["pairs"] == pairs
    assert st_pruned["pairs"] == pairs
    assert st_warp["pairs"] == pairs
    assert np.array_equal(Fw1.view(np.uint32), Fw2.view(np.uint32))
    assert np.array_equal(F1.view(np.uint32), F2.view(np.uint32))
    assert np.isfinite(F1).all()
