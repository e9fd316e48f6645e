"""Force-kernel tiles and the autotuner on the GPU.

Every tile keeps parity with the oracle (partner counts and pair totals exact, forces within
SUM_TOL * sum_j |f_ij|) and is bit-reproducible run to run; tiles differ from one another only in
the rounding of FP32 partial sums inside a work piece.  The autotuner picks the fastest candidate,
caches it per process and, with MDRL_TUNE_CACHE, across processes.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems
from helpers import oracle_from_ctx

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
SUM_TOL = 2e-6
FIX_ABS = 64 * 2.0 ** -24
CANDIDATES = {(w, s, p) for w in (4, 8) for s in (3, 4, 6, 8, 12) for p in (0, 1)} | {(1, g, 1) for g in (1, 2, 3)}


@pytest.fixture(scope="module")
def sysm():
    return systems.small_ljc(3000, 37.5, 12.0, seed=21)     # 3 x 3 x 3 cells, ~110 per cell


@pytest.mark.parametrize("tile", [(4, 3, 0), (4, 12, 1), (8, 6, 1), (8, 1, 0), (4, 32, 1), (4, 6, 1),
                                  (1, 1, 1), (1, 2, 1), (1, 4, 1)])
@pytest.mark.parametrize("grid", ["3 cells", "4 cells"])
@pytest.mark.parametrize("exact", [False, True])
def test_tile_parity_and_reproducibility(sysm, tile, grid, exact):
    if grid.startswith("4"):
        sysm = systems.small_ljc(6400, 50.0, 12.0, seed=22)
        assert sysm.ncell == (4, 4, 4)
    p = sysm.params(table_bins=512, table_order=2 if exact else 1,
                    flags=m.FLAG_ENERGY | (m.FLAG_EXACT_DIFF if exact else 0))
    x, y, z = (np.ascontiguousarray(sysm.pos[:, k]) for k in range(3))
    with m.Context(p) as ctx:
        ctx.set_tile(*tile)
        assert ctx.tile() == tile
        F, st, cnt = ctx.force(x, y, z, sysm.q, sysm.type, counts=True)
        F2, _, _ = ctx.force(x, y, z, sysm.q, sysm.type)
        o = oracle_from_ctx(ctx, sysm)
    Fo, Fabs, cnto, sto = o.force_cells()
    assert np.array_equal(cnt, cnto)
    assert st["pairs"] == sto["pairs"]
    assert np.array_equal(F.view(np.uint32), F2.view(np.uint32))
    err = np.abs(F - Fo) / (SUM_TOL * Fabs + FIX_ABS)
    assert err.max() <= 1.0, err.max()


@pytest.mark.parametrize("tile", [(1, 1, 1), (1, 3, 1)])
@pytest.mark.parametrize("order,arith,exact", [(0, m.ARITH_FMA, False), (0, m.ARITH_FMA, True),
                                               (1, m.ARITH_SEPARATE, False), (2, m.ARITH_SEPARATE, False),
                                               (3, m.ARITH_FMA, False), (3, m.ARITH_FMA, True)])
def test_warp_tile_every_evaluation_mode(sysm, tile, order, arith, exact):
    """The one-warp-per-item kernel for every table order (0 = direct evaluation), both arithmetic
    modes of the reference's difference rule and the exact rule: partner counts and pair totals
    exact, forces within the parity bound, energies within 1e-5, bit-reproducible."""
    kw = dict(table_bins=512, arith=arith, flags=m.FLAG_ENERGY | (m.FLAG_EXACT_DIFF if exact else 0))
    if order == 0:
        kw["eval"] = m.EVAL_DIRECT
    else:
        kw["table_order"] = order
    p = sysm.params(**kw)
    x, y, z = (np.ascontiguousarray(sysm.pos[:, k]) for k in range(3))
    with m.Context(p) as ctx:
        ctx.set_tile(*tile)
        F, st, cnt = ctx.force(x, y, z, sysm.q, sysm.type, counts=True)
        F2, _, _ = ctx.force(x, y, z, sysm.q, sysm.type)
        o = oracle_from_ctx(ctx, sysm)
    Fo, Fabs, cnto, sto = o.force_cells()
    assert np.array_equal(cnt, cnto)
    assert st["pairs"] == sto["pairs"]
    assert np.array_equal(F.view(np.uint32), F2.view(np.uint32))
    err = np.abs(F - Fo) / (SUM_TOL * Fabs + FIX_ABS)
    assert err.max() <= 1.0, err.max()
    for key in ("e_lj", "e_coul", "virial"):
        assert abs(st[key] - sto[key]) <= 1e-5 * max(abs(sto[key]), 1.0), (key, st[key], sto[key])


def test_autotune_picks_a_candidate_and_caches(sysm):
    p = sysm.params(table_bins=512)
    args = (sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
    with m.Context(p) as ctx:
        ctx.set_state(*args)
        before = ctx.state()
        r = ctx.autotune(retime=True)
        assert r["tile"] in CANDIDATES
        assert 0 < r["ms"] <= r["default_ms"]
        assert ctx.tile() == r["tile"]
        for a, b in zip(before, ctx.state()):          # tuning leaves the state untouched
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        ctx.step(5)
        tuned_state = ctx.state()
    with m.Context(p) as ctx:                          # same key: served from the cache
        ctx.set_state(*args)
        r2 = ctx.autotune()
        assert r2["tile"] == r["tile"]
    with m.Context(p) as ctx:                          # the same calls with an explicit tile
        ctx.set_state(*args)
        ctx.set_tile(*r["tile"])
        ctx.step(5)
        for a, b in zip(tuned_state, ctx.state()):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


_CHILD = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems
s = systems.small_ljc(3000, 37.5, 12.0, seed=21)
with m.Context(s.params(table_bins=512)) as ctx:
    ctx.set_state(s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.vel, s.q, s.type)
    print(json.dumps(ctx.autotune()))
"""


def test_tune_cache_file_across_processes(tmp_path):
    cache = tmp_path / "tune.txt"
    env = dict(os.environ, MDRL_TUNE_CACHE=str(cache))
    outs = []
    for _ in range(2):
        r = subprocess.run([sys.executable, "-c", _CHILD, str(ROOT)], env=env, capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(json.loads(r.stdout.strip().splitlines()[-1]))
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 1                         # the second process read it instead of tuning
    key, w, s, pr, ms = lines[0].split()
    assert (int(w), int(s), int(pr)) == tuple(outs[0]["tile"]) == tuple(outs[1]["tile"])


def test_batch_autotune_and_tile_parity():
    reps = [systems.replica(n, r) for r, n in enumerate([1200, 3000, 9000])]
    pos, vel, q, t, spec = systems.concat(reps)
    p = reps[0].params(table_bins=512)
    with m.Batch(p, spec) as b:
        b.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, q, t)
        r = b.autotune(retime=True)
        assert (r["tile"][0] == 4 and r["tile"][1] in (3, 4, 6, 8, 12) and r["tile"][2] in (0, 1)) or \
            (r["tile"][0] == 1 and r["tile"][1] in (1, 2, 3) and r["tile"][2] == 1)
        assert 0 < r["ms"] <= r["default_ms"]
        with pytest.raises(m.MdrlError):
            b.set_tile(8, 6)
        b.set_tile(4, 3, 1)
        F, _, _ = b.force(pos[:, 0], pos[:, 1], pos[:, 2], q, t)
        offs = b.offsets
    for k in (1, 2):                               # half-shell replicas: equal to a lone context
        s = reps[k]
        with m.Context(s.params(table_bins=512)) as ctx:
            ctx.set_tile(4, 3, 1)
            F1, _, _ = ctx.force(s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.q, s.type)
        assert np.array_equal(F[offs[k]:offs[k + 1]].view(np.uint32), F1.view(np.uint32))


def test_tile_validation(sysm):
    with m.Context(sysm.params(accum=m.ACC_FP32_ATOMIC)) as ctx:
        with pytest.raises(m.MdrlError) as e:
            ctx.set_tile(8, 6)
        assert e.value.status == 1
        with pytest.raises(m.MdrlError):
            ctx.set_tile(4, 0)
        with pytest.raises(m.MdrlError):
            ctx.set_tile(2, 6)
        with pytest.raises(m.MdrlError):
            ctx.set_tile(4, 6, 2)
        with pytest.raises(m.MdrlError):
            ctx.set_tile(4, 6, 1)                   # pruned kernels exist for fixed point only
        with pytest.raises(m.MdrlError):
            ctx.set_tile(1, 1, 1)                   # one warp per item: fixed point only
        ctx.set_tile(4, 12)
        assert ctx.tile() == (4, 12, 0)
    with m.Context(sysm.params()) as ctx:
        for bad in ((1, 0, 1), (1, 5, 1), (1, 2, 0)):
            with pytest.raises(m.MdrlError):
                ctx.set_tile(*bad)
        ctx.set_tile(1, 3, 1)
        assert ctx.tile() == (1, 3, 1)
