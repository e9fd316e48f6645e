"""Batched replicas on the GPU (mdrl_batch_*).

* Half-shell replicas (>= 3 cells per axis): forces, partner counts, pair totals and whole
  trajectories bit-identical to a single-system context running the same replica alone.
* All-pairs replicas (fewer cells; edge in (rc, 3 rc)): pair totals and partner counts equal to
  the oracle's all-image restatement, forces within SUM_TOL * sum_j |f_ij| of the oracle's sum of
  the same FP32 pair forces, energies within 1e-5 of its FP64 table evaluation.
* Determinism run to run, energy conservation of liquid-argon replicas on every path, and the
  error paths.
"""
import numpy as np
import pytest

import oracle
import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems
from helpers import oracle_from_ctx

pytestmark = pytest.mark.gpu

SUM_TOL = 2e-6
FIX_ABS = 64 * 2.0 ** -24

# all images (14.4 A, 19.1 A), minimum image (22.9 A, 27.1 A), half shell with the per-pair
# wrap of 3 cells (31.1 A, 39.1 A) and with 4 cells (44.8 A, where a lone context uses per-unit
# shifts)
SIZES = [300, 700, 1200, 2000, 3000, 6000, 9000]
PATHS = [m.PATH_ALL_IMAGES, m.PATH_ALL_IMAGES, m.PATH_MIN_IMAGE, m.PATH_MIN_IMAGE,
         m.PATH_HALF_SHELL, m.PATH_HALF_SHELL, m.PATH_HALF_SHELL]


@pytest.fixture(scope="module")
def reps():
    return [systems.replica(n, r) for r, n in enumerate(SIZES)]


def _params(sysm, **kw):
    kw.setdefault("table_bins", 512)
    return sysm.params(**kw)


def _split(a, offs, r):
    return a[offs[r]:offs[r + 1]]


def test_batch_layout(reps):
    pos, vel, q, t, spec = systems.concat(reps)
    with m.Batch(_params(reps[0]), spec) as b:
        lay = b.layout()
    assert list(lay["path"]) == PATHS
    for r, s in enumerate(reps):
        assert tuple(lay["ncell"][r]) == s.ncell
        nct = int(np.prod(s.ncell))
        if PATHS[r] == m.PATH_HALF_SHELL:
            assert lay["items"][r] == nct * 14
        elif PATHS[r] == m.PATH_MIN_IMAGE:
            assert lay["items"][r] == nct * (nct + 1) // 2     # every pair of its 2 x 2 x 2 cells
        else:
            assert lay["items"][r] == (s.n + 127) // 128
    assert lay["total_items"] == lay["items"].sum()


@pytest.mark.parametrize("tile", [None, (1, 2, 1)])
def test_batch_force_half_shell_equals_single_context(reps, tile):
    """With the default tile and with one warp per item (half-shell replicas in the warp kernel,
    the others in the CTA kernel), each half-shell replica equals a lone context on the same tile."""
    pos, vel, q, t, spec = systems.concat(reps)
    p = _params(reps[0], flags=m.FLAG_ENERGY)
    with m.Batch(p, spec) as b:
        if tile is not None:
            b.set_tile(*tile)
        F, st, cnt = b.force(pos[:, 0], pos[:, 1], pos[:, 2], q, t, counts=True)
        rs = b.replica_stats()
        offs = b.offsets
    assert st["pairs"] == sum(s["pairs"] for s in rs)
    for r, s in enumerate(reps):
        if PATHS[r] != m.PATH_HALF_SHELL:
            continue
        with m.Context(_params(s, flags=m.FLAG_ENERGY)) as ctx:
            if tile is not None:
                ctx.set_tile(*tile)
            F1, st1, cnt1 = ctx.force(s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.q, s.type, counts=True)
        assert np.array_equal(_split(F, offs, r).view(np.uint32), F1.view(np.uint32)), f"replica {r}"
        assert np.array_equal(_split(cnt, offs, r), cnt1)
        assert rs[r]["pairs"] == st1["pairs"]
        assert rs[r]["below_table"] == st1["below_table"]
        for key in ("e_lj", "e_coul", "virial"):
            assert abs(rs[r][key] - st1[key]) <= 1e-9 * max(abs(st1[key]), 1.0), (r, key)


@pytest.mark.parametrize("arith,tile", [(m.ARITH_FMA, None), (m.ARITH_SEPARATE, None), (m.ARITH_FMA, (1, 1, 1))])
def test_batch_force_all_pairs_vs_oracle(reps, arith, tile):
    pos, vel, q, t, spec = systems.concat(reps)
    p = _params(reps[0], flags=m.FLAG_ENERGY, arith=arith)
    with m.Batch(p, spec) as b:
        if tile is not None:
            b.set_tile(*tile)
        F, st, cnt = b.force(pos[:, 0], pos[:, 1], pos[:, 2], q, t, counts=True)
        F2, _, _ = b.force(pos[:, 0], pos[:, 1], pos[:, 2], q, t)
        rs = b.replica_stats()
        offs = b.offsets
    assert np.array_equal(F.view(np.uint32), F2.view(np.uint32)), "not bit-reproducible"
    checked = 0
    for r, s in enumerate(reps):
        if PATHS[r] == m.PATH_HALF_SHELL:
            continue
        with m.Context(_params(s, flags=m.FLAG_ENERGY, arith=arith)) as ctx:
            o = oracle_from_ctx(ctx, s)
        F64, F32sum, Fabs, cnto, sto = o.force_allimage()
        assert rs[r]["pairs"] == sto["pairs"], r
        assert rs[r]["below_table"] == sto["below_table"], r
        assert np.array_equal(_split(cnt, offs, r), cnto), r
        err = np.abs(_split(F, offs, r) - F32sum) / (SUM_TOL * Fabs + FIX_ABS)
        assert err.max() <= 1.0, (r, float(err.max()))
        for key in ("e_lj", "e_coul", "virial"):
            assert abs(rs[r][key] - sto[key]) <= 1e-5 * max(abs(sto[key]), 1.0), (r, key, rs[r][key], sto[key])
        checked += 1
    assert checked == 4


@pytest.mark.parametrize("tile", [None, (1, 3, 1)])
def test_batch_md_half_shell_equals_single_context(reps, tile):
    pos, vel, q, t, spec = systems.concat(reps)
    p = _params(reps[0])
    with m.Batch(p, spec) as b:
        if tile is not None:
            b.set_tile(*tile)
        b.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, q, t)
        b.step(25)
        X, V, F = b.state()
        offs = b.offsets
    for r, s in enumerate(reps):
        if PATHS[r] != m.PATH_HALF_SHELL:
            continue
        with m.Context(_params(s)) as ctx:
            if tile is not None:
                ctx.set_tile(*tile)
            ctx.set_state(s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.vel, s.q, s.type)
            ctx.step(25)
            X1, V1, F1 = ctx.state()
        for a, a1 in ((X, X1), (V, V1), (F, F1)):
            assert np.array_equal(_split(a, offs, r).view(np.uint32), a1.view(np.uint32)), f"replica {r}"


def test_batch_md_deterministic(reps):
    pos, vel, q, t, spec = systems.concat(reps)
    out = []
    for _ in range(2):
        with m.Batch(_params(reps[0]), spec) as b:
            b.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, q, t)
            b.step(9)
            out.append(b.state())
    for a, c in zip(out[0], out[1]):
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32))


def _argon_replica(nside, seed, rc=12.0):
    rng = np.random.default_rng(seed)
    L = nside * (1.0 / 0.021) ** (1.0 / 3.0)
    g = (np.arange(nside) + 0.5) * (L / nside)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) + rng.uniform(-0.05, 0.05, (nside ** 3, 3))
    pos = systems.wrap_into_box(pos, (L, L, L))
    vel = systems.maxwell(len(pos), np.full(len(pos), 39.95), 120.0, rng)
    nc = int(np.floor(np.float32(L) / np.float32(rc)))
    return systems.System("argon", (L, L, L), rc, (nc, nc, nc), pos, vel, np.zeros(len(pos), np.float32),
                          np.zeros(len(pos), np.int32), [3.4], [0.238], [39.95], 0.0)


def test_batch_energy_conservation_every_path():
    """Liquid-argon replicas (0.021 /A^3, 120 K, rc 12 A) of 6^3 (21.8 A box: all images),
    9^3 (32.6 A: minimum image) and 12^3 atoms (43.5 A: half shell): per-replica total energy
    drift over 400 steps of 2 fs below 1e-2 of the replica's kinetic energy.  (The potential is
    not shifted, so every cutoff crossing changes the total energy by V(rc); the relative drift
    this causes falls as 1/sqrt(N), which sets the smallest replica that can be held to 1e-2.)"""
    reps = [_argon_replica(6, 1), _argon_replica(9, 2), _argon_replica(12, 3)]
    pos, vel, q, t, spec = systems.concat(reps)
    p = reps[0].params(table_bins=1024, table_order=2, flags=m.FLAG_ENERGY)
    with m.Batch(p, spec) as b:
        assert list(b.layout()["path"]) == [m.PATH_ALL_IMAGES, m.PATH_MIN_IMAGE, m.PATH_HALF_SHELL]
        b.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, q, t)
        e = []
        for _ in range(8):
            b.step(50)
            e.append([(s["e_lj"], s["kinetic"]) for s in b.replica_stats()])
    e = np.asarray(e)                          # (checkpoint, replica, 2)
    tot = e[:, :, 0] + e[:, :, 1]
    assert np.isfinite(tot).all()
    for r in range(3):
        drift = np.abs(tot[:, r] - tot[0, r]).max()
        assert drift < 1e-2 * e[:, r, 1].mean(), (r, drift, e[:, r, 1].mean())


def test_batch_errors(reps):
    pos, vel, q, t, spec = systems.concat(reps[:2])
    p = _params(reps[0])
    with m.Batch(p, spec) as b:
        with pytest.raises(m.MdrlError) as e:
            b.step(1)
        assert e.value.status == 6
        bad = pos.copy()
        bad[5, 0] = 100.0                       # outside replica 0's 14.4 A box
        with pytest.raises(m.MdrlError) as e:
            b.force(bad[:, 0], bad[:, 1], bad[:, 2], q, t)
        assert e.value.status == 1 and "positions" in str(e.value)
        tt = t.copy()
        tt[3] = 2
        with pytest.raises(m.MdrlError) as e:
            b.force(pos[:, 0], pos[:, 1], pos[:, 2], q, tt)
        assert e.value.status == 1 and "types" in str(e.value)


def test_batch512_full_size_pair_counts():
    """The full batched workload (512 replicas, 2.52M atoms): every replica's pair count equals
    the oracle's -- the half-shell traversal (multi-threaded restatement) for replicas with 3+
    cells per axis, the all-image rule for the others -- and the batch total is their sum."""
    reps = systems.batch512()
    pos, vel, q, t, spec = systems.concat(reps)
    p = reps[0].params(table_bins=512)
    with m.Batch(p, spec) as b:
        path = b.layout()["path"]
        F, st, _ = b.force(pos[:, 0], pos[:, 1], pos[:, 2], q, t)
        rs = b.replica_stats()
    assert np.isfinite(F).all()
    assert st["pairs"] == sum(r["pairs"] for r in rs)
    for r, s in enumerate(reps):
        pc64 = oracle.lb_coefficients(s.sigma, s.epsilon)
        o = oracle.System(s.pos, s.box, s.ncell, s.cutoff, pc64.astype(np.float32), q=s.q, type=s.type,
                          ke=s.coulomb_k, eval=1, pcoef64=pc64, ke64=s.coulomb_k)
        if path[r] == m.PATH_HALF_SHELL:
            _, pairs = o.force_cells_mt()
        else:
            pairs = o.force_allimage()[4]["pairs"]
        assert rs[r]["pairs"] == pairs, (r, s.n, int(path[r]), rs[r]["pairs"], pairs)
