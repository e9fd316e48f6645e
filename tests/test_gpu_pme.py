"""Smooth-PME long-range electrostatics on the GPU against the FP64 Ewald oracle.

The oracle (orc_ewald64) is pinned by the rock-salt Madelung constant and by the independence of
the Ewald energy from beta (tests/test_oracle_ewald.py).  Here the GPU's real-space tables plus
its PME reciprocal part are compared with the oracle's converged Ewald forces and energy on a
pure-Coulomb system; the error must fall with the B-spline order and the grid; results are
bit-reproducible; switching PME off restores the truncated path bit for bit; a charged LJ liquid
conserves energy.
"""
import numpy as np
import pytest

import oracle
import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems

pytestmark = pytest.mark.gpu

KE = systems.COULOMB_K


def _coulomb_system(n=2000, L=30.0, seed=41):
    s = systems.small_ljc(n, L, 10.0, seed=seed, ntypes=1, dmin=1.5)
    return s


def _params(s, **kw):
    kw.setdefault("table_bins", 1024)
    p = m.default_params(box=s.box, cutoff=s.cutoff, ntypes=1, sigma=[3.0], epsilon=[0.0], mass=[20.0],
                         coulomb_k=KE, flags=m.FLAG_ENERGY, **kw)
    return p


def _ewald(s, beta):
    L = s.box[0]
    nmax = int(np.ceil(1.55 * L * beta)) + 1
    o = oracle.System(s.pos, s.box, s.ncell, s.cutoff, np.zeros((1, 4), np.float32), q=s.q, ke=KE, ke64=KE)
    return o.ewald64(beta, nmax)


def _err(F, Fref):
    return float(np.sqrt(((F - Fref) ** 2).sum(1).mean() / (Fref ** 2).sum(1).mean()))


@pytest.fixture(scope="module")
def case():
    s = _coulomb_system()
    out = {}
    for name, kw in (("order4", {}), ("order6", {"order": 6}), ("fine", {"order": 6, "spacing": 0.6})):
        with m.Context(_params(s)) as ctx:
            r = ctx.set_pme(**kw)
            F, st, _ = ctx.force(s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.q, s.type)
            F2, _, _ = ctx.force(s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.q, s.type)
        out[name] = (r, F, F2, st)
    beta = out["order4"][0]["beta"]
    Fe, e = _ewald(s, beta)
    return s, out, Fe, e


def test_pme_matches_ewald_oracle(case):
    s, out, Fe, e = case
    r, F, F2, st = out["order4"]
    assert abs(r["beta"] * s.cutoff - 3.123) < 0.01          # erfc(beta rc) = 1e-5
    assert all(k >= 30 for k in r["grid"])
    err = _err(F, Fe)
    print("order 4 rms force error", err, "energy", st["e_coul"], e["total"])
    assert err < 1e-3
    assert abs(st["e_coul"] - e["total"]) <= 2e-3 * abs(e["total"])     # order 4 at 1 A spacing
    assert np.array_equal(F.view(np.uint32), F2.view(np.uint32))


def test_pme_error_falls_with_order_and_grid(case):
    s, out, Fe, e = case
    e4, e6, ef = (_err(out[k][1], Fe) for k in ("order4", "order6", "fine"))
    print("rms force errors", e4, e6, ef)
    assert e6 < e4 and ef < e6
    assert ef < 2e-4
    assert abs(out["fine"][3]["e_coul"] - e["total"]) <= 2e-5 * abs(e["total"])


def test_pme_off_restores_truncated_path():
    s = _coulomb_system(1500, 31.0, 3)
    p = _params(s)
    args = (s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.q, s.type)
    with m.Context(p) as ctx:
        F0, st0, _ = ctx.force(*args)
    with m.Context(p) as ctx:
        ctx.set_pme()
        ctx.force(*args)
        assert ctx.pme()
        ctx.set_pme(False)
        assert ctx.pme() == {}
        F1, st1, _ = ctx.force(*args)
    assert np.array_equal(F0.view(np.uint32), F1.view(np.uint32))
    assert st0["e_coul"] == st1["e_coul"]


def test_pme_md_energy_conservation():
    """A charged LJ liquid (argon-like, 0.021 /A^3, +-0.3 e on alternate lattice sites, 120 K,
    rc 10 A, PME order 4): after 300 fs of melting, the total energy drifts by less than 1e-2 of
    the kinetic energy over 400 steps of 1 fs.  (While the lattice melts, pairs cross into the
    unshifted LJ cutoff and the total energy moves by V(rc) per crossing, ~2 kcal/mol in all,
    the same with PME order 4 or 6, dt 1 or 0.5 fs and without charges; truncated Coulomb instead
    of PME jumps by 1e3 kcal/mol.)"""
    rng = np.random.default_rng(5)
    nside = 10
    L = nside * (1.0 / 0.021) ** (1.0 / 3.0)
    g = (np.arange(nside) + 0.5) * (L / nside)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) + rng.uniform(-0.05, 0.05, (nside ** 3, 3))
    pos = systems.wrap_into_box(pos, (L, L, L))
    idx = np.stack(np.meshgrid(*(np.arange(nside),) * 3, indexing="ij"), -1).reshape(-1, 3)
    q = np.where(idx.sum(1) % 2 == 0, 0.3, -0.3).astype(np.float32)
    vel = systems.maxwell(len(pos), np.full(len(pos), 39.95), 120.0, rng)
    p = m.default_params(box=(L, L, L), cutoff=10.0, ntypes=1, sigma=[3.4], epsilon=[0.238], mass=[39.95],
                         coulomb_k=KE, table_bins=1024, table_order=2, dt_fs=1.0, flags=m.FLAG_ENERGY)
    with m.Context(p) as ctx:
        ctx.set_pme()
        ctx.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, q, np.zeros(len(pos), np.int32))
        ctx.step(300)
        e = []
        for _ in range(8):
            st = ctx.step(50)
            e.append((st["e_lj"] + st["e_coul"], st["kinetic"]))
    e = np.asarray(e)
    tot = e[:, 0] + e[:, 1]
    assert np.isfinite(tot).all()
    drift = np.abs(tot - tot[0]).max()
    print("drift", drift, "kinetic", e[:, 1].mean())
    assert drift < 1e-2 * e[:, 1].mean()


def test_pme_validation():
    s = _coulomb_system(500, 20.0, 2)
    with m.Context(_params(s)) as ctx:
        with pytest.raises(m.MdrlError):
            ctx.set_pme(order=5)
        with pytest.raises(m.MdrlError):
            ctx.set_pme(grid=(4, 4, 4))
    p = _params(s)
    p.coulomb_k = 0.0
    with m.Context(p) as ctx:
        with pytest.raises(m.MdrlError):
            ctx.set_pme()
