"""Bonded terms on the GPU (mdrl_set_bonded) against the FP64 oracle (oracle/bonded.cpp).

* Bonded-only forces (zero LJ, no charges) of chain molecules straddling the periodic box, for
  every accumulation mode: max |dF| / rms |F| <= 2e-5 (FP32 terms against FP64), energies within
  2e-5 relative.
* With pair forces on: the forces are the pair path's plus the bonded terms' (the same
  accumulators), within the sum of both tolerances.
* MD: total energy (kinetic + pair + bonded) is conserved over 2,000 velocity-Verlet steps.
* Terms set after mdrl_set_state re-capture the step graphs; removing them restores the pair-only
  forces; atom indices beyond the particles and bad periodicities are refused.
"""
import dataclasses

import numpy as np
import pytest

import oracle
import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems
from helpers import oracle_from_ctx

pytestmark = pytest.mark.gpu

TOL = 2e-5


def _system(seed=11, noise=0.08):
    sysm, T = systems.chains(40, 30, 40.0, seed=seed)
    rng = np.random.default_rng(seed)
    pos = systems.wrap_into_box(sysm.pos.astype(np.float64) + rng.normal(0, noise, sysm.pos.shape), sysm.box)
    sysm.pos = pos
    return sysm, T


def _err(F, Fo):
    d = np.linalg.norm(F - Fo, axis=1)
    return d.max() / np.sqrt((np.linalg.norm(Fo, axis=1) ** 2).mean())


@pytest.mark.parametrize("accum", [m.ACC_FIXED64, m.ACC_FP32_ATOMIC, m.ACC_KAHAN])
def test_bonded_only_matches_oracle(accum):
    sysm, T = _system()
    p = dataclasses.replace(sysm, epsilon=[0.0]).params(accum=accum, flags=m.FLAG_ENERGY)
    with m.Context(p) as ctx:
        ctx.set_bonded(**T)
        assert ctx.bonded_counts() == tuple(len(v[0]) for v in (T["bonds"], T["angles"], T["dihedrals"]))
        F, st, _ = ctx.force(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], None, sysm.type)
    Fo, Eo = oracle.bonded64(sysm.pos.astype(np.float64), sysm.box, **T)
    assert np.abs(Fo).max() > 10.0
    assert _err(F, Fo) <= TOL, _err(F, Fo)
    assert st["e_lj"] == 0.0
    for key, name in (("e_bond", "bond"), ("e_angle", "angle"), ("e_dihedral", "dihedral")):
        assert abs(st[key] - Eo[name]) <= TOL * max(abs(Eo[name]), 1.0), (key, st[key], Eo[name])


def test_bonded_plus_pairs():
    sysm, T = _system(seed=12)
    p = sysm.params(table_bins=512, flags=m.FLAG_ENERGY)
    x, y, z = (np.ascontiguousarray(sysm.pos[:, k]) for k in range(3))
    with m.Context(p) as ctx:
        Fp, stp, _ = ctx.force(x, y, z, None, sysm.type)
        ctx.set_bonded(**T)
        Fb, stb, _ = ctx.force(x, y, z, None, sysm.type)
        o = oracle_from_ctx(ctx, sysm)
        ctx.set_bonded()                                   # removed: the pair forces again
        assert ctx.bonded_counts() == (0, 0, 0)
        Fp2, stp2, _ = ctx.force(x, y, z, None, sysm.type)
    assert np.array_equal(Fp.view(np.uint32), Fp2.view(np.uint32))
    assert stp2["e_bond"] == 0.0 and stp2["e_dihedral"] == 0.0
    assert stb["pairs"] == stp["pairs"] and stb["e_lj"] == stp["e_lj"]
    Fo_pair, Fabs, _, _ = o.force_cells()
    Fo_b, Eo = oracle.bonded64(sysm.pos.astype(np.float64), sysm.box, **T)
    rms = np.sqrt((np.linalg.norm(Fo_pair + Fo_b, axis=1) ** 2).mean())
    d = np.linalg.norm(Fb - (Fo_pair + Fo_b), axis=1).max()
    assert d <= TOL * rms + 2e-6 * np.abs(Fabs).max(), (d, rms)
    assert stb["e_angle"] == pytest.approx(Eo["angle"], rel=TOL, abs=TOL)


def test_md_with_bonded_terms_conserves_energy():
    sysm, T = systems.chains(40, 30, 40.0, seed=13)
    p = sysm.params(table_bins=1024, table_order=2, dt_fs=0.5, flags=m.FLAG_ENERGY)
    with m.Context(p) as ctx:
        ctx.set_bonded(**T)
        ctx.set_state(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, None, sysm.type)
        etot = []
        for _ in range(20):
            st = ctx.step(100)
            etot.append(st["kinetic"] + st["e_lj"] + st["e_bond"] + st["e_angle"] + st["e_dihedral"])
        assert st["e_bond"] > 0 and st["e_angle"] > 0 and st["e_dihedral"] > 0
    etot = np.array(etot)
    ke_scale = 1.5 * sysm.n * systems.KB_KCAL * 300.0
    assert np.abs(etot - etot[0]).max() <= 0.02 * ke_scale, (etot - etot[0]).tolist()


def test_terms_set_after_state_take_effect_in_steps():
    sysm, T = _system(seed=14)
    p = dataclasses.replace(sysm, epsilon=[0.0]).params(flags=m.FLAG_ENERGY)
    args = (sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, None, sysm.type)
    with m.Context(p) as ctx:
        ctx.set_state(*args)
        ctx.step(2)                                        # graphs captured without terms
        ctx.set_state(*args)
        ctx.set_bonded(**T)
        st = ctx.step(1)
        assert st["e_bond"] > 0
        s1 = ctx.state()
    with m.Context(p) as ctx:
        ctx.set_bonded(**T)
        ctx.set_state(*args)
        ctx.step(1)
        s2 = ctx.state()
    # set_state evaluated the first forces without the terms in the first context
    assert not np.array_equal(s1[1], s2[1])
    with m.Context(p) as ctx:
        ctx.set_bonded(**T)
        ctx.set_state(*args)
        ctx.step(1)
        s3 = ctx.state()
    for a, b in zip(s2, s3):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_bad_terms_are_refused():
    sysm, T = _system(seed=15)
    p = dataclasses.replace(sysm, epsilon=[0.0]).params()
    with m.Context(p) as ctx:
        ctx.set_bonded(bonds=(np.array([[0, sysm.n]]), np.array([[1.0, 1.0]])))
        with pytest.raises(m.MdrlError) as e:
            ctx.force(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2])
        assert "bonded" in str(e.value)
        with pytest.raises(m.MdrlError):
            ctx.set_bonded(dihedrals=(np.array([[0, 1, 2, 3]]), np.array([[1.0, 2.5, 0.0]])))
        with pytest.raises(m.MdrlError):
            ctx.set_bonded(bonds=(np.array([[0, -1]]), np.array([[1.0, 1.0]])))
        with pytest.raises(m.MdrlError):
            ctx.set_bonded(bonds=(np.array([[0, 1]]), np.array([[np.nan, 1.0]])))


def test_dhfr_bonded_matches_oracle():
    """The reference's DHFR dataset (23,558 atoms; 23,592 bonds, 4,561 angles, 8,166 dihedrals
    from its Amber topology) through the GPU bonded path, pair forces off."""
    from helpers import dhfr_bonded
    pos, box, T = dhfr_bonded()
    n = len(pos)
    p = m.default_params(box=box, cutoff=8.0, ncell=(7, 7, 7), sigma=[1.0], epsilon=[0.0], mass=[12.0],
                         flags=m.FLAG_ENERGY)
    with m.Context(p) as ctx:
        ctx.set_bonded(**T)
        F, st, _ = ctx.force(pos[:, 0], pos[:, 1], pos[:, 2])
    # the library holds the box edge in FP32 (62.23 -> 62.2299995...): the oracle takes the same
    # edge, or a bond across the boundary differs by 2 k x 1.9e-6 A before any arithmetic
    box32 = tuple(float(np.float32(b)) for b in box)
    Fo, Eo = oracle.bonded64(pos.astype(np.float64), box32, **T)
    assert _err(F, Fo) <= TOL, _err(F, Fo)
    for key, name in (("e_bond", "bond"), ("e_angle", "angle"), ("e_dihedral", "dihedral")):
        assert abs(st[key] - Eo[name]) <= TOL * abs(Eo[name]), (key, st[key], Eo[name])
    assert n == 23558
