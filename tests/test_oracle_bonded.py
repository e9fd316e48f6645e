"""The bonded-term oracle (oracle/bonded.cpp) on the CPU: forces are minus the gradient of the
energy (central differences), the net force and torque of every term vanish, closed-form cases,
the IUPAC dihedral sign, periodic wrapping, and argument checks."""
import numpy as np
import pytest

import oracle
from sc2019_md_gb300 import systems


def _chain_terms(rng, n=7):
    pos = np.cumsum(rng.normal(0, 0.6, (n, 3)) + np.array([1.3, 0.4, 0.2]), 0)
    bonds = (np.array([[k, k + 1] for k in range(n - 1)]), np.column_stack([rng.uniform(100, 400, n - 1),
                                                                            rng.uniform(1.0, 1.6, n - 1)]))
    angles = (np.array([[k, k + 1, k + 2] for k in range(n - 2)]),
              np.column_stack([rng.uniform(20, 80, n - 2), rng.uniform(1.7, 2.1, n - 2),
                               rng.choice([0.0, 15.0], n - 2), rng.uniform(2.2, 2.6, n - 2)]))
    dat = np.array([[k, k + 1, k + 2, k + 3] for k in range(n - 3)] * 2)
    dpar = np.column_stack([rng.uniform(0.2, 2.0, len(dat)), rng.integers(0, 5, len(dat)),
                            rng.uniform(-np.pi, np.pi, len(dat))])
    return pos, bonds, angles, (dat, dpar)


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_forces_are_minus_energy_gradient(seed):
    rng = np.random.default_rng(seed)
    pos, b, a, d = _chain_terms(rng)
    F, E = oracle.bonded64(pos, None, b, a, d)
    etot = lambda p: sum(oracle.bonded64(p, None, b, a, d)[1].values())
    h = 1e-6
    num = np.zeros_like(pos)
    for i in range(len(pos)):
        for k in range(3):
            pp, pm = pos.copy(), pos.copy()
            pp[i, k] += h
            pm[i, k] -= h
            num[i, k] = -(etot(pp) - etot(pm)) / (2 * h)
    assert np.abs(F - num).max() <= 1e-6 * max(1.0, np.abs(F).max())
    assert np.abs(F.sum(0)).max() <= 1e-10 * np.abs(F).max()
    assert np.abs(np.cross(pos, F).sum(0)).max() <= 1e-9 * np.abs(F).max() * np.abs(pos).max()


def test_closed_forms():
    # bond stretched 0.1 A past r0 = 1.5: E = k * 0.01, |F| = 2 k 0.1 along the bond
    F, E = oracle.bonded64([[0, 0, 0], [1.6, 0, 0]], None, ([[0, 1]], [[250.0, 1.5]]))
    assert E["bond"] == pytest.approx(2.5)
    assert F[0] == pytest.approx([50.0, 0, 0]) and F[1] == pytest.approx([-50.0, 0, 0])
    # right angle at theta0 = pi/2: no angle energy or force; Urey-Bradley at s0 = sqrt(2)
    pos = [[1, 0, 0], [0, 0, 0], [0, 1, 0]]
    F, E = oracle.bonded64(pos, None, angles=([[0, 1, 2]], [[50.0, np.pi / 2, 10.0, np.sqrt(2)]]))
    assert E["angle"] == pytest.approx(0.0, abs=1e-20) and np.abs(F).max() < 1e-12
    # 120 degrees against theta0 = 90: E = k (pi/6)^2
    pos = [[1, 0, 0], [0, 0, 0], [np.cos(2 * np.pi / 3), np.sin(2 * np.pi / 3), 0]]
    F, E = oracle.bonded64(pos, None, angles=([[0, 1, 2]], [[50.0, np.pi / 2, 0.0, 0.0]]))
    assert E["angle"] == pytest.approx(50.0 * (np.pi / 6) ** 2)
    # dihedral: trans has E = 0 for n = 3, delta = 0; gauche+ is +60 degrees (IUPAC)
    trans = [[1, 0, 0], [0, 0, 0], [0, 0, 1], [-1, 0, 1]]
    F, E = oracle.bonded64(trans, None, dihedrals=([[0, 1, 2, 3]], [[2.0, 3, 0.0]]))
    assert E["dihedral"] == pytest.approx(0.0, abs=1e-12)
    gauche = [[1, 0, 0], [0, 0, 0], [0, 0, 1], [0.5, np.sqrt(3) / 2, 1]]
    F, E = oracle.bonded64(gauche, None, dihedrals=([[0, 1, 2, 3]], [[1.0, 1, np.pi / 2]]))
    assert E["dihedral"] == pytest.approx(1.0 - np.sin(np.pi / 3))
    # harmonic (n = 0) with the difference wrapped: phi = 60, delta = -170 degrees -> diff = -130
    F, E = oracle.bonded64(gauche, None, dihedrals=([[0, 1, 2, 3]], [[1.0, 0, np.deg2rad(-170.0)]]))
    assert E["dihedral"] == pytest.approx(np.deg2rad(-130.0) ** 2)


def test_periodic_wrap_equals_unwrapped_chain():
    sysm, T = systems.chains(6, 12, 18.0, seed=5, cutoff=6.0)
    rng = np.random.default_rng(2)
    pos = sysm.pos.astype(np.float64) + rng.normal(0, 0.05, sysm.pos.shape)
    pos = np.mod(pos, 18.0)
    F, E = oracle.bonded64(pos, sysm.box, **T)
    # unwrap each chain along its bonds, then evaluate without a box
    un = pos.copy()
    for c in range(6):
        for k in range(1, 12):
            i = c * 12 + k
            d = un[i] - un[i - 1]
            un[i] -= 18.0 * np.round(d / 18.0)
    F2, E2 = oracle.bonded64(un, None, **T)
    assert np.abs(F - F2).max() <= 1e-9 * np.abs(F).max()
    for k in E:
        assert E[k] == pytest.approx(E2[k], rel=1e-12, abs=1e-12)
    assert (pos.min(0) < 1.0).all() and (pos.max(0) > 17.0).all()     # chains do straddle the box


def test_bad_arguments():
    with pytest.raises(ValueError):
        oracle.bonded64([[0, 0, 0], [1, 0, 0]], None, ([[0, 2]], [[1.0, 1.0]]))
    with pytest.raises(ValueError):
        oracle.bonded64([[0, 0, 0], [1, 0, 0]], None, ([[-1, 0]], [[1.0, 1.0]]))


def test_dhfr_bonded_terms():
    """The DHFR topology's 36,319 bonded terms on its own coordinates: finite energies of the
    equilibrated structure, zero net force, and forces equal to minus the energy gradient for a
    sample of atoms."""
    from helpers import dhfr_bonded
    pos, box, T = dhfr_bonded()
    p64 = pos.astype(np.float64)
    F, E = oracle.bonded64(p64, box, **T)
    assert all(np.isfinite(v) and v > 0 for v in E.values())
    assert np.abs(F.sum(0)).max() <= 1e-9 * np.abs(F).max() * len(F)
    rng = np.random.default_rng(0)
    h = 1e-5
    for i in rng.choice(2489, 8, replace=False):       # protein atoms (all three kinds of terms)
        for k in range(3):
            pp, pm = p64.copy(), p64.copy()
            pp[i, k] += h
            pm[i, k] -= h
            num = -(sum(oracle.bonded64(pp, box, **T)[1].values()) - sum(oracle.bonded64(pm, box, **T)[1].values())) / (2 * h)
            assert abs(F[i, k] - num) <= 1e-4 * max(1.0, abs(F[i, k])), (i, k, F[i, k], num)
