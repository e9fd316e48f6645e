"""Synthetic workload generators (CPU only)."""
import numpy as np
import pytest
from scipy.spatial import cKDTree

from sc2019_md_gb300 import systems


def test_ljc92k_shape_density_and_separation():
    s = systems.ljc92k()
    assert s.n == 92224 and s.ncell == (9, 9, 6)
    vol = np.prod(s.box)
    assert abs(s.n / vol - 0.1) < 1e-3
    assert (s.pos >= 0).all() and (s.pos < np.asarray(s.box, np.float32)).all()
    tree = cKDTree(s.pos.astype(np.float64), boxsize=np.asarray(s.box))
    assert len(tree.query_pairs(0.999)) == 0
    assert abs(float(s.q.astype(np.float64).sum())) < 1e-6
    assert set(np.unique(s.type)) == {0, 1, 2, 3}
    s2 = systems.ljc92k()
    assert np.array_equal(s.pos, s2.pos)


def test_lj1728_lattice():
    s = systems.lj1728()
    assert s.n == 1728 and s.ncell == (3, 3, 3)
    v = s.vel.astype(np.float64)
    assert np.abs(v.sum(0)).max() < 1e-5
    t = (39.95 * (v ** 2).sum() / systems.KCAL_PER_AMU_A2_FS2 * 0 + 1)
    assert t == 1
    ke = 0.5 * 39.95 * (v ** 2).sum() * systems.KCAL_PER_AMU_A2_FS2
    temp = 2 * ke / (3 * s.n * systems.KB_KCAL)
    assert 250 < temp < 350


def test_wrap_into_box():
    p = np.array([[-0.1, 10.0, 25.5], [25.499, 0.0, 30.0]])
    w = systems.wrap_into_box(p, (25.5, 25.5, 25.5))
    assert (w >= 0).all() and (w < np.float32(25.5)).all()
