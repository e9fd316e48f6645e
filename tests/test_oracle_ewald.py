"""The FP64 Ewald oracle pinned (CPU only): the rock-salt Madelung constant (1.747564594633...)
and the independence of the Ewald energy and forces from the splitting parameter beta."""
import numpy as np

import oracle
from sc2019_md_gb300 import systems

MADELUNG_NACL = 1.7475645946331822


def test_rock_salt_madelung_constant():
    n, r0 = 4, 2.0
    g = np.arange(n) * r0
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    idx = np.stack(np.meshgrid(*(np.arange(n),) * 3, indexing="ij"), -1).reshape(-1, 3)
    q = np.where(idx.sum(1) % 2 == 0, 1.0, -1.0).astype(np.float32)
    L = n * r0
    for beta in (1.2, 1.6, 2.0):
        s = oracle.System(pos, (L, L, L), (1, 1, 1), L / 2, np.zeros((1, 4), np.float32), q=q, ke=1.0, ke64=1.0)
        F, e = s.ewald64(beta, 24)
        M = -e["total"] / (len(q) / 2) * r0
        assert abs(M - MADELUNG_NACL) < 1e-9, (beta, M)
        assert np.abs(F).max() < 1e-9          # every ion sits at a centre of symmetry


def test_ewald_independent_of_beta():
    s0 = systems.small_ljc(300, 18.0, 9.0, seed=4, ntypes=1, dmin=1.5)
    o = oracle.System(s0.pos, s0.box, s0.ncell, 9.0, np.zeros((1, 4), np.float32), q=s0.q, ke=332.0637,
                      ke64=332.0637)
    # both betas leave erfc(beta rc) <= 1e-8, so the real-space cutoff error is negligible
    res = [o.ewald64(beta, int(np.ceil(1.6 * 18.0 * beta)) + 2) for beta in (0.45, 0.55)]
    (F1, e1), (F2, e2) = res
    assert abs(e1["total"] - e2["total"]) <= 1e-7 * abs(e1["total"])
    scale = np.sqrt((F1 ** 2).sum(1).mean())
    assert np.abs(F1 - F2).max() <= 1e-5 * scale
