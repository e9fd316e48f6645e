"""The oracle's all-image pair rule (boxes with edge in (rc, 3 rc), where the half shell does not
apply), pinned two ways (CPU only):

* where the half shell does apply (3 cells of edge >= rc per axis, so edge >= 2 rc), the
  all-image pair set equals the half-shell oracle's (the reference's traversal) pair for pair;
* for a box below 2 rc, an independent pure-Python loop over all 27 image shifts, with every
  FP32 operation rounded by numpy, gives the same pairs and per-particle counts.
"""
import numpy as np

import oracle
from sc2019_md_gb300 import systems

F32 = np.float32


def _oracle_system(s, eval_mode=0, bins=256, min_log2=-2):
    rcf = F32(s.cutoff)
    rc2 = F32(rcf * rcf)
    nseg = int(np.floor(np.log2(float(rc2)))) - min_log2 + 1
    tab = oracle.fit_tables(1, nseg, bins, min_log2)
    pc64 = oracle.lb_coefficients(s.sigma, s.epsilon)
    return oracle.System(s.pos, s.box, s.ncell, s.cutoff, pc64.astype(np.float32), q=s.q, type=s.type,
                         ke=s.coulomb_k, tab=tab, order=1, nseg=nseg, bins=bins, min_log2=min_log2,
                         eval=eval_mode, arith=0, pcoef64=pc64, ke64=s.coulomb_k)


def test_allimage_equals_halfshell_where_cells_apply():
    s = systems.small_ljc(2979, 31.0, 10.0, seed=11)     # 3 x 3 x 3 cells of 10.33 A
    assert s.ncell == (3, 3, 3)
    o = _oracle_system(s)
    F_hs, _, cnt_hs, st_hs = o.force_cells()
    F_tab, _ = o.force_tables64()
    F_ai, F32_ai, A_ai, cnt_ai, st_ai = o.force_allimage()
    assert st_ai["pairs"] == st_hs["pairs"] > 0
    assert np.array_equal(cnt_ai, cnt_hs)
    scale = np.sqrt((np.linalg.norm(F_tab, axis=1) ** 2).mean())
    assert np.abs(F_ai - F_tab).max() <= 1e-9 * scale
    assert abs(st_ai["e_lj"] - st_hs["e_lj"]) <= 1e-4 * abs(st_hs["e_lj"])
    # the ordered-pair FP32 sums equal the half-shell sums of the same FP32 pair forces up to
    # the rounding of QQ = (ke*qi)*qj on the two sides of a pair
    assert np.all(np.abs(F32_ai - F_hs) <= 1e-6 * A_ai + 1e-9)


def _bruteforce_pairs(pos, box, rc2):
    n = len(pos)
    L = [F32(b) for b in box]
    cnt = np.zeros(n, np.int64)
    pairs = 0
    for i in range(n):
        for j in range(i + 1, n):
            d0 = [F32(pos[i, a]) - F32(pos[j, a]) for a in range(3)]
            for kx in (-1, 0, 1):
                for ky in (-1, 0, 1):
                    for kz in (-1, 0, 1):
                        d = [d0[0] + F32(kx) * L[0], d0[1] + F32(ky) * L[1], d0[2] + F32(kz) * L[2]]
                        r2 = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]
                        if F32(0) < r2 <= rc2:
                            pairs += 1
                            cnt[i] += 1
                            cnt[j] += 1
    return pairs, cnt


def test_allimage_bruteforce_small_box():
    s = systems.small_ljc(60, 13.0, 10.0, seed=5, dmin=1.5)   # edge 13 < 2 rc: up to 8 images a pair
    o = _oracle_system(s)
    _, _, _, cnt, st = o.force_allimage()
    rcf = F32(s.cutoff)
    pairs, cnt_bf = _bruteforce_pairs(s.pos, s.box, F32(rcf * rcf))
    assert st["pairs"] == pairs
    assert np.array_equal(cnt, cnt_bf)
    # more than one image of some pairs is within rc, and every particle has more
    # neighbours than the 59 other particles
    assert pairs > 60 * 59 // 2
    assert cnt.min() > 59


def test_allimage_direct_forces_sum_to_zero():
    """Each pair adds equal and opposite FP64 forces, so the total force vanishes."""
    s = systems.small_ljc(200, 15.0, 10.0, seed=9)
    o = _oracle_system(s, eval_mode=1)
    F, _, _, _, st = o.force_allimage()
    assert st["pairs"] > 0
    scale = np.abs(F).max()
    assert np.abs(F.sum(0)).max() <= 1e-9 * scale * len(F)
