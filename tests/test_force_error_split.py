"""Where the force error against the FP64 oracle comes from (CPU, oracle only).

The primary norm is max_i |dF_i| / rms_j |F_j| against FP64 direct evaluation with exact
differences (orc_force_direct64).  The error of the FP32 datapath splits into three parts, each
measured alone with the others in FP64 (orc_force_split64):

* difference rounding: FP64 physics on the datapath's rounded differences;
* table interpolation: the FP32 tables evaluated in FP64 at the exact r2;
* FP32 evaluation: the datapath (orc_force_cells: the exact sum of the FP32 pair forces) against
  FP64 evaluation of the same tables on the same rounded differences.

Measured (printed by the tests below):

* With the reference's difference rule, d = fl(fl(xi - xj) -+ L) (SC/r2_compute_with_pbc.v:81-127),
  the difference rounding alone exceeds 1e-5 on both systems (1.07e-5 on the 1,728-atom cube,
  3.7e-4 on the 92k system): a pair across the boundary first rounds the difference of two
  far-apart coordinates, an absolute error up to ulp(L)/2 that r^-14 amplifies 14-fold, and on
  the 92k system the largest forces are ~40x the rms.  No table or evaluation choice can undo it.
* With the exact-difference rule (MDRL_FLAG_EXACT_DIFF) and bin-local order-2 tables the total is
  within 1e-5 on both systems; what remains is the FP32 evaluation (~8e-6 on the 92k system).
* Monomial order-1 tables leave a table error of 3.2e-4 (512 bins) on the 92k system.
"""
import numpy as np
import pytest

import oracle
from sc2019_md_gb300 import systems


def _oracle(s, order, bins, exact):
    m0 = s.table_min_log2
    rc2 = np.float32(np.float32(s.cutoff) * np.float32(s.cutoff))
    nseg = int(np.floor(np.log2(rc2))) - m0 + 1
    local = order >= 2
    pc64 = oracle.lb_coefficients(s.sigma, s.epsilon)
    return oracle.System(s.pos, s.box, s.ncell, s.cutoff, pc64.astype(np.float32), q=s.q, type=s.type,
                         ke=s.coulomb_k, tab=oracle.fit_tables(order, nseg, bins, m0, local=local), order=order,
                         nseg=nseg, bins=bins, min_log2=m0, pcoef64=pc64, ke64=s.coulomb_k, local=local,
                         exact=exact)


def _max_over_rms(F, R):
    d = np.linalg.norm(F - R, axis=1)
    return float(d.max() / np.sqrt((np.linalg.norm(R, axis=1) ** 2).mean()))


def split(s, order, bins, exact):
    o = _oracle(s, order, bins, exact)
    F64, _ = o.force_direct64()
    F32, _, _, st = o.force_cells()
    out = {"total": _max_over_rms(F32, F64),
           "difference rounding": _max_over_rms(o.force_split64(1, False)[0], F64),
           "table interpolation": _max_over_rms(o.force_split64(0, True)[0], F64),
           "FP32 evaluation": _max_over_rms(F32, o.force_split64(1, True)[0]),
           "pairs": st["pairs"]}
    print(f"{s.name} order {order} bins {bins} {'exact' if exact else 'reference'} differences: "
          + ", ".join(f"{k} {v:.3e}" if k != "pairs" else f"{k} {v}" for k, v in out.items()))
    return out


def test_split_lj1728():
    s = systems.lj1728()
    ref = split(s, 1, 1024, False)
    assert ref["difference rounding"] > 1e-5          # the reference's rule alone breaks the bound
    best = split(s, 2, 512, True)
    assert best["total"] <= 1e-5
    assert best["difference rounding"] < 0.3 * ref["difference rounding"]
    assert best["table interpolation"] < 1e-6         # bin-local order 2: no cancellation floor
    assert best["pairs"] == ref["pairs"]


def test_split_ljc92k():
    s = systems.ljc92k()
    ref = split(s, 1, 512, False)
    assert ref["difference rounding"] > 1e-4
    assert ref["table interpolation"] > 1e-4
    best = split(s, 2, 512, True)
    assert best["total"] <= 1e-5
    assert best["FP32 evaluation"] > best["table interpolation"]   # what remains is FP32 arithmetic
    assert best["pairs"] == ref["pairs"]
