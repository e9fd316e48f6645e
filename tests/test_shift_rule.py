"""The force kernel's per-unit periodic shift against the reference's per-pair wrap (CPU, numpy).

The reference wraps each pair difference once: d = fl(xi - xj), then d - L if d > L/2 and d + L
if d < -L/2 (Range_Limited_demo/SourceCode/r2_compute_with_pbc.v:81-127).  A half-shell unit of
the GPU kernel instead adds one -L/0/+L per axis, chosen by whether the neighbour cell lies across
the box boundary: d = fl(fl(xi - xj) + s).  With at least 3 cells of edge >= rc per axis the two
rules must accept the same pairs (0 < r2 <= rc2, r2 = fl(fl(dx^2 + dy^2) + dz^2)) with the same
difference bits; with 2 cells, where the half shell is not used, they must not.

The exact-difference rule (MDRL_FLAG_EXACT_DIFF) is checked the same way: per pair, the wrap
direction from fl(xi - xj), then the box edge off the high coordinate, d = fl(fl(xi - L) - xj) or
fl(xi - fl(xj - L)); per unit, the kernel's staging takes the edge off the home particles (unit
across the +L face) or off the neighbour's (across the -L face) and subtracts once.  Both must
accept the same pairs with the same bits, and d must be the exact minimum-image difference
rounded once.
"""
import numpy as np
import pytest

f32 = np.float32
HALF_SHELL = [(0, 0, 0), (0, 0, 1), (0, 1, -1), (0, 1, 0), (0, 1, 1), (1, -1, -1), (1, -1, 0), (1, -1, 1),
              (1, 0, -1), (1, 0, 0), (1, 0, 1), (1, 1, -1), (1, 1, 0), (1, 1, 1)]


def _r2(d):
    q = (d * d).astype(f32)
    return ((q[:, 0] + q[:, 1]).astype(f32) + q[:, 2]).astype(f32)


def _compare(L, rc, n, seed, rule="reference"):
    """(pairs accepted by the per-pair wrap, pairs whose decision or difference bits differ, cells)."""
    rng = np.random.default_rng(seed)
    Lf = f32(L)
    h = Lf / f32(2)
    nc = int(np.floor(Lf / f32(rc)))
    e = Lf / f32(nc)
    P = (rng.random((n, 3)) * L).astype(f32)
    P = np.minimum(P, np.nextafter(Lf, f32(0)))
    # a fifth of the particles on cell and box faces, where the two rules are most likely to split
    k = n // 5
    P[np.arange(k), rng.integers(0, 3, k)] = rng.choice(
        [f32(0), np.nextafter(Lf, f32(0)), e, np.nextafter(e, f32(0)), f32(2) * e], k)
    c3 = np.minimum(np.floor(P / e).astype(int), nc - 1)
    rc2 = f32(rc) * f32(rc)
    cells = {}
    for idx, c in enumerate(map(tuple, c3)):
        cells.setdefault(c, []).append(idx)
    accepted = differ = 0
    for hc, hi in cells.items():
        hi = np.asarray(hi)
        for f, off in enumerate(HALF_SHELL):
            raw = np.asarray(hc) + np.asarray(off)
            s = np.where(raw >= nc, -Lf, np.where(raw < 0, Lf, f32(0))).astype(f32)
            cc = tuple(raw % nc)
            if cc not in cells:
                continue
            I, J = np.meshgrid(hi, np.asarray(cells[cc]), indexing="ij")
            I, J = I.ravel(), J.ravel()
            if f == 0:
                keep = I < J
                I, J = I[keep], J[keep]
            d0 = (P[I] - P[J]).astype(f32)
            if rule == "reference":
                dw = np.where(d0 > h, (d0 - Lf).astype(f32), np.where(d0 < -h, (d0 + Lf).astype(f32), d0)).astype(f32)
                ds = (d0 + s).astype(f32)
            else:
                xi, xj = P[I], P[J]
                dw = np.where(d0 > h, ((xi - Lf).astype(f32) - xj).astype(f32),
                              np.where(d0 < -h, (xi - (xj - Lf).astype(f32)).astype(f32), d0)).astype(f32)
                si = np.where(s < 0, s, f32(0)).astype(f32)       # edge off the home particle
                sj = np.where(s > 0, s, f32(0)).astype(f32)       # edge off the neighbour
                xi2, xj2 = (xi + si).astype(f32), (xj - sj).astype(f32)
                # the staging shifts are exact (Sterbenz: the shifted coordinate is above L/2)
                assert np.array_equal(xi2.astype(np.float64), xi.astype(np.float64) + si)
                assert np.array_equal(xj2.astype(np.float64), xj.astype(np.float64) - sj)
                ds = (xi2 - xj2).astype(f32)
                # one rounding of the exact minimum-image difference
                exact = xi2.astype(np.float64) - xj2.astype(np.float64)
                assert np.array_equal(ds, exact.astype(f32))
            rw, rs = _r2(dw), _r2(ds)
            aw = (rw > 0) & (rw <= rc2)
            as_ = (rs > 0) & (rs <= rc2)
            both = aw & as_
            differ += int(np.sum(aw != as_))
            differ += int(np.sum(np.any(dw[both].view(np.uint32) != ds[both].view(np.uint32), axis=1)))
            accepted += int(aw.sum())
    return accepted, differ, nc


@pytest.mark.parametrize("L,rc,seed", [(30.0, 10.0, 1), (30.0001, 10.0, 2), (39.9, 10.0, 3), (25.5, 8.5, 4)])
def test_shift_rule_equals_per_pair_wrap_on_three_cells(L, rc, seed):
    accepted, differ, nc = _compare(L, rc, 1500, seed)
    assert nc == 3
    assert accepted > 10000
    assert differ == 0


@pytest.mark.parametrize("L,rc,seed", [(30.0, 10.0, 6), (30.0001, 10.0, 7), (39.9, 10.0, 8), (25.5, 8.5, 9),
                                       (49.6, 12.0, 10)])
def test_exact_rule_per_unit_equals_per_pair(L, rc, seed):
    accepted, differ, nc = _compare(L, rc, 1500, seed, rule="exact")
    assert nc >= 3
    assert accepted > 5000
    assert differ == 0


def test_shift_rule_differs_on_two_cells():
    """The same comparison on a 2-cell grid (not a half-shell grid) finds differences: the test
    can see a wrong rule."""
    accepted, differ, nc = _compare(35.9999, 12.0, 1500, 5)
    assert nc == 2
    assert differ > 0
