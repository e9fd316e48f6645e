"""The block culling of the force kernels never drops a block that holds an accepted pair.

The kernels skip a (4-particle i group, 8-particle j step) block when the two bounding boxes are
farther apart than rc (`mdrl_force_warp.cuh` mask pass, `mdrl_force.cuh` pre-pass); the half
widths of the i group carry a margin of 2^-20 x the largest box edge for the FP32 rounding of the
centres, widths, gaps and the pair differences.  This test restates both computations in FP32
with IEEE rounding per operation (numpy float32), for the three difference rules (per-unit
shift, exact minimum image, per-pair wrap), on near-cutoff and across-boundary blocks, with the
box test's sum of squares evaluated with and without fused multiply-adds, and checks that every
block with a pair passing 0 < r2 <= rc2 is kept."""
import numpy as np
import pytest

f32 = np.float32
MARGIN = f32(9.5367431640625e-07)   # 2^-20


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def _wrap(d, L, h):
    return np.where(d > h, (d - L).astype(f32), np.where(d < -h, (d + L).astype(f32), d)).astype(f32)


def _blocks(rng, T, mode):
    """T blocks: i groups (T, 4, 3) and j steps (T, 8, 3) in [0, L), the unit shift s (T, 3), box
    edges L (T, 3) and the cutoff, placed so that the closest pair lies near rc."""
    rc = f32(rng.choice([8.5, 10.0, 12.0]))
    if mode == "wrap":
        L = rng.uniform(2 * rc + 0.1, 60.0, (T, 3)).astype(f32)
    else:
        L = rng.uniform(3 * rc, 230.0, (T, 3)).astype(f32)
    # cluster spread: single points (a degenerate box) up to 1 A
    sig = rng.choice([0.0, 1e-5, 1e-3, 0.1, 1.0], T)[:, None, None]
    u = rng.standard_normal((T, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    # |D| at rc within a few FP32 ulps, or within the clusters' spread of it
    k = rng.integers(-64, 65, T)[:, None]
    length = rc * (1.0 + k * 2.0 ** -23) + np.where(sig[:, :, 0] > 0, rng.uniform(-3, 1, (T, 1)) * sig[:, :, 0], 0.0)
    D = u * length
    ci = rng.uniform(0, 1, (T, 3)) * L
    # push a third of the i centres against the box faces (largest coordinates, boundary shifts)
    face = rng.random(T) < 0.33
    ci[face] = np.where(rng.random((face.sum(), 3)) < 0.5, L[face] * (1 - 1e-6), 1e-6 * L[face])
    cj = ci - D
    s = np.zeros((T, 3))
    if mode != "wrap":
        s = np.where(cj < 0, 1.0, np.where(cj >= L, -1.0, 0.0)) * L
        cj = cj + s
    else:
        cj = np.mod(cj, L)
    pi = ci[:, None, :] + rng.uniform(-1, 1, (T, 4, 3)) * sig
    pj = cj[:, None, :] + rng.uniform(-1, 1, (T, 8, 3)) * sig
    # keep every particle inside [0, L) on the side of the boundary its cluster is on
    Lb = L[:, None, :].astype(np.float64)
    pi = np.clip(pi, 0.0, np.nextafter(Lb, 0)).astype(f32)
    pj = np.clip(pj, 0.0, np.nextafter(Lb, 0)).astype(f32)
    return pi, pj, s.astype(f32), L, rc


def _accepted(pi, pj, s, L, rc, mode, near=False):
    """Any pair of the block with 0 < r2 <= rc2 under the kernels' FP32 pair arithmetic (near:
    any with rc2 (1 - 1e-5) <= r2 <= rc2)."""
    xi = pi[:, :, None, :]
    xj = pj[:, None, :, :]
    sb = s[:, None, None, :]
    Lb = L[:, None, None, :]
    if mode == "shift":
        d = ((xi - xj).astype(f32) + sb).astype(f32)
    elif mode == "exact":
        xi2 = (xi + np.where(sb < 0, sb, f32(0))).astype(f32)
        xj2 = (xj - np.where(sb > 0, sb, f32(0))).astype(f32)
        d = (xi2 - xj2).astype(f32)
    else:
        d = _wrap((xi - xj).astype(f32), Lb, (f32(0.5) * Lb).astype(f32))
    sq = (d * d).astype(f32)
    r2 = ((sq[..., 0] + sq[..., 1]).astype(f32) + sq[..., 2]).astype(f32)
    rc2 = f32(rc * rc)
    lo = rc2 * (1 - 1e-5) if near else 0.0
    return ((r2 > lo) & (r2 <= rc2)).any(axis=(1, 2))


def _kept(pi, pj, s, L, rc, mode, fused):
    """The kernels' box test for the block, in FP32."""
    half = f32(0.5)
    if mode == "exact":   # boxes of the exact-rule coordinates, no shift on the centre
        pi = (pi + np.where(s < 0, s, f32(0))[:, None, :]).astype(f32)
        pj = (pj - np.where(s > 0, s, f32(0))[:, None, :]).astype(f32)
    li, ui = pi.min(1), pi.max(1)
    lj, uj = pj.min(1), pj.max(1)
    margin = (MARGIN * L.max(axis=1, keepdims=True)).astype(f32)
    ci = (half * (li + ui).astype(f32)).astype(f32)
    if mode == "shift":
        ci = (ci + s).astype(f32)
    hi = ((half * (ui - li).astype(f32)).astype(f32) + margin).astype(f32)
    cj = (half * (lj + uj).astype(f32)).astype(f32)
    hj = (half * (uj - lj).astype(f32)).astype(f32)
    e = (ci - cj).astype(f32)
    if mode == "wrap":
        e = _wrap(e, L, (half * L).astype(f32))
    gap = np.maximum((np.abs(e) - (hi + hj).astype(f32)).astype(f32), f32(0))
    gx, gy, gz = gap[:, 0], gap[:, 1], gap[:, 2]
    if fused:
        ss = _fma(gz, gz, _fma(gy, gy, (gx * gx).astype(f32)))
    else:
        ss = (((gx * gx).astype(f32) + (gy * gy).astype(f32)).astype(f32) + (gz * gz).astype(f32)).astype(f32)
    return ss <= f32(rc * rc)


@pytest.mark.parametrize("mode", ["shift", "exact", "wrap"])
def test_culling_keeps_every_block_with_an_accepted_pair(mode):
    rng = np.random.default_rng({"shift": 11, "exact": 12, "wrap": 13}[mode])
    near = 0
    for _ in range(4):
        pi, pj, s, L, rc = _blocks(rng, 50_000, mode)
        acc = _accepted(pi, pj, s, L, rc, mode)
        for fused in (False, True):
            kept = _kept(pi, pj, s, L, rc, mode, fused)
            bad = np.flatnonzero(acc & ~kept)
            assert bad.size == 0, (mode, fused, bad[:5])
        # the cases decide near the threshold: blocks whose accepted pair has r2 within 1e-5 of rc2
        near += int(_accepted(pi, pj, s, L, rc, mode, near=True).sum())
    assert near > 10_000


def test_margin_is_needed():
    """Without the margin the same FP32 box test drops blocks that hold accepted pairs, so the
    cases above exercise the rounding the margin is there for."""
    global MARGIN
    rng = np.random.default_rng(7)
    saved = MARGIN
    try:
        MARGIN = f32(0)
        dropped = 0
        for mode in ("shift", "exact"):
            pi, pj, s, L, rc = _blocks(rng, 50_000, mode)
            acc = _accepted(pi, pj, s, L, rc, mode)
            dropped += int((acc & ~_kept(pi, pj, s, L, rc, mode, False)).sum())
    finally:
        MARGIN = saved
    assert dropped > 0
