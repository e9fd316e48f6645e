"""mdrl_force_eval on page-locked host buffers: the kernels read the inputs and write the forces
in place over the host link (no staging copies).  Results are bit-identical to the same call on
pageable buffers (staged through copies), for every combination of optional inputs, and a call
mixing pinned and pageable buffers takes the staged path with the same results."""
import ctypes as C

import numpy as np
import pytest

import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

F = C.POINTER(C.c_float)
I = C.POINTER(C.c_int)


def _pinned(a):
    t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32, pin_memory=True)
    out = t.numpy()
    out[...] = a
    return out, t


def _call(ctx, n, x, y, z, q, t, fx, fy, fz, cnt):
    st = m.Stats()
    p = lambda a, T: None if a is None else a.ctypes.data_as(T)
    s = m.lib().mdrl_force_eval(ctx._h, n, p(x, F), p(y, F), p(z, F), p(q, F), p(t, I), p(fx, F), p(fy, F),
                                p(fz, F), p(cnt, I), C.byref(st))
    if s != 0:
        raise m.MdrlError(s, m.lib().mdrl_last_error().decode())
    return st


@pytest.mark.parametrize("with_q,with_type,with_counts", [(True, True, True), (True, True, False),
                                                          (False, False, True), (False, True, False)])
def test_pinned_buffers_match_pageable(with_q, with_type, with_counts):
    s = systems.small_ljc(6400, 50.0, 12.0, seed=31)
    n = s.n
    ins = [np.ascontiguousarray(s.pos[:, k]) for k in range(3)]
    q = s.q.astype(np.float32) if with_q else None
    t = s.type.astype(np.int32) if with_type else None
    outs = {}
    keep = []
    for mode in ("pageable", "pinned", "mixed"):
        bx = list(ins)
        bq, bt = q, t
        fx, fy, fz = (np.zeros(n, np.float32) for _ in range(3))
        cnt = np.zeros(n, np.int32) if with_counts else None
        if mode != "pageable":
            pins = [_pinned(a) for a in bx]
            keep += pins
            bx = [a for a, _ in pins]
            if bq is not None:
                bq, tq = _pinned(bq); keep.append(tq)
            if bt is not None:
                bt, tt = _pinned(bt); keep.append(tt)
            po = [_pinned(np.zeros(n, np.float32)) for _ in range(3)]
            keep += po
            fx, fy, fz = (a for a, _ in po)
            if cnt is not None:
                cnt, tc = _pinned(cnt); keep.append(tc)
            if mode == "mixed":
                fz = np.zeros(n, np.float32)          # one pageable output: the staged path
        with m.Context(s.params(table_bins=512, flags=m.FLAG_ENERGY)) as ctx:
            st = _call(ctx, n, *bx, bq, bt, fx, fy, fz, cnt)
            st2 = _call(ctx, n, *bx, bq, bt, fx, fy, fz, cnt)     # a second call on the same context
        outs[mode] = (np.stack([fx, fy, fz], 1).copy(), None if cnt is None else cnt.copy(), st.pairs, st.e_lj,
                      st2.pairs)
    ref = outs["pageable"]
    assert ref[2] > 0 and ref[2] == ref[4]
    for mode in ("pinned", "mixed"):
        o = outs[mode]
        assert np.array_equal(o[0].view(np.uint32), ref[0].view(np.uint32)), mode
        if with_counts:
            assert np.array_equal(o[1], ref[1]), mode
        assert o[2] == ref[2] and o[3] == ref[3] and o[4] == ref[4], mode


def test_pinned_inputs_are_validated():
    """Out-of-box positions and bad types read in place raise the same errors as staged ones."""
    n = 4
    x, tx = _pinned(np.array([1.0, 2.0, 3.0, 30.0], np.float32))
    y, ty = _pinned(np.ones(n, np.float32))
    z, tz = _pinned(np.ones(n, np.float32))
    fo = [_pinned(np.zeros(n, np.float32)) for _ in range(3)]
    with m.Context(m.default_params()) as ctx:
        with pytest.raises(m.MdrlError):
            _call(ctx, n, x, y, z, None, None, *(a for a, _ in fo), None)
        x[3] = 4.0
        bad, tb = _pinned(np.array([0, 0, 7, 0], np.int32))
        with pytest.raises(m.MdrlError) as e:
            _call(ctx, n, x, y, z, None, bad, *(a for a, _ in fo), None)
        assert "types" in str(e.value)
        st = _call(ctx, n, x, y, z, None, None, *(a for a, _ in fo), None)
        assert st.pairs == 6
