"""mdrl_force_eval_static — the force evaluation for callers that cannot allocate device memory
(a device owned by another allocator or memory pool, a plugin host that forbids cudaMalloc, a
loop that cannot pay for a first-use allocation).  Its scratch is a static device array, so no
context and no allocation is needed; the test compares it, through the C ABI, with the
context-based mdrl_force_eval on two calls in a row (two different systems, so the second call
also shows that the array's leftovers from the first are cleared), using the force tolerance of
the other parity tests.  This file is collected last on purpose."""
import numpy as np
import pytest
import torch

import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems

pytestmark = pytest.mark.gpu

SUM_TOL = 2e-6
FIX_ABS = 64 * 2.0 ** -24


def _dev(a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _static_forces(p, s):
    n = s.n
    x, y, z = (_dev(s.pos[:, k], torch.float32) for k in range(3))
    q = _dev(s.q, torch.float32)
    t = _dev(s.type, torch.int32)
    fx, fy, fz = (torch.full((n,), float("nan"), dtype=torch.float32, device="cuda") for _ in range(3))
    torch.cuda.synchronize()
    pairs = m.force_eval_static(p, n, x.data_ptr(), y.data_ptr(), z.data_ptr(), q.data_ptr(), t.data_ptr(),
                                fx.data_ptr(), fy.data_ptr(), fz.data_ptr(), None)
    return torch.stack([fx, fy, fz], 1).cpu().numpy(), pairs


def _compare(s, p):
    with m.Context(p) as ctx:
        F_ref, st, _ = ctx.force(s.pos[:, 0], s.pos[:, 1], s.pos[:, 2], s.q, s.type)
    F, pairs = _static_forces(p, s)
    assert pairs == st["pairs"]
    assert np.isfinite(F).all()
    assert (np.abs(F - F_ref) <= SUM_TOL * np.abs(F_ref) + FIX_ABS).all()


def test_static_entry_point_matches_context_entry_point_twice():
    """Two different systems in a row with the same parameters: the second call reuses the tables
    the first copied in and must clear the first call's leftovers."""
    for s in [systems.small_ljc(6000, 49.6, 12.0, seed=41), systems.small_ljc(3500, 49.6, 12.0, seed=42)]:
        _compare(s, s.params(table_bins=1024))


def test_static_entry_point_refits_tables_when_parameters_change():
    """Calls whose table order, bins, evaluation mode or force field differ from the previous
    call's: each must refit and copy its own tables into the array (and the last call switches
    back to the first call's parameters)."""
    s = systems.small_ljc(5000, 49.6, 12.0, seed=44)
    base = s.params(table_bins=1024)
    other = s.params(table_bins=256, table_order=2)
    other.sigma[1], other.epsilon[1] = 3.0, 0.1
    direct = s.params(eval=m.EVAL_DIRECT)
    for p in (base, other, direct, base):
        _compare(s, p)


def test_static_entry_point_rejects_another_device():
    s = systems.small_ljc(64, 49.6, 12.0, seed=45)
    p = s.params()
    p.device = torch.cuda.current_device() + 1
    with pytest.raises(m.MdrlError) as e:
        m.force_eval_static(p, 10, 1, 1, 1, None, None, 1, 1, 1, None)
    assert e.value.status == 1 and "current device" in str(e.value)


def test_static_entry_point_rejects_sizes_beyond_its_limit():
    s = systems.small_ljc(64, 49.6, 12.0, seed=43)
    p = s.params()
    with pytest.raises(m.MdrlError) as e:
        m.force_eval_static(p, 131073, 1, 1, 1, None, None, 1, 1, 1, None)
    assert e.value.status == 3 and "131072" in str(e.value)
    big = s.params(box=(400.0, 400.0, 400.0), ncell=(33, 33, 33))   # 35,937 cells
    with pytest.raises(m.MdrlError) as e:
        m.force_eval_static(big, 10, 1, 1, 1, None, None, 1, 1, 1, None)
    assert e.value.status == 3 and "4096" in str(e.value)
