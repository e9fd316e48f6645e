"""Failure handling on the GPU without a GPU fault.

* Host-side fault injection (MDRL_FAULT): a named CUDA runtime call of an entry point is made to
  report failure on the host (the call is not made); the entry point must return
  MDRL_ERR_CUDA with an error text that names the injected call, the same context must give the
  right answer on the next call, and it must still be destroyable.
* Force sums the accumulators cannot hold (NaN, infinite, or beyond the int64 fixed-point range)
  are reported as MDRL_ERR_RANGE instead of being converted silently.
* Cells above 1,024 particles are ordered by the chunked sort (parity with the oracle); a cell
  above the 65,536-particle limit returns MDRL_ERR_CELL_OVERFLOW in bounded time.

Nothing here faults, traps or hangs the GPU: every failure is made on the host or comes from
finite inputs that the kernels' own checks turn into a status.
"""
import dataclasses
import os

import numpy as np
import pytest
import torch

import oracle
import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems
from helpers import oracle_from_ctx

pytestmark = pytest.mark.gpu

SUM_TOL = 2e-6
FIX_ABS = 64 * 2.0 ** -24


@pytest.fixture(scope="module")
def sysm():
    return systems.small_ljc(2500, 37.5, 12.0, seed=31)


def arm(spec: str) -> None:
    """Arm MDRL_FAULT: the variable is read when a context is created, and the count starts when
    mdrl_create returns, so a throwaway context arms the fault for the next entry point called."""
    os.environ["MDRL_FAULT"] = spec
    try:
        with m.Context(m.default_params()):
            pass
    finally:
        del os.environ["MDRL_FAULT"]


def expect_injected(fn, call: str):
    with pytest.raises(m.MdrlError) as e:
        fn()
    assert e.value.status == 4, e.value
    assert "injected" in str(e.value) and call.rstrip("(") in str(e.value), str(e.value)


def _dev(a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def test_create_fault_leaves_nothing_behind(sysm):
    os.environ["MDRL_FAULT"] = "create:cudaMalloc"
    try:
        expect_injected(lambda: m.Context(sysm.params()), "cudaMalloc")
    finally:
        del os.environ["MDRL_FAULT"]
    with m.Context(sysm.params()) as ctx:          # the library is still usable
        F, st, _ = ctx.force(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q, sysm.type)
    assert st["pairs"] > 0


@pytest.mark.parametrize("call", ["cudaMemcpyAsync", "cudaStreamSynchronize", "cudaMemsetAsync",
                                  "cudaEventRecord", "cudaGetLastError"])
def test_force_eval_faults(sysm, call):
    x, y, z = (np.ascontiguousarray(sysm.pos[:, k]) for k in range(3))
    with m.Context(sysm.params()) as ctx:
        F0, st0, _ = ctx.force(x, y, z, sysm.q, sysm.type)
        arm(call)
        expect_injected(lambda: ctx.force(x, y, z, sysm.q, sysm.type), call)
        F1, st1, _ = ctx.force(x, y, z, sysm.q, sysm.type)
    assert np.array_equal(F0.view(np.uint32), F1.view(np.uint32)) and st0["pairs"] == st1["pairs"]


def test_force_eval_device_fault(sysm):
    n = sysm.n
    x, y, z, q = (_dev(a, torch.float32) for a in (sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q))
    t = _dev(sysm.type, torch.int32)
    out = [torch.zeros(n, dtype=torch.float32, device="cuda") for _ in range(3)]
    lib = m.lib()
    import ctypes as C

    def call():
        st = m.Stats()
        s = lib.mdrl_force_eval_device(ctx._h, n, *(C.cast(v.data_ptr(), C.POINTER(C.c_float)) for v in (x, y, z, q)),
                                       C.cast(t.data_ptr(), C.POINTER(C.c_int)),
                                       *(C.cast(v.data_ptr(), C.POINTER(C.c_float)) for v in out), None, C.byref(st))
        if s != 0:
            raise m.MdrlError(s, lib.mdrl_last_error().decode())
        return st

    with m.Context(sysm.params()) as ctx:
        st0 = call()
        F0 = torch.stack(out, 1).cpu().numpy()
        arm("cudaMemsetAsync")
        expect_injected(call, "cudaMemsetAsync")
        st1 = call()
        F1 = torch.stack(out, 1).cpu().numpy()
    assert np.array_equal(F0, F1) and st0.pairs == st1.pairs


@pytest.mark.parametrize("call", ["cudaStreamBeginCapture", "cudaGraphInstantiate", "cudaGraphLaunch",
                                  "cudaEventElapsedTime", "cudaMemsetAsync"])
def test_step_faults(sysm, call):
    args = (sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
    with m.Context(sysm.params()) as ref:
        ref.set_state(*args)
        ref.step(3)
        want = ref.state()
    with m.Context(sysm.params()) as ctx:
        ctx.set_state(*args)
        arm(call)
        expect_injected(lambda: ctx.step(3), call)
        if call in ("cudaEventElapsedTime",):
            # the steps ran (only the timing read failed): start again from the same state
            ctx.set_state(*args)
        ctx.step(3)
        got = ctx.state()
    for a, b in zip(want, got):
        assert np.array_equal(np.asarray(a), np.asarray(b))


@pytest.mark.parametrize("entry,call", [("set_state", "cudaStreamSynchronize"), ("get_state", "cudaMemcpyAsync"),
                                        ("time_force", "cudaEventElapsedTime"), ("autotune", "cudaEventElapsedTime"),
                                        ("bin", "cudaMemcpyAsync"), ("pair_eval", "cudaMemcpyAsync"),
                                        ("set_pme", "cudaMalloc"), ("set_tables", "cudaMemcpy("),
                                        ("set_pair_coefficients", "cudaStreamSynchronize"),
                                        ("set_bonded", "cudaMalloc")])
def test_entry_point_faults(sysm, entry, call):
    args = (sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
    with m.Context(sysm.params()) as ctx:
        ctx.set_state(*args)
        tab, meta = ctx.tables()
        pc = ctx.pair_coefficients()
        ops = {
            "set_state": lambda: ctx.set_state(*args),
            "get_state": lambda: ctx.state(),
            "time_force": lambda: ctx.time_force(),
            "autotune": lambda: ctx.autotune(retime=True),
            "bin": lambda: ctx.bin(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2]),
            "pair_eval": lambda: ctx.pair_eval(np.column_stack([sysm.pos[:64], sysm.q[:64]]),
                                               np.column_stack([sysm.pos[64:128], sysm.q[64:128]])),
            "set_pme": lambda: ctx.set_pme(),
            "set_tables": lambda: ctx.set_tables(tab, order=meta["order"], nseg=meta["nseg"], bins=meta["bins"],
                                                 min_log2=meta["min_log2"]),
            "set_pair_coefficients": lambda: ctx.set_pair_coefficients(np.ones((4 * 4 * 4,))),
            "set_bonded": lambda: ctx.set_bonded(bonds=(np.array([[0, 1]], np.int32), np.array([[100.0, 1.5]]))),
        }
        arm(call)
        expect_injected(ops[entry], call)
        ops[entry]()                                   # the fault is spent: the same call succeeds
    # destroyed without error; a fresh context on the same device works
    with m.Context(sysm.params()) as ctx:
        _, st, _ = ctx.force(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q, sysm.type)
    assert st["pairs"] > 0


@pytest.mark.parametrize("entry,call", [("force", "cudaMemcpyAsync"), ("set_state", "cudaStreamSynchronize"),
                                        ("step", "cudaGraphLaunch"), ("time_force", "cudaEventElapsedTime")])
def test_batch_faults(entry, call):
    reps = [systems.replica(n, r) for r, n in enumerate([900, 3000, 6000])]
    pos, vel, q, t, spec = systems.concat(reps)
    p = reps[0].params()
    with m.Batch(p, spec) as b:
        b.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, q, t)
        ops = {"force": lambda: b.force(pos[:, 0], pos[:, 1], pos[:, 2], q, t),
               "set_state": lambda: b.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, q, t),
               "step": lambda: b.step(2), "time_force": lambda: b.time_force()}
        arm(call)
        expect_injected(ops[entry], call)
        ops[entry]()


def test_static_entry_point_fault(sysm):
    n = sysm.n
    x, y, z, q = (_dev(a, torch.float32) for a in (sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q))
    t = _dev(sysm.type, torch.int32)
    f = [torch.zeros(n, dtype=torch.float32, device="cuda") for _ in range(3)]
    p = sysm.params()
    call = lambda: m.force_eval_static(p, n, x.data_ptr(), y.data_ptr(), z.data_ptr(), q.data_ptr(), t.data_ptr(),
                                       f[0].data_ptr(), f[1].data_ptr(), f[2].data_ptr(), None)
    os.environ["MDRL_FAULT"] = "cudaMemsetAsync"
    try:
        expect_injected(call, "cudaMemsetAsync")
    finally:
        del os.environ["MDRL_FAULT"]
    assert call() > 0


@pytest.mark.parametrize("accum", [m.ACC_FIXED64, m.ACC_FP32_ATOMIC, m.ACC_KAHAN])
def test_unrepresentable_forces_are_reported(sysm, accum):
    """A pair planted 0.8 A apart and an r^-14 multiplier of 3e38 make a force infinite (FP32
    modes; 3e38 x 0.64^-7 overflows) or push it past the fixed-point range: the call returns
    MDRL_ERR_RANGE; with sane multipliers again the same context matches a fresh one."""
    pos = sysm.pos.copy()
    pos[1] = pos[0] + np.float32(0.8) * np.array([1, 0, 0], np.float32)
    pos[1, 0] = pos[1, 0] - np.float32(1.6) if pos[1, 0] >= np.float32(sysm.box[0]) else pos[1, 0]
    x, y, z = (np.ascontiguousarray(pos[:, k]) for k in range(3))
    p = sysm.params(accum=accum, table_min_log2=-2)
    with m.Context(p) as ref:
        F0, _, _ = ref.force(x, y, z, sysm.q, sysm.type)
        pc = ref.pair_coefficients().astype(np.float64)
    with m.Context(p) as ctx:
        huge = pc.copy()
        huge[:, 0] = 3.0e38
        ctx.set_pair_coefficients(huge)
        with pytest.raises(m.MdrlError) as e:
            ctx.force(x, y, z, sysm.q, sysm.type)
        assert e.value.status == 3 and "force component" in str(e.value)
        with pytest.raises(m.MdrlError) as e:
            ctx.set_state(x, y, z, sysm.vel, sysm.q, sysm.type)
        assert e.value.status == 3 and "force component" in str(e.value)
        ctx.set_pair_coefficients(pc)
        F1, _, _ = ctx.force(x, y, z, sysm.q, sysm.type)
    if accum != m.ACC_FP32_ATOMIC:
        assert np.array_equal(F0.view(np.uint32), F1.view(np.uint32))
    else:
        assert np.allclose(F0, F1, rtol=1e-5, atol=1e-3)


def test_fixed_point_range_is_reported_during_md(sysm):
    """A state that is fine at set_state and whose forces leave the fixed-point range during
    mdrl_step: the step returns MDRL_ERR_RANGE."""
    x, y, z = (np.ascontiguousarray(sysm.pos[:, k]) for k in range(3))
    with m.Context(sysm.params()) as ctx:
        pc = ctx.pair_coefficients().astype(np.float64)
        ctx.set_state(x, y, z, sysm.vel, sysm.q, sysm.type)
        big = pc.copy()
        big[:, 0] = 1.0e30                             # A14: far beyond 5.4e11 kcal/mol/A at 1 A
        ctx.set_pair_coefficients(big)
        with pytest.raises(m.MdrlError) as e:
            ctx.step(1)
        assert e.value.status == 3


def clustered(n_big: int, n_rest: int, L: float = 37.5, seed: int = 5):
    """n_big particles crowded into one corner cell (3x3x3 cells of 12.5 A) plus n_rest spread
    uniformly; type 0 only (sigma 2.0 A, epsilon 0.02), so the crowded pairs below the first table
    point stay far inside the fixed-point range."""
    rng = np.random.default_rng(seed)
    big = rng.uniform(0.25, 12.25, (n_big, 3))
    rest = rng.uniform(0.0, L, (n_rest, 3))
    pos = np.concatenate([big, rest]).astype(np.float32)
    pos[pos >= np.float32(L)] = 0.0
    q = np.where(rng.random(len(pos)) < 0.5, -0.42, 0.42).astype(np.float32)
    t = np.zeros(len(pos), np.int32)
    base = systems.small_ljc(64, L, 12.0, seed=seed)
    return dataclasses.replace(base, pos=pos, vel=np.zeros_like(pos), q=q, type=t)


@pytest.mark.parametrize("tile", [None, (1, 1, 1), (1, 3, 1)])
def test_large_cell_chunked_sort_matches_oracle(tile):
    """A cell of 3,000 particles (above the 1,024 of the one-pass sort): the binning order equals
    the oracle's and the forces, counts and pair total keep parity, with the default tile and with
    one warp per item (whose j cell is taken 256 particles at a time)."""
    sysm = clustered(3000, 1500)
    pos = sysm.pos
    p = sysm.params(table_bins=512, flags=m.FLAG_ENERGY)
    with m.Context(p) as ctx:
        if tile is not None:
            ctx.set_tile(*tile)
        cell_of, count, order = ctx.bin(pos[:, 0], pos[:, 1], pos[:, 2])
        assert count.max() >= 3000
        F, st, cnt = ctx.force(pos[:, 0], pos[:, 1], pos[:, 2], sysm.q, sysm.type, counts=True)
        o = oracle_from_ctx(ctx, sysm)
    oc, _, oorder, _ = oracle.bin_cells(pos, p.box, tuple(p.ncell))
    assert np.array_equal(cell_of, oc) and np.array_equal(order, oorder)
    Fo, Fabs, cnto, sto = o.force_cells()
    assert np.array_equal(cnt, cnto) and st["pairs"] == sto["pairs"]
    assert (np.abs(F - Fo) <= SUM_TOL * Fabs + FIX_ABS).all()


def test_cell_overflow_is_reported_and_bounded():
    """70,000 particles in one cell (above the 65,536 limit): MDRL_ERR_CELL_OVERFLOW, returned
    in bounded time, and the context then evaluates an ordinary system correctly."""
    base = clustered(70000, 100, seed=6)
    pos = base.pos
    ok = systems.small_ljc(2500, 37.5, 12.0, seed=31)
    with m.Context(base.params()) as ctx:
        with pytest.raises(m.MdrlError) as e:
            ctx.force(pos[:, 0], pos[:, 1], pos[:, 2], base.q, base.type)
        assert e.value.status == 2 and "65536" in str(e.value)
        F, st, _ = ctx.force(ok.pos[:, 0], ok.pos[:, 1], ok.pos[:, 2], ok.q, ok.type)
    with m.Context(base.params()) as ref:
        F0, st0, _ = ref.force(ok.pos[:, 0], ok.pos[:, 1], ok.pos[:, 2], ok.q, ok.type)
    assert np.array_equal(F.view(np.uint32), F0.view(np.uint32)) and st["pairs"] == st0["pairs"]
