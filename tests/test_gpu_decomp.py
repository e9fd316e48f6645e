"""The library's half of the spatial decomposition on the GPU: mdrl_force_eval_fixed restricted to
a slab's home layers, on the slab's particles plus its imported halo layer.  The ranks are
evaluated one after another in this process (independent evaluations; nothing waits on another
rank); their int64 forces, with the halo rows added to the owners, must equal the single-domain
int64 forces bit for bit, and their pair counts must add up."""
import numpy as np
import pytest

import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which,nranks,exact,tile", [("small", 2, True, None), ("small", 5, False, None),
                                                    ("ljc92k", 3, True, None), ("small", 3, True, (1, 2, 1)),
                                                    ("ljc92k", 2, False, (1, 1, 1))])
def test_slab_evaluations_sum_to_the_single_domain(which, nranks, exact, tile):
    sysm = systems.small_ljc(6400, 62.5, 12.0, seed=77) if which == "small" else systems.ljc92k()
    p = sysm.params(table_order=2 if exact else 1, table_bins=512, flags=m.FLAG_EXACT_DIFF if exact else 0)
    x = sysm.pos[:, 0]
    with m.Context(p) as ctx:
        if tile is not None:
            ctx.set_tile(*tile)
        F_ref, st_ref = ctx.force_fixed(x, sysm.pos[:, 1], sysm.pos[:, 2], sysm.q, sysm.type)
        F = np.zeros_like(F_ref)
        pairs = 0
        plans = [m.slab_plan(p, nranks, r) for r in range(nranks)]
        sel = [m.slab_select(p, s, x) for s in plans]
        for r, s in enumerate(plans):
            owned = sel[r][0]
            halo = sel[s.import_from][1] if nranks > 1 else owned[:0]   # the next slab's first layer
            loc = np.concatenate([owned, halo])
            Fl, st = ctx.force_fixed(sysm.pos[loc, 0], sysm.pos[loc, 1], sysm.pos[loc, 2], sysm.q[loc],
                                     sysm.type[loc], home=(s.x0, s.x1))
            np.add.at(F, loc, Fl)
            pairs += st["pairs"]
    assert pairs == st_ref["pairs"]
    assert np.array_equal(F, F_ref)


def test_fixed_forces_match_the_float_path():
    """Over the whole box, the int64 forces are what mdrl_force_eval converts to FP32."""
    sysm = systems.small_ljc(3000, 37.5, 12.0, seed=21)
    p = sysm.params(table_bins=512)
    with m.Context(p) as ctx:
        F64, st = ctx.force_fixed(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q, sysm.type)
        F, st2, _ = ctx.force(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.q, sysm.type)
    assert st["pairs"] == st2["pairs"]
    conv = (F64.astype(np.float32) * np.float32(2.0 ** -24)).astype(np.float32)
    assert np.array_equal(conv, F)


def test_fixed_eval_validation():
    sysm = systems.small_ljc(500, 37.5, 12.0, seed=2)
    with m.Context(sysm.params()) as ctx:
        with pytest.raises(m.MdrlError):
            ctx.force_fixed(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], home=(2, 1))
        with pytest.raises(m.MdrlError):
            ctx.force_fixed(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], home=(0, 4))
    with m.Context(sysm.params(accum=m.ACC_FP32_ATOMIC)) as ctx:
        with pytest.raises(m.MdrlError):
            ctx.force_fixed(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2])
