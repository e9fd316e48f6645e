"""Spatial decomposition over ranks on the CPU (gloo, world sizes 2 and 3), checked by the oracle.

Each rank starts with the particles of its slab of cell layers (mdrl_slab_plan / mdrl_slab_select,
host code of the library), exchanges the half-shell halo with its neighbours through
sc2019_md_gb300.decomp (torch.distributed point-to-point), evaluates the units whose home cell lies
in its slab with the oracle's int64 fixed-point traversal, and returns the halo forces to their
owners.  Gathered on rank 0, the owned forces must equal the single-domain oracle bit for bit and
the ranks' pair counts must add up to the single-domain count."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle
import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems
from sc2019_md_gb300.decomp import SlabDomain


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _system():
    return systems.small_ljc(6400, 62.5, 12.0, seed=77)          # 5 x 5 x 5 cells of 12.5 A


def _oracle(sysm, pos, q, t, exact):
    pc64 = oracle.lb_coefficients(sysm.sigma, sysm.epsilon)
    m0 = sysm.table_min_log2
    nseg = int(np.floor(np.log2(np.float32(np.float32(sysm.cutoff) ** 2)))) - m0 + 1
    return oracle.System(pos, sysm.box, sysm.ncell, sysm.cutoff, pc64.astype(np.float32), q=q, type=t,
                         ke=sysm.coulomb_k, tab=oracle.fit_tables(2, nseg, 512, m0, local=True), order=2,
                         nseg=nseg, bins=512, min_log2=m0, local=True, exact=exact)


def _worker(rank, world, port, exact, qout):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sysm = _system()
    p = sysm.params(table_order=2, table_bins=512, flags=m.FLAG_EXACT_DIFF if exact else 0)
    dom = SlabDomain(p, world, rank)
    mine = dom.owned(sysm.pos[:, 0])                  # this rank's particles, increasing global id
    lpos, lq, lt, lg = dom.halo(dist, sysm.pos[mine], sysm.q[mine], sysm.type[mine], mine.astype(np.int64))
    o = _oracle(sysm, lpos, lq, lt, exact)
    F_local, pairs = o.force_cells_fixed(*dom.home_cells)
    F_own = dom.return_forces(dist, F_local)
    qout.put((rank, mine, F_own, pairs, len(lg) - len(mine)))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,exact", [(2, True), (3, False)])
def test_slab_decomposition_equals_single_domain(world, exact):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, exact, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    sysm = _system()
    F_ref, pairs_ref = _oracle(sysm, sysm.pos, sysm.q, sysm.type, exact).force_cells_fixed()
    F = np.zeros_like(F_ref)
    seen = np.zeros(sysm.n, np.int32)
    pairs = 0
    for rank, mine, F_own, p, nhalo in out:
        F[mine] = F_own
        seen[mine] += 1
        pairs += p
        assert nhalo > 0                                  # a halo was imported
    assert (seen == 1).all()                              # every particle owned exactly once
    assert pairs == pairs_ref
    assert np.array_equal(F, F_ref)


def test_slab_plan_covers_the_layers():
    p = _system().params()
    for world in (1, 2, 3, 5):
        layers = []
        for r in range(world):
            s = m.slab_plan(p, world, r)
            assert s.x1 > s.x0 and s.halo_x == s.x1 % 5
            assert s.import_from == (r + 1) % world and s.export_to == (r - 1) % world
            layers += list(range(s.x0, s.x1))
        assert layers == list(range(5))
    with pytest.raises(m.MdrlError):
        m.slab_plan(p, 6, 0)                              # more ranks than layers
