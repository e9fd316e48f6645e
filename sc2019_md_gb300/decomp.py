"""Spatial decomposition of one system over ranks: slabs of cell layers along x (mdrl_slab_plan).

The data plane the library leaves to the caller, over torch.distributed point-to-point messages
(NCCL between GPUs, gloo on the CPU):

1. Each rank holds the particles of its slab (x, y, z, q, type and their global ids), in increasing
   global id.
2. halo(): a rank sends its first cell layer to the rank before it (export_to) and receives the
   first layer of the rank after it (import_from): its half-shell halo.  The local set is the
   owned particles followed by the halo, both in increasing global id, so every cell keeps its
   particles in the same relative order as in the undivided system.
3. The caller evaluates the units whose home cell lies in the slab on the local set
   (Context.force_fixed with home = (x0, x1)): int64 2^-24 fixed-point forces.
4. return_forces(): the halo rows go back to import_from, the rows of this rank's exported
   particles come back from export_to and are added -- integer sums, so the owned forces equal
   the single-domain forces bit for bit.

This follows the export/import pattern of the reference's strong-scaling model
(MatlabScripts/SC19_MD_Strong_Scale_Performance.m:130-212).  Every call here exchanges whole
arrays; no rank waits on another inside a kernel.
"""
from __future__ import annotations

import numpy as np

from . import Params, slab_plan, slab_select


class SlabDomain:
    """One rank's slab of a decomposed system."""

    def __init__(self, params: Params, nranks: int, rank: int):
        self.params = params
        self.slab = slab_plan(params, nranks, rank)
        ny, nz = self.slab.ncell[1], self.slab.ncell[2]
        self.home = (self.slab.x0, self.slab.x1)
        self.home_cells = (self.slab.x0 * ny * nz, self.slab.x1 * ny * nz)

    def owned(self, x) -> np.ndarray:
        """Indices (into x) of the particles this rank owns."""
        return slab_select(self.params, self.slab, x)[0]

    # ---- communication -----------------------------------------------------------------------
    def _sendrecv(self, dist, device, send: list, dtypes: list) -> list:
        """Send the arrays `send` to export_to and receive the same kinds from import_from
        (sizes first, then data)."""
        import torch
        s = self.slab
        if s.nranks == 1:
            return [np.asarray(a).copy() for a in send]
        n_out = torch.tensor([len(send[0])], dtype=torch.int64, device=device)
        n_in = torch.zeros(1, dtype=torch.int64, device=device)
        reqs = [dist.isend(n_out, s.export_to), dist.irecv(n_in, s.import_from)]
        for r in reqs:
            r.wait()
        m = int(n_in.item())
        out, recv, reqs = [], [], []
        for a, dt in zip(send, dtypes):
            t = torch.as_tensor(np.ascontiguousarray(a, dtype=dt)).to(device)
            shape = (m,) + tuple(t.shape[1:])
            r = torch.empty(shape, dtype=t.dtype, device=device)
            out.append(t)
            recv.append(r)
            reqs += [dist.isend(t, s.export_to), dist.irecv(r, s.import_from)]
        for r in reqs:
            r.wait()
        return [r.cpu().numpy() for r in recv]

    def _return(self, dist, device, rows: np.ndarray) -> np.ndarray:
        """Send `rows` to import_from (the halo's owner) and receive this rank's exported rows
        from export_to."""
        import torch
        s = self.slab
        if s.nranks == 1:
            return rows.copy()
        t = torch.as_tensor(np.ascontiguousarray(rows)).to(device)
        r = torch.empty((self._n_exported,) + tuple(t.shape[1:]), dtype=t.dtype, device=device)
        reqs = [dist.isend(t, s.import_from), dist.irecv(r, s.export_to)]
        for q in reqs:
            q.wait()
        return r.cpu().numpy()

    def halo(self, dist, pos, q, type, gid, device="cpu"):
        """Exchange the half-shell halo.  pos (n,3), q (n,), type (n,), gid (n,) are this rank's
        owned particles in increasing gid.  Returns the local set (pos, q, type, gid) = owned
        followed by the halo, and remembers the split."""
        pos = np.asarray(pos, np.float32)
        _, exported = slab_select(self.params, self.slab, pos[:, 0])
        self._exported = exported
        self._n_exported = len(exported)
        self._n_owned = len(pos)
        pq = np.concatenate([pos[exported], np.asarray(q, np.float32)[exported, None]], 1)
        hp, ht, hg = self._sendrecv(dist, device, [pq, np.asarray(type)[exported], np.asarray(gid)[exported]],
                                    [np.float32, np.int32, np.int64])
        if self.slab.nranks == 1:
            hp, ht, hg = hp[:0], ht[:0], hg[:0]
        lpos = np.concatenate([pos, hp[:, :3]]).astype(np.float32)
        lq = np.concatenate([np.asarray(q, np.float32), hp[:, 3]]).astype(np.float32)
        lt = np.concatenate([np.asarray(type, np.int32), ht]).astype(np.int32)
        lg = np.concatenate([np.asarray(gid, np.int64), hg]).astype(np.int64)
        return lpos, lq, lt, lg

    def return_forces(self, dist, F_local: np.ndarray, device="cpu") -> np.ndarray:
        """Send the halo rows of the int64 forces back to their owner, add the rows returned for
        this rank's exported particles; returns the owned particles' forces (int64, (n_owned, 3))."""
        F_local = np.asarray(F_local, np.int64)
        own = F_local[: self._n_owned].copy()
        if self.slab.nranks == 1:
            return own
        back = self._return(dist, device, F_local[self._n_owned:])
        own[self._exported] += back
        return own
