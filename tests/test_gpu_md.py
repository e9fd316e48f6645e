"""GPU molecular dynamics (velocity Verlet on device-resident cell-sorted state) and the
MD_Evaluation_Model drop-in."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
import sc2019_md_gb300 as m
from sc2019_md_gb300 import systems
from helpers import GOLDEN, oracle_from_ctx

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def _vv_reference(sysm, ctx, F0, dt, nsteps):
    """Velocity Verlet in numpy (FP32 fused updates as in the kernels) with oracle forces."""
    p = ctx.params
    conv = 4.184e-4
    cm = np.array([np.float32(0.5 * dt * conv / p.mass[t]) for t in range(p.ntypes)], np.float32)[sysm.type]
    x = sysm.pos.astype(np.float32).copy()
    v = sysm.vel.astype(np.float32).copy()
    F = F0.astype(np.float32)
    box = np.asarray(sysm.box, np.float32)
    for _ in range(nsteps):
        v = (F * cm[:, None] + v).astype(np.float32)
        x = (v * np.float32(dt) + x).astype(np.float32)
        x = np.where(x < 0, x + box, np.where(x >= box, x - box, x)).astype(np.float32)
        sysm2 = systems.System(sysm.name, sysm.box, sysm.cutoff, sysm.ncell, x, v, sysm.q, sysm.type,
                               sysm.sigma, sysm.epsilon, sysm.mass, sysm.coulomb_k)
        Fo, _, _, _ = oracle_from_ctx(ctx, sysm2).force_cells()
        F = Fo.astype(np.float32)
        v = (F * cm[:, None] + v).astype(np.float32)
    return x, v, F


@pytest.mark.parametrize("tile", [None, (1, 1, 1)])
def test_step_matches_reference_integration(tile):
    """Three velocity-Verlet steps (one captured graph each) against numpy integration with oracle
    forces, with the default tile and with the persistent one-warp-per-item kernel."""
    sysm = systems.lj1728()
    p = sysm.params(table_bins=512)
    with m.Context(p) as ctx:
        if tile is not None:
            ctx.set_tile(*tile)
        ctx.set_state(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, None, sysm.type)
        x0, v0, F0 = ctx.state()
        st = ctx.step(3)
        x, v, F = ctx.state()
        xr, vr, Fr = _vv_reference(sysm, ctx, F0, 2.0, 3)
    assert st["pairs"] > 0 and st["pairs_total"] >= 3 * st["pairs"] * 0.9
    assert np.abs(x - xr).max() < 1e-4
    rel = np.abs(F - Fr).max() / np.abs(Fr).max()
    assert rel < 1e-4, rel


def test_step_energy_conservation_liquid_argon():
    """A liquid-argon state point (0.021 /A^3, 120 K, rc 8.5 A in a 36 A box): total energy drift
    over 500 velocity-Verlet steps of 2 fs stays below 1e-3 of the kinetic energy."""
    rng = np.random.default_rng(3)
    L = 36.0
    nside = 12
    g = (np.arange(nside) + 0.5) * (L / nside)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) + rng.uniform(-0.05, 0.05, (nside ** 3, 3))
    pos = systems.wrap_into_box(pos, (L, L, L))
    vel = systems.maxwell(len(pos), np.full(len(pos), 39.95), 120.0, rng)
    sysm = systems.System("argon", (L, L, L), 8.5, (4, 4, 4), pos, vel, None, np.zeros(len(pos), np.int32),
                          [3.4], [0.238], [39.95], 0.0)
    p = sysm.params(table_bins=1024, table_order=2, flags=m.FLAG_ENERGY)
    with m.Context(p) as ctx:
        ctx.set_state(pos[:, 0], pos[:, 1], pos[:, 2], vel, None, sysm.type)
        e = []
        for _ in range(10):
            st = ctx.step(50)
            e.append((st["e_lj"], st["kinetic"]))
    e = np.asarray(e)
    tot = e[:, 0] + e[:, 1]
    assert np.isfinite(tot).all()
    drift = np.abs(tot - tot[0]).max()
    assert drift < 1e-2 * np.abs(e[:, 1]).mean(), (drift, e[:, 1].mean())


@pytest.mark.parametrize("tile", [None, (1, 2, 1)])
def test_step_deterministic(tile):
    """Two runs of 7 steps are bit-identical (with the persistent warp kernel, whichever warp takes
    an item computes it the same way)."""
    sysm = systems.small_ljc(2500, 37.5, 12.0, seed=31)
    p = sysm.params(table_bins=512)
    out = []
    for _ in range(2):
        with m.Context(p) as ctx:
            if tile is not None:
                ctx.set_tile(*tile)
            ctx.set_state(sysm.pos[:, 0], sysm.pos[:, 1], sysm.pos[:, 2], sysm.vel, sysm.q, sysm.type)
            ctx.step(7)
            out.append(ctx.state())
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def _ref_lines():
    return (GOLDEN / "cmodel_ref_output.txt").read_text().splitlines()


def test_cmodel_run_matches_reference_binary():
    """mdrl_cmodel_run on the PDB the reference C model read: every printed energy line equal to
    the unmodified reference binary's stdout (fixture), and bit-equal to the oracle's restatement."""
    pos = oracle.read_pdb_like_reference(GOLDEN / "cmodel_input.pdb", 500)
    p, v, e, cnt = m.cmodel_run(pos, np.zeros_like(pos), 100, counts=True)
    lines = [f"Iteration {i}, System energy is {e[i, 0]:f}, Kinetic Energy is {e[i, 1]:f}" for i in range(100)]
    assert lines == _ref_lines()
    po, vo, eo, co = oracle.cmodel_run(pos, np.zeros_like(pos), 100)
    assert np.array_equal(e.view(np.uint32), eo.view(np.uint32))
    assert np.array_equal(p.view(np.uint32), po.view(np.uint32))
    assert np.array_equal(cnt, co)


def test_md_evaluation_model_entry_point():
    """int MD_Evaluation_Model(void) in a child process: stdout equal to the reference's."""
    code = ("import sys; sys.path.insert(0, %r); import sc2019_md_gb300 as m; "
            "sys.exit(0 if m.md_evaluation_model() == 1 else 3)" % str(ROOT))
    env = dict(os.environ, MDRL_INPUT=str(GOLDEN / "cmodel_input.pdb"))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.splitlines() == _ref_lines()
    env["MDRL_INPUT"] = str(GOLDEN / "missing.pdb")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 3
