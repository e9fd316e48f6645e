"""Data formats either side of the path (CPU only).

* RTL cell-memory images: from the 20k LJArgon positions (KAT-2 fixture), write_cell_mif and
  write_cell_hex reproduce the reference's 64 cell_ini_file_gen/cell_ini_file_*.{mif,hex} byte for
  byte (SHA-256 fixture); the reference's cell assignment equals the oracle's binning.
* Amber readers: a synthetic topology in both file formats parses to the same fields; with the
  reference tree present, the DHFR dataset parses to the committed digest.
* Amber A/B -> the kernel's per-type-pair multipliers: fscal * r2 equals -r dE/dr.
"""
import hashlib
import json
import os
from pathlib import Path

import numpy as np
import pytest

import oracle
from sc2019_md_gb300 import formats as F
from helpers import GOLDEN, kat2_positions

# the reference project's tree, when a caller names it (MDRL_REFERENCE); the DHFR checks skip without it
REF = Path(os.environ["MDRL_REFERENCE"]) if os.environ.get("MDRL_REFERENCE") else None
DHFR = (REF / "Range_Limited_demo" / "SourceCode" / "MatlabScripts" / "DHFR_23k_Input_Dataset") if REF else Path("/nonexistent")


def _sha(text: str) -> str:
    return hashlib.sha256(text.encode()).hexdigest()


def test_cell_images_reproduce_reference_files():
    pos, _ = kat2_positions()
    cells, outside = F.cell_memories(pos, 8.5, (7, 6, 6))
    assert outside == 0
    expect = json.loads((GOLDEN / "cell_images_20k.json").read_text())
    assert len(expect) == 64
    for key, e in expect.items():
        x, y, z = (int(v) for v in key.split("_"))
        p = cells.get((x, y, z), np.zeros((0, 3), np.float32))
        assert len(p) == e["count"], key
        assert _sha(F.write_cell_mif(None, p)) == e["mif"], key
        assert _sha(F.write_cell_hex(None, p)) == e["hex"], key


def test_cell_assignment_equals_oracle_binning():
    pos, _ = kat2_positions()
    cells, _ = F.cell_memories(pos, 8.5, (7, 6, 6))
    cell_of, start, order, _ = oracle.bin_cells(pos, (7 * 8.5, 6 * 8.5, 6 * 8.5), (7, 6, 6))
    for c in range(7 * 6 * 6):
        key = (c // 36 + 1, (c // 6) % 6 + 1, c % 6 + 1)
        ids = order[start[c]:start[c + 1]]
        got = cells.get(key, np.zeros((0, 3), np.float32))
        assert np.array_equal(got.view(np.uint32), pos[ids].view(np.uint32)), key


def test_cell_image_roundtrip_and_checksums(tmp_path):
    rng = np.random.default_rng(1)
    p = rng.uniform(0, 8.5, (37, 3)).astype(np.float32)
    F.write_cell_mif(tmp_path / "c.mif", p)
    back = F.read_cell_mif(tmp_path / "c.mif")
    assert np.array_equal(back.view(np.uint32), p.view(np.uint32))
    text = F.write_cell_hex(tmp_path / "c.hex", p, depth=100)
    recs = text.strip().split("\r\n")
    assert len(recs) == 101 and recs[-1] == ":00000001FF"
    for a, r in enumerate(recs[:-1]):
        b = bytes.fromhex(r[1:])
        assert sum(b) % 256 == 0 and b[0] == 12 and (b[1] << 8 | b[2]) == a
    with pytest.raises(ValueError):
        F.write_cell_mif(None, np.zeros((100, 3), np.float32), depth=100)


def _synthetic_topology():
    """5 atoms, 2 types, 2 residues: the fields the readers return."""
    return {"NATOM": 5, "NTYPES": 2, "NRES": 2, "names": ["OW", "HW1", "HW2", "AR", "AR"],
            "charge_e": [-0.834, 0.417, 0.417, 0.0, 0.0], "mass": [16.0, 1.008, 1.008, 39.948, 39.948],
            "type": [1, 2, 2, 1, 1], "numex": [2, 1, 0, 0, 0], "ico": [1, 2, 2, 3],
            "acoef": [582000.0, 0.0, 0.0], "bcoef": [595.0, 0.0, 0.0], "labels": ["WAT", "AR"], "ptr": [1, 4],
            # bonded sections: Amber lists atoms as 3 x index, types 1-based; a negative third /
            # fourth dihedral atom flags "no 1-4" / "improper"
            "rk": [553.0, 10.0], "req": [0.9572, 3.8], "tk": [100.0], "teq": [1.824],
            "pk": [1.4, 10.5], "pn": [3.0, 2.0], "phase": [0.0, 3.14159400],
            "bonh": [0, 3, 1, 0, 6, 1], "bona": [9, 12, 2], "theth": [3, 0, 6, 1], "theta": [],
            "phih": [], "phia": [3, 0, -9, 12, 1, 6, 0, 9, -12, 2], "natex": [2, 3, 0]}


def _fmt(vals, kind, width, per_line):
    out, line = [], ""
    for k, v in enumerate(vals):
        line += (f"{v:<{width}s}" if kind == "a" else f"{v:{width}d}" if kind == "i" else f"{v:{width}.8E}")
        if (k + 1) % per_line == 0:
            out.append(line)
            line = ""
    if line or not vals:
        out.append(line)
    return out


def _pointers(t):
    ptr = [0] * 30
    ptr[0], ptr[1], ptr[11] = t["NATOM"], t["NTYPES"], t["NRES"]
    ptr[2], ptr[4], ptr[6] = len(t["bonh"]) // 3, len(t["theth"]) // 4, len(t["phih"]) // 5
    ptr[3] = ptr[12] = len(t["bona"]) // 3
    ptr[5] = ptr[13] = len(t["theta"]) // 4
    ptr[7] = ptr[14] = len(t["phia"]) // 5
    ptr[10] = len(t["natex"])
    ptr[15], ptr[16], ptr[17], ptr[18] = len(t["rk"]), len(t["tk"]), len(t["pk"]), 1
    return ptr


def _write_old(path, t):
    ptr = _pointers(t)
    q = [c * F.AMBER_CHARGE_SCALE for c in t["charge_e"]]
    lines = [" " * 80] + _fmt(ptr, "i", 6, 12) + _fmt(t["names"], "a", 4, 20) + _fmt(q, "e", 16, 5) + \
        _fmt(t["mass"], "e", 16, 5) + _fmt(t["type"], "i", 6, 12) + _fmt(t["numex"], "i", 6, 12) + \
        _fmt(t["ico"], "i", 6, 12) + _fmt(t["labels"], "a", 4, 20) + _fmt(t["ptr"], "i", 6, 12)
    for key in ("rk", "req", "tk", "teq", "pk", "pn", "phase"):
        lines += _fmt(t[key], "e", 16, 5)
    lines += _fmt([1.0], "e", 16, 5)                   # SOLTY
    lines += _fmt(t["acoef"], "e", 16, 5) + _fmt(t["bcoef"], "e", 16, 5)
    for key in ("bonh", "bona", "theth", "theta", "phih", "phia", "natex"):
        lines += _fmt(t[key], "i", 6, 12)
    Path(path).write_text("\n".join(lines) + "\n")


def _write_flags(path, t):
    ptr = _pointers(t)
    q = [c * F.AMBER_CHARGE_SCALE for c in t["charge_e"]]
    sec = [("POINTERS", "10I8", ptr, "i", 8, 10), ("ATOM_NAME", "20a4", t["names"], "a", 4, 20),
           ("CHARGE", "5E16.8", q, "e", 16, 5), ("MASS", "5E16.8", t["mass"], "e", 16, 5),
           ("ATOM_TYPE_INDEX", "10I8", t["type"], "i", 8, 10),
           ("NONBONDED_PARM_INDEX", "10I8", t["ico"], "i", 8, 10),
           ("RESIDUE_LABEL", "20a4", t["labels"], "a", 4, 20), ("RESIDUE_POINTER", "10I8", t["ptr"], "i", 8, 10),
           ("BOND_FORCE_CONSTANT", "5E16.8", t["rk"], "e", 16, 5), ("BOND_EQUIL_VALUE", "5E16.8", t["req"], "e", 16, 5),
           ("ANGLE_FORCE_CONSTANT", "5E16.8", t["tk"], "e", 16, 5), ("ANGLE_EQUIL_VALUE", "5E16.8", t["teq"], "e", 16, 5),
           ("DIHEDRAL_FORCE_CONSTANT", "5E16.8", t["pk"], "e", 16, 5),
           ("DIHEDRAL_PERIODICITY", "5E16.8", t["pn"], "e", 16, 5), ("DIHEDRAL_PHASE", "5E16.8", t["phase"], "e", 16, 5),
           ("LENNARD_JONES_ACOEF", "5E16.8", t["acoef"], "e", 16, 5),
           ("LENNARD_JONES_BCOEF", "5E16.8", t["bcoef"], "e", 16, 5),
           ("BONDS_INC_HYDROGEN", "10I8", t["bonh"], "i", 8, 10), ("BONDS_WITHOUT_HYDROGEN", "10I8", t["bona"], "i", 8, 10),
           ("ANGLES_INC_HYDROGEN", "10I8", t["theth"], "i", 8, 10),
           ("ANGLES_WITHOUT_HYDROGEN", "10I8", t["theta"], "i", 8, 10),
           ("DIHEDRALS_INC_HYDROGEN", "10I8", t["phih"], "i", 8, 10),
           ("DIHEDRALS_WITHOUT_HYDROGEN", "10I8", t["phia"], "i", 8, 10),
           ("EXCLUDED_ATOMS_LIST", "10I8", t["natex"], "i", 8, 10)]
    lines = ["%VERSION  VERSION_STAMP = V0001.000  DATE = 01/01/20  00:00:00"]
    for name, fm, vals, kind, w, pl in sec:
        lines += [f"%FLAG {name}", f"%FORMAT({fm})"] + _fmt(vals, kind, w, pl)
    Path(path).write_text("\n".join(lines) + "\n")


@pytest.mark.parametrize("writer", [_write_old, _write_flags])
def test_amber_prmtop_both_formats(tmp_path, writer):
    t = _synthetic_topology()
    writer(tmp_path / "top", t)
    prm = F.read_amber_prmtop(tmp_path / "top")
    assert prm["POINTERS"]["NATOM"] == 5 and prm["POINTERS"]["NTYPES"] == 2
    assert prm["ATOM_NAME"] == t["names"] and prm["RESIDUE_LABEL"] == t["labels"]
    nb = F.amber_nonbonded(prm)
    assert np.allclose(nb["charge"], t["charge_e"], rtol=0, atol=1e-8)
    assert list(nb["type"]) == [0, 1, 1, 0, 0]
    assert nb["A"][0, 0] == 582000.0 and nb["B"][0, 0] == 595.0 and nb["A"][1, 1] == 0.0
    b = F.amber_bonded(prm)
    assert b["bonds"][0].tolist() == [[0, 1], [0, 2], [3, 4]]
    assert np.allclose(b["bonds"][1], [[553.0, 0.9572], [553.0, 0.9572], [10.0, 3.8]])
    assert b["angles"][0].tolist() == [[1, 0, 2]] and np.allclose(b["angles"][1], [[100.0, 1.824, 0, 0]])
    assert b["dihedrals"][0].tolist() == [[1, 0, 3, 4], [2, 0, 3, 4]]
    assert np.allclose(b["dihedrals"][1], [[1.4, 3.0, 0.0], [10.5, 2.0, -3.141594]])
    assert prm["EXCLUDED_ATOMS_LIST"] == t["natex"]


def test_amber_inpcrd(tmp_path):
    rng = np.random.default_rng(2)
    pos = rng.uniform(0, 30, (5, 3))
    vel = rng.uniform(-1, 1, (5, 3))
    vals = list(pos.ravel()) + list(vel.ravel())
    lines = ["synthetic", "    5  0.1000000E+01"]
    for k in range(0, len(vals), 6):
        lines.append("".join(f"{v:12.7f}" for v in vals[k:k + 6]))
    lines.append("".join(f"{v:12.7f}" for v in (30.0, 31.0, 32.0, 90.0, 90.0, 90.0)))
    (tmp_path / "crd").write_text("\n".join(lines) + "\n")
    c = F.read_amber_inpcrd(tmp_path / "crd")
    assert c["natom"] == 5 and c["time"] == 1.0
    assert np.allclose(c["pos"], pos, atol=1e-7) and np.allclose(c["vel"], vel, atol=1e-7)
    assert list(c["box"][:3]) == [30.0, 31.0, 32.0]


@pytest.mark.skipif(not DHFR.exists(), reason="reference tree not mounted")
def test_amber_dhfr_matches_digest():
    d = json.loads((GOLDEN / "amber_dhfr.json").read_text())
    assert hashlib.sha256((DHFR / "prmtop").read_bytes()).hexdigest() == d["prmtop_sha256"]
    prm = F.read_amber_prmtop(DHFR / "prmtop")
    crd = F.read_amber_inpcrd(DHFR / "inpcrd")
    nb = F.amber_nonbonded(prm)
    assert prm["POINTERS"] == d["pointers"]
    assert list(crd["box"]) == d["box"]
    assert abs(nb["charge"].sum() - d["net_charge_e"]) < 1e-9
    assert np.array_equal(nb["A"], np.asarray(d["A"])) and np.array_equal(nb["B"], np.asarray(d["B"]))
    for i, a in enumerate(d["first_atoms"]):
        assert prm["ATOM_NAME"][i] == a["name"] and int(nb["type"][i]) == a["type"]
        assert list(crd["pos"][i]) == a["pos"] and list(crd["vel"][i]) == a["vel"]
    assert len(crd["pos"]) == d["pointers"]["NATOM"] == 23558


@pytest.mark.skipif(not DHFR.exists(), reason="reference tree not mounted")
def test_amber_dhfr_bonded_matches_fixture():
    """formats.amber_bonded on the DHFR topology reproduces the committed fixture, with the
    pointer counts of terms."""
    prm = F.read_amber_prmtop(DHFR / "prmtop")
    b = F.amber_bonded(prm)
    d = np.load(GOLDEN / "dhfr_bonded.npz")
    P = prm["POINTERS"]
    counts = {"bonds": P["NBONH"] + P["NBONA"], "angles": P["NTHETH"] + P["NTHETA"],
              "dihedrals": P["NPHIH"] + P["NPHIA"]}
    for name, (atoms, params) in b.items():
        assert len(atoms) == counts[name]
        assert np.array_equal(atoms, d[f"{name}_atoms"])
        assert np.array_equal(params, d[f"{name}_table"][d[f"{name}_type"]])
        assert atoms.min() >= 0 and atoms.max() < P["NATOM"]


def test_pair_coefficients_from_AB_are_forces():
    A = np.array([[582000.0, 1.2e5], [1.2e5, 3.0e4]])
    B = np.array([[595.0, 300.0], [300.0, 120.0]])
    pc = F.pair_coefficients_from_AB(A, B)
    r = 3.1
    for a in range(2):
        for b in range(2):
            A14, B8, A12, B6 = pc[a * 2 + b]
            E = lambda x: A[a, b] / x ** 12 - B[a, b] / x ** 6
            dEdr = (E(r + 1e-6) - E(r - 1e-6)) / 2e-6
            fscal = A14 * r ** -14 + B8 * r ** -8
            assert abs(fscal * r - (-dEdr)) <= 1e-6 * abs(dEdr)
            assert abs(A12 * r ** -12 + B6 * r ** -6 - E(r)) <= 1e-12 * abs(E(r)) + 1e-15
