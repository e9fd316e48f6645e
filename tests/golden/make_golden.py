"""Generate the golden fixtures of tests/golden/ from the reference project.

Run where the reference tree is mounted, naming it in MDRL_REFERENCE:
    MDRL_REFERENCE=<reference project root> python tests/golden/make_golden.py
Every fixture is derived from the reference's own files or from the unmodified reference C model
(oracle/_ref/cmodel_ref, built by oracle/build_ref.sh); nothing here is read at test time
except the .npz/.txt files it writes.

  kat1_pairs.npz   MatlabScripts/VERIFICATION_REFERENCE_OUTPUT.txt (per-pair r2, dx, dy, dz, F,
                   Fx, Fy, Fz as FP32 bits for the first 100 x 100 ApoA1 atoms) and the ROM images
                   OpenCL_HDL_Lib/HDL_Source/c{0,1}_{14,8}.hex (14 segments x 256 bins from 2^-6)
  kat2_cells.npz   MatlabScripts/input_positions_ljargon_20000_box_58_49_49.txt (as integer
                   micro-Angstrom, exactly the 6-decimal text) and the 27
                   cell_ini_file_{1..3}_{1..3}_{1..3}.txt (count and FP32 bits, cell order)
  kat3_tables.npz  MatlabScripts/c{0,1}_{14,8,12,6,3,1}.txt (LJArgon 1st-order tables:
                   sigma 2.1, eps 1.995996^2, 9 segments x 256 bins from 2^-2)
  cmodel_*.txt     a seeded 500-atom argon PDB and the stdout of the unmodified reference C model
                   run on it (100 iterations)
  cell_images_20k.json  SHA-256 and particle count of the 64 RTL cell-memory images
                   MatlabScripts/cell_ini_file_gen/cell_ini_file_{1..4}_{1..4}_{1..4}.{mif,hex}
                   (built by the reference from the same 20k positions, 7 x 6 x 6 cells of 8.5 A)
  pair_stream_222.json  SHA-256 of a canonical form of MatlabScripts/VERIFICATION_PARTICLE_PAIR_INPUT.txt
                   (the RTL pair generator's input stream for home cell (2,2,2) of the 20k LJArgon
                   set: per reference particle and cycle the 8 filters' neighbour IDs, valid bits,
                   the reference position and the valid neighbours' positions; invalid slots print
                   stale reservoir data there and are left out), with its line count
  energy_20k.json  step-1 energies of the reference golden model's 20k LJArgon runs
                   (MatlabScripts/ICS19Results/{Double,Single,Interpolation}_PBC_20k.txt: potential,
                   kinetic, total as printed; sigma 2.1 A, eps 1.995996^2, rc 8.5 A, 59.5 x 51 x 51 A)
  dhfr_bonded.npz  the bonded terms of MatlabScripts/DHFR_23k_Input_Dataset/prmtop as
                   formats.amber_bonded returns them (atoms, parameter-type index, parameter table)
                   and the inpcrd positions wrapped into the 62.23 A box (FP32)
  amber_dhfr.json  a digest of MatlabScripts/DHFR_23k_Input_Dataset/{prmtop,inpcrd}: file SHA-256,
                   pointers, box, net charge, the first atoms' fields and the 16 x 16 LJ A / B
                   (checked by the readers' tests when the reference tree is present)

Select fixtures by name on the command line (default: all).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
if not os.environ.get("MDRL_REFERENCE"):
    raise SystemExit("set MDRL_REFERENCE to the reference project's root")
REF = Path(os.environ["MDRL_REFERENCE"])
SC = REF / "Range_Limited_demo" / "SourceCode"
MS = SC / "MatlabScripts"
HDL = SC / "OpenCL_HDL_Lib" / "HDL_Source"


def hex_to_u32(h: str) -> int:
    return int(h, 16) & 0xFFFFFFFF


def read_intel_hex(path: Path, depth: int) -> np.ndarray:
    """Intel-HEX ROM image of 32-bit words (one data record per address)."""
    out = np.zeros(depth, np.uint32)
    seen = np.zeros(depth, bool)
    for line in path.read_text().split():
        line = line.strip()
        if not line.startswith(":"):
            continue
        n = int(line[1:3], 16)
        addr = int(line[3:7], 16)
        rtype = int(line[7:9], 16)
        if rtype != 0:
            continue
        assert n == 4, line
        out[addr] = int(line[9:17], 16)
        seen[addr] = True
    assert seen.all(), f"{path}: missing addresses"
    return out


def kat1() -> None:
    text = (MS / "VERIFICATION_REFERENCE_OUTPUT.txt").read_text().replace("\r", "")
    lines = [l for l in text.split("\n") if l.strip()]
    pair_re = re.compile(r"\(([0-9A-F]+),([0-9A-F]+),([0-9A-F]+)\),\(([0-9A-F]+),([0-9A-F]+),([0-9A-F]+)\):"
                         r"\s*([0-9A-F]+)\s+([0-9A-F]+)\s+([0-9A-F]+)\s+([0-9A-F]+)")
    dist_re = re.compile(r"Distance info:\s*([0-9A-F]+),\s*([0-9A-F]+),\s*([0-9A-F]+),\s*([0-9A-F]+)")
    rows = []
    k = 2
    while k < len(lines):
        m = pair_re.search(lines[k])
        d = dist_re.search(lines[k + 1])
        assert m and d, lines[k]
        rows.append([hex_to_u32(g) for g in m.groups()] + [hex_to_u32(g) for g in d.groups()])
        k += 2
    a = np.asarray(rows, np.uint32)
    assert a.shape == (10000, 14), a.shape
    pos = a[::100, 0:3].copy()                 # reference particle i = row // 100
    assert (a[:100, 3:6] == pos).all()          # neighbour j = row % 100 (same 100 atoms)
    expect = a[:, 6:14]                         # F, Fx, Fy, Fz, r2, dx, dy, dz
    tabs = {name: read_intel_hex(HDL / f"{name}.hex", 14 * 256) for name in ("c0_14", "c1_14", "c0_8", "c1_8")}
    np.savez_compressed(HERE / "kat1_pairs.npz", pos=pos, expect=expect, **tabs)
    print("kat1:", expect.shape, int((expect[:, 0] != 0).sum()), "nonzero forces")


def kat2() -> None:
    raw = []
    for line in (MS / "input_positions_ljargon_20000_box_58_49_49.txt").read_text().split("\n"):
        f = line.split()
        if len(f) == 4:
            raw.append([int(round(float(v) * 1e6)) for v in f[1:]])
    micro = np.asarray(raw, np.int64)
    assert micro.shape == (20000, 3)
    counts = np.zeros((3, 3, 3), np.int32)
    bits = {}
    for cx in range(1, 4):
        for cy in range(1, 4):
            for cz in range(1, 4):
                t = (MS / f"cell_ini_file_{cx}_{cy}_{cz}.txt").read_text().replace("\r", "")
                n = int(re.search(r"Num Particles In the Cell : (\d+)", t).group(1))
                hx = re.findall(r"HEX \d+ : ([0-9A-F]+)\s+([0-9A-F]+)\s+([0-9A-F]+)", t)
                assert len(hx) == n
                counts[cx - 1, cy - 1, cz - 1] = n
                # file columns are (z, y, x); stored here as (x, y, z)
                bits[f"c{cx}{cy}{cz}"] = np.asarray([[hex_to_u32(x), hex_to_u32(y), hex_to_u32(z)]
                                                      for (z, y, x) in hx], np.uint32)
    np.savez_compressed(HERE / "kat2_cells.npz", micro=micro, counts=counts, **bits)
    print("kat2:", int(counts.sum()), "particles in the 27 cells")


def kat3() -> None:
    out = {}
    for f in ("14", "8", "12", "6", "3", "1"):
        for c in ("0", "1"):
            # printed with 25 decimals, which truncates the smallest coefficients: keep FP64
            out[f"c{c}_{f}"] = np.asarray([float(v) for v in (MS / f"c{c}_{f}.txt").read_text().split()],
                                          np.float64)
    np.savez_compressed(HERE / "kat3_tables.npz", **out)
    print("kat3:", {k: v.shape for k, v in out.items()}["c0_14"])


def cmodel() -> None:
    exe = REPO / "oracle" / "_ref" / "cmodel_ref"
    if not exe.exists():
        subprocess.run(["sh", str(REPO / "oracle" / "build_ref.sh")], check=True)
    rng = np.random.default_rng(20191117)
    # 250 close argon dimers (0.33-0.55 A apart, the reference's sigma is 0.335 A) at random
    # centres in the reference's 24 A box: forces and kinetic energy are large enough for the
    # printed six decimals to carry many significant digits.
    centres = rng.uniform(1.0, 23.0, (250, 3))
    direc = rng.standard_normal((250, 3))
    direc /= np.linalg.norm(direc, axis=1, keepdims=True)
    sep = rng.uniform(0.375, 0.385, 250)
    pos = np.concatenate([centres - 0.5 * sep[:, None] * direc, centres + 0.5 * sep[:, None] * direc])
    pdb = HERE / "cmodel_input.pdb"
    with open(pdb, "w") as fh:
        for k in range(5):
            fh.write(f"REMARK   {k + 1} synthetic argon dimers for the C-model differential test\n")
        for i, (x, y, z) in enumerate(pos):
            fh.write(f"ATOM  {i + 1:5d}  AR   AR A{i + 1:4d}    {x:8.3f}{y:8.3f}{z:8.3f}  1.00  0.00\n")
    res = subprocess.run([str(exe)], env=dict(os.environ, MDRL_REF_PDB=str(pdb)),
                         capture_output=True, text=True, check=True)
    (HERE / "cmodel_ref_output.txt").write_text(res.stdout)
    print("cmodel:", res.stdout.splitlines()[-1])


def cell_images() -> None:
    import hashlib
    import json
    out = {}
    for x in range(1, 5):
        for y in range(1, 5):
            for z in range(1, 5):
                base = MS / "cell_ini_file_gen" / f"cell_ini_file_{x}_{y}_{z}"
                mif = base.with_suffix(".mif").read_bytes()
                count = int(re.search(rb"\n0 : ([0-9A-F]{24});", mif).group(1), 16)
                out[f"{x}_{y}_{z}"] = {"count": count,
                                       "mif": hashlib.sha256(mif).hexdigest(),
                                       "hex": hashlib.sha256(base.with_suffix(".hex").read_bytes()).hexdigest()}
    (HERE / "cell_images_20k.json").write_text(json.dumps(out, indent=0, sort_keys=True) + "\n")
    print("cell_images:", len(out), "cells")


def amber() -> None:
    import hashlib
    import json
    sys.path.insert(0, str(REPO))
    from sc2019_md_gb300 import formats
    d = MS / "DHFR_23k_Input_Dataset"
    prm = formats.read_amber_prmtop(d / "prmtop")
    crd = formats.read_amber_inpcrd(d / "inpcrd")
    nb = formats.amber_nonbonded(prm)
    out = {"prmtop_sha256": hashlib.sha256((d / "prmtop").read_bytes()).hexdigest(),
           "inpcrd_sha256": hashlib.sha256((d / "inpcrd").read_bytes()).hexdigest(),
           "pointers": prm["POINTERS"], "box": [float(v) for v in crd["box"]],
           "net_charge_e": float(nb["charge"].sum()), "mass_total": float(nb["mass"].sum()),
           "first_atoms": [{"name": prm["ATOM_NAME"][i], "charge_e": float(nb["charge"][i]),
                            "type": int(nb["type"][i]), "mass": float(nb["mass"][i]),
                            "pos": [float(v) for v in crd["pos"][i]], "vel": [float(v) for v in crd["vel"][i]]}
                           for i in range(3)],
           "residues_first": prm["RESIDUE_LABEL"][:5],
           "A": nb["A"].tolist(), "B": nb["B"].tolist()}
    (HERE / "amber_dhfr.json").write_text(json.dumps(out, indent=0) + "\n")
    print("amber:", out["pointers"]["NATOM"], "atoms")


def pair_stream() -> None:
    import hashlib
    import json
    sys.path.insert(0, str(REPO))
    sys.path.insert(0, str(REPO / "tests"))
    from helpers import pair_stream_canon_from_text
    text = (MS / "VERIFICATION_PARTICLE_PAIR_INPUT.txt").read_bytes().decode()
    canon = pair_stream_canon_from_text(text)
    out = {"lines": len(canon), "sha256": hashlib.sha256("\n".join(canon).encode()).hexdigest()}
    (HERE / "pair_stream_222.json").write_text(json.dumps(out, indent=0) + "\n")
    print("pair_stream:", out["lines"], "lines")


def energy_20k() -> None:
    import json
    out = {}
    for name in ("Double", "Single", "Interpolation"):
        f = (MS / "ICS19Results" / f"{name}_PBC_20k.txt").read_text().splitlines()[0].split()
        out[name] = {"step": int(f[0]), "potential": float(f[1]), "kinetic": float(f[2]), "total": float(f[3])}
    (HERE / "energy_20k.json").write_text(json.dumps(out, indent=0) + "\n")
    print("energy_20k:", out["Double"])


def dhfr_bonded() -> None:
    """The DHFR topology's bonded terms (via formats.amber_bonded: atoms, 0-based parameter-type
    index, the parameter tables) and the inpcrd positions wrapped into the box as FP32."""
    sys.path.insert(0, str(REPO))
    from sc2019_md_gb300 import formats as F
    d = MS / "DHFR_23k_Input_Dataset"
    prm = F.read_amber_prmtop(d / "prmtop")
    crd = F.read_amber_inpcrd(d / "inpcrd")
    b = F.amber_bonded(prm)
    from sc2019_md_gb300 import systems
    out = {"box": np.asarray(crd["box"][:3], np.float64)}
    L = out["box"]
    out["pos"] = systems.wrap_into_box(np.mod(np.asarray(crd["pos"], np.float64), L), tuple(L))
    for name, (atoms, params) in b.items():
        table, idx = np.unique(params, axis=0, return_inverse=True)
        out[f"{name}_atoms"] = atoms.astype(np.int32)
        out[f"{name}_type"] = idx.reshape(-1).astype(np.int16)
        out[f"{name}_table"] = table
    np.savez_compressed(HERE / "dhfr_bonded.npz", **out)
    print("dhfr_bonded:", {k: v.shape for k, v in out.items()})


FIXTURES = {"kat1": kat1, "kat2": kat2, "kat3": kat3, "cmodel": cmodel, "cell_images": cell_images,
            "amber": amber, "pair_stream": pair_stream, "energy_20k": energy_20k, "dhfr_bonded": dhfr_bonded}

if __name__ == "__main__":
    if not MS.exists():
        sys.exit(f"reference tree not found at {REF}")
    for name in (sys.argv[1:] or list(FIXTURES)):
        FIXTURES[name]()
