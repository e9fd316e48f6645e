"""Data formats on either side of the range-limited force path: the reference's input datasets
and the memory-initialisation files its RTL is cross-checked with.

Readers
  read_named_xyz     "<name> x y z" per line (LJArgon inputs, e.g.
                     MatlabScripts/20k_Input_Dataset/input_positions_ljargon_20000_box_58_49_49.txt),
                     parsed as the reference's textscan('%s %f64 %f64 %f64') does
                     (MatlabScripts/GenInputCellList_LJArgon.m:72-83)
  read_xyz           "x y z" per line (MatlabScripts/input_positions_ApoA1.txt)
  shift_to_origin    subtract the per-axis minimum in FP64, then store FP32
                     (GenInputCellList_LJArgon.m:86-98)
  read_amber_inpcrd  Amber restart/coordinate file: title, atom count, 6F12.7 coordinates,
                     optional velocities, box line (MatlabScripts/DHFR_23k_Input_Dataset/inpcrd)
  read_amber_prmtop  Amber topology, both the fixed-order format without %FLAG sections
                     (MatlabScripts/DHFR_23k_Input_Dataset/prmtop) and the %FLAG format
  amber_nonbonded    per-atom type, charge (e) and mass, and the per-type-pair LJ A / B of a topology
  amber_bonded       the topology's bonds, angles and dihedrals as mdrl_set_bonded terms

Writers (the RTL cell-memory images, cell_ini_file_<x>_<y>_<z>.*)
  write_cell_mif     Altera MIF written by GenInputCellList_LJArgon.m:142-203: address 0 holds the
                     particle count, addresses 1.. hold {z, y, x} as IEEE-754 single hex, the rest
                     zero, DEPTH lines in all
  write_cell_hex     the same memory as Intel HEX (one 12-byte data record per word, word
                     addresses, two's-complement checksums, end-of-file record), the form
                     Quartus' mif2hex makes of the MIF (cell_ini_file_gen/GenInputCellList_LJArgon.m:146,178)
  cell_memories      per-cell position lists in the reference's 1-based cell numbering, in input
                     order, from positions (GenInputCellList_LJArgon.m:100-136)
"""
from __future__ import annotations

import re
import struct
from pathlib import Path

import numpy as np

AMBER_CHARGE_SCALE = 18.2223   # Amber stores q * 18.2223 (e -> sqrt(kcal A / mol))


# ---- position files -------------------------------------------------------------------------

def read_named_xyz(path) -> tuple[list, np.ndarray]:
    names, xyz = [], []
    with open(path, "r") as f:
        for line in f:
            parts = line.split()
            if len(parts) < 4:
                continue
            names.append(parts[0])
            xyz.append([float(parts[1]), float(parts[2]), float(parts[3])])
    return names, np.asarray(xyz, dtype=np.float64)


def read_xyz(path) -> np.ndarray:
    xyz = []
    with open(path, "r") as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 3:
                xyz.append([float(parts[0]), float(parts[1]), float(parts[2])])
    return np.asarray(xyz, dtype=np.float64)


def shift_to_origin(xyz64: np.ndarray) -> np.ndarray:
    xyz64 = np.asarray(xyz64, dtype=np.float64)
    return (xyz64 - xyz64.min(axis=0)).astype(np.float32)


# ---- cell memories --------------------------------------------------------------------------

def cell_memories(pos32: np.ndarray, cutoff: float, ncell) -> tuple[dict, int]:
    """{(cx, cy, cz) 1-based: float32 (m, 3) positions in input order} and the number of particles
    outside the grid.  cell = floor(pos / rc) + 1 in FP32, a coordinate of exactly 0 -> cell 1."""
    pos32 = np.asarray(pos32, dtype=np.float32)
    rc = np.float32(cutoff)
    c = np.floor(pos32 / rc).astype(np.int64) + 1
    c[pos32 == 0] = 1
    nc = np.asarray(ncell, dtype=np.int64)
    ok = np.all((c >= 1) & (c <= nc), axis=1)
    cells: dict = {}
    for i in np.nonzero(ok)[0]:
        cells.setdefault((int(c[i, 0]), int(c[i, 1]), int(c[i, 2])), []).append(i)
    return {k: pos32[v] for k, v in cells.items()}, int((~ok).sum())


def _f32hex(v) -> str:
    return "%08X" % struct.unpack(">I", struct.pack(">f", float(np.float32(v))))[0]


def _words(pos32: np.ndarray, depth: int) -> list:
    """The cell memory as 96-bit words (24 hex digits): count, then {z, y, x}, then zeros."""
    m = len(pos32)
    if m > depth - 1:
        raise ValueError(f"{m} particles do not fit a cell memory of depth {depth}")
    if m > 0xFFFFFF:
        raise ValueError("particle count does not fit the count word")
    words = ["%08X%08X%08X" % (0, 0, m)]
    for p in np.asarray(pos32, dtype=np.float32):
        words.append(_f32hex(p[2]) + _f32hex(p[1]) + _f32hex(p[0]))
    words += ["0" * 24] * (depth - 1 - m)
    return words


def write_cell_mif(path, pos32: np.ndarray, depth: int = 100, width: int = 96, newline: str = "\r\n") -> str:
    """Write (and return) the MIF image of one cell memory; pos32 is (m, 3) x, y, z."""
    lines = [f"DEPTH = {depth};", f"WIDTH = {width};", "ADDRESS_RADIX = DEC;", "DATA_RADIX = HEX;",
             "CONTENT", "BEGIN"]
    lines += [f"{a} : {w};" for a, w in enumerate(_words(pos32, depth))]
    lines.append("END;")
    text = newline.join(lines) + newline
    if path is not None:
        with open(path, "w", newline="") as f:
            f.write(text)
    return text


def _ihex_record(addr: int, rtype: int, data: bytes) -> str:
    body = bytes([len(data), (addr >> 8) & 0xFF, addr & 0xFF, rtype]) + data
    return ":" + body.hex().upper() + "%02X" % ((-sum(body)) & 0xFF)


def write_cell_hex(path, pos32: np.ndarray, depth: int = 100, newline: str = "\r\n") -> str:
    """Write (and return) the Intel HEX image of one cell memory (12-byte words, word addresses)."""
    if depth > 0x10000:
        raise ValueError("word addresses beyond 16 bits need extended records")
    lines = [_ihex_record(a, 0, bytes.fromhex(w)) for a, w in enumerate(_words(pos32, depth))]
    lines.append(_ihex_record(0, 1, b""))
    text = newline.join(lines) + newline
    if path is not None:
        with open(path, "w", newline="") as f:
            f.write(text)
    return text


def read_cell_mif(path) -> np.ndarray:
    """Positions (m, 3) x, y, z stored in a cell MIF (the inverse of write_cell_mif)."""
    words = {}
    for line in Path(path).read_text().splitlines():
        mm = re.match(r"\s*(\d+)\s*:\s*([0-9A-Fa-f]+);", line)
        if mm:
            words[int(mm.group(1))] = mm.group(2)
    m = int(words[0], 16)
    out = np.zeros((m, 3), np.float32)
    for a in range(1, m + 1):
        w = words[a]
        z, y, x = (struct.unpack(">f", bytes.fromhex(w[8 * k:8 * k + 8]))[0] for k in range(3))
        out[a - 1] = (x, y, z)
    return out


# ---- Amber ----------------------------------------------------------------------------------

def read_amber_inpcrd(path) -> dict:
    """{'title', 'natom', 'time', 'pos' (n,3) f64, 'vel' (n,3) f64 or None, 'box' (6,) or None}."""
    lines = Path(path).read_text().splitlines()
    head = lines[1].split()
    natom = int(head[0])
    time = float(head[1]) if len(head) > 1 else None
    vals = []
    for line in lines[2:]:
        for k in range(0, len(line.rstrip()), 12):
            field = line[k:k + 12].strip()
            if field:
                vals.append(float(field))
    vals = np.asarray(vals, dtype=np.float64)
    n3 = 3 * natom
    pos = vals[:n3].reshape(natom, 3)
    rest = vals[n3:]
    vel = box = None
    if len(rest) >= n3:
        vel = rest[:n3].reshape(natom, 3)
        rest = rest[n3:]
    if len(rest) in (3, 6):
        box = rest
    return {"title": lines[0].rstrip(), "natom": natom, "time": time, "pos": pos, "vel": vel, "box": box}


_POINTER_NAMES = ["NATOM", "NTYPES", "NBONH", "MBONA", "NTHETH", "MTHETA", "NPHIH", "MPHIA", "NHPARM",
                  "NPARM", "NNB", "NRES", "NBONA", "NTHETA", "NPHIA", "NUMBND", "NUMANG", "NPTRA",
                  "NATYP", "NPHB", "IFPERT", "NBPER", "NGPER", "NDPER", "MBPER", "MGPER", "MDPER",
                  "IFBOX", "NMXRS", "IFCAP"]


def _fixed_fields(lines, start, count, width, per_line, kind):
    """`count` fixed-width fields from lines[start:], `per_line` a line; returns (values, next line).
    A section of zero items still occupies one (empty) line."""
    out = []
    k = start
    if count == 0:
        return out, start + 1
    while len(out) < count:
        line = lines[k]
        for j in range(per_line):
            if len(out) == count:
                break
            field = line[j * width:(j + 1) * width]
            if kind == "a":
                out.append(field.strip())
            elif kind == "i":
                out.append(int(field))
            else:
                out.append(float(field))
        k += 1
    return out, k


def read_amber_prmtop(path) -> dict:
    """Sections of an Amber topology by their %FLAG names (both file formats): POINTERS (dict),
    ATOM_NAME, CHARGE, MASS, ATOM_TYPE_INDEX, NUMBER_EXCLUDED_ATOMS, NONBONDED_PARM_INDEX,
    RESIDUE_LABEL, RESIDUE_POINTER, the bond / angle / dihedral parameter tables, SOLTY,
    LENNARD_JONES_ACOEF, LENNARD_JONES_BCOEF, BONDS_*, ANGLES_*, DIHEDRALS_* (with and without
    hydrogen), EXCLUDED_ATOMS_LIST (and, in the %FLAG format, every other section)."""
    lines = Path(path).read_text().splitlines()
    if any(l.startswith("%FLAG") for l in lines[:10]):
        return _read_prmtop_flags(lines)
    ptr, k = _fixed_fields(lines, 1, 30, 6, 12, "i")
    P = dict(zip(_POINTER_NAMES, ptr))
    n, t, nres = P["NATOM"], P["NTYPES"], P["NRES"]
    out = {"POINTERS": P}
    order = [("ATOM_NAME", n, 4, 20, "a"), ("CHARGE", n, 16, 5, "e"), ("MASS", n, 16, 5, "e"),
             ("ATOM_TYPE_INDEX", n, 6, 12, "i"), ("NUMBER_EXCLUDED_ATOMS", n, 6, 12, "i"),
             ("NONBONDED_PARM_INDEX", t * t, 6, 12, "i"), ("RESIDUE_LABEL", nres, 4, 20, "a"),
             ("RESIDUE_POINTER", nres, 6, 12, "i"), ("BOND_FORCE_CONSTANT", P["NUMBND"], 16, 5, "e"),
             ("BOND_EQUIL_VALUE", P["NUMBND"], 16, 5, "e"), ("ANGLE_FORCE_CONSTANT", P["NUMANG"], 16, 5, "e"),
             ("ANGLE_EQUIL_VALUE", P["NUMANG"], 16, 5, "e"), ("DIHEDRAL_FORCE_CONSTANT", P["NPTRA"], 16, 5, "e"),
             ("DIHEDRAL_PERIODICITY", P["NPTRA"], 16, 5, "e"), ("DIHEDRAL_PHASE", P["NPTRA"], 16, 5, "e"),
             ("SOLTY", P["NATYP"], 16, 5, "e"), ("LENNARD_JONES_ACOEF", t * (t + 1) // 2, 16, 5, "e"),
             ("LENNARD_JONES_BCOEF", t * (t + 1) // 2, 16, 5, "e"),
             ("BONDS_INC_HYDROGEN", 3 * P["NBONH"], 6, 12, "i"), ("BONDS_WITHOUT_HYDROGEN", 3 * P["NBONA"], 6, 12, "i"),
             ("ANGLES_INC_HYDROGEN", 4 * P["NTHETH"], 6, 12, "i"),
             ("ANGLES_WITHOUT_HYDROGEN", 4 * P["NTHETA"], 6, 12, "i"),
             ("DIHEDRALS_INC_HYDROGEN", 5 * P["NPHIH"], 6, 12, "i"),
             ("DIHEDRALS_WITHOUT_HYDROGEN", 5 * P["NPHIA"], 6, 12, "i"),
             ("EXCLUDED_ATOMS_LIST", P["NNB"], 6, 12, "i")]
    for name, count, width, per_line, kind in order:
        out[name], k = _fixed_fields(lines, k, count, width, per_line, kind)
    return out


_FMT = re.compile(r"\((\d+)([aAiIeEfF])(\d+)(?:\.\d+)?\)")


def _read_prmtop_flags(lines) -> dict:
    out, k = {}, 0
    while k < len(lines):
        if not lines[k].startswith("%FLAG"):
            k += 1
            continue
        name = lines[k].split()[1]
        fm = _FMT.search(lines[k + 1])
        per_line, kind, width = int(fm.group(1)), fm.group(2).lower(), int(fm.group(3))
        k += 2
        vals = []
        while k < len(lines) and not lines[k].startswith("%"):
            line = lines[k]
            for j in range(per_line):
                field = line[j * width:(j + 1) * width]
                if not field.strip():
                    continue
                vals.append(field.strip() if kind == "a" else int(field) if kind == "i" else float(field))
            k += 1
        out[name] = vals
    out["POINTERS"] = dict(zip(_POINTER_NAMES, out["POINTERS"]))
    return out


def amber_nonbonded(prm: dict) -> dict:
    """{'ntypes', 'type' (n,) 0-based, 'charge' (n,) e, 'mass' (n,) amu, 'A' (T,T), 'B' (T,T)}:
    E_LJ(r) = A/r^12 - B/r^6 for the pair's types (via NONBONDED_PARM_INDEX; a negative index
    marks a 10-12 pair, whose A and B are taken as 0 here)."""
    P = prm["POINTERS"]
    T = P["NTYPES"]
    ico = np.asarray(prm["NONBONDED_PARM_INDEX"], dtype=np.int64).reshape(T, T)
    acoef = np.asarray(prm["LENNARD_JONES_ACOEF"], dtype=np.float64)
    bcoef = np.asarray(prm["LENNARD_JONES_BCOEF"], dtype=np.float64)
    A = np.where(ico > 0, acoef[np.maximum(ico, 1) - 1], 0.0)
    B = np.where(ico > 0, bcoef[np.maximum(ico, 1) - 1], 0.0)
    return {"ntypes": T, "type": np.asarray(prm["ATOM_TYPE_INDEX"], dtype=np.int32) - 1,
            "charge": np.asarray(prm["CHARGE"], dtype=np.float64) / AMBER_CHARGE_SCALE,
            "mass": np.asarray(prm["MASS"], dtype=np.float64), "A": A, "B": B}


def amber_bonded(prm: dict) -> dict:
    """The topology's bonded terms in mdrl_set_bonded's forms, terms with hydrogen first:
    {'bonds': (atoms (m, 2), params (m, 2) {k, r0}), 'angles': (atoms (m, 3), params (m, 4)
    {k, theta0, 0, 0}), 'dihedrals': (atoms (m, 4), params (m, 3) {k, n, delta})}.  Amber lists
    atoms as 3 x (0-based index) and types 1-based; its E = PK (1 + cos(PN phi - PHASE)) is
    k = PK, n = |PN|, delta = -PHASE here (the same IUPAC phi).  The signs Amber puts on the third
    and fourth atoms (no 1-4 pair; improper) are dropped: there are no exclusions or 1-4 pairs
    in the pair path.  SHAKE constraints are not applied: every bond is a harmonic term."""
    def terms(with_h, without_h, width):
        a = np.concatenate([np.asarray(prm.get(with_h, []), dtype=np.int64),
                            np.asarray(prm.get(without_h, []), dtype=np.int64)]).reshape(-1, width)
        return np.abs(a[:, :-1]) // 3, a[:, -1] - 1
    ba, bt = terms("BONDS_INC_HYDROGEN", "BONDS_WITHOUT_HYDROGEN", 3)
    aa, at = terms("ANGLES_INC_HYDROGEN", "ANGLES_WITHOUT_HYDROGEN", 4)
    da, dt = terms("DIHEDRALS_INC_HYDROGEN", "DIHEDRALS_WITHOUT_HYDROGEN", 5)
    f = lambda name: np.asarray(prm[name], dtype=np.float64)
    bp = np.stack([f("BOND_FORCE_CONSTANT")[bt], f("BOND_EQUIL_VALUE")[bt]], axis=1)
    ap = np.stack([f("ANGLE_FORCE_CONSTANT")[at], f("ANGLE_EQUIL_VALUE")[at], np.zeros(len(at)),
                   np.zeros(len(at))], axis=1)
    dp = np.stack([f("DIHEDRAL_FORCE_CONSTANT")[dt], np.abs(f("DIHEDRAL_PERIODICITY")[dt]),
                   -f("DIHEDRAL_PHASE")[dt]], axis=1)
    return {"bonds": (ba.astype(np.int32), bp), "angles": (aa.astype(np.int32), ap),
            "dihedrals": (da.astype(np.int32), dp)}


def pair_coefficients_from_AB(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """(T*T, 4) multipliers of the unit tables (A14, B8, A12, B6) for E = A r^-12 - B r^-6:
    fscal = 12 A r^-14 - 6 B r^-8."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    return np.stack([12.0 * A, -6.0 * B, A, -B], axis=-1).reshape(-1, 4)
