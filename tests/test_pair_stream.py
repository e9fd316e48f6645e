"""The half-shell traversal and its energy pinned to the reference's own outputs (CPU only).

MatlabScripts/VERIFICATION_PARTICLE_PAIR_INPUT.txt is the input stream of
SC/Particle_Pair_Gen_HalfShell.v for home cell (2,2,2) of the 20k LJArgon set (7 x 6 x 6 cells of
8.5 A): 78 reference particles x 180 cycles x 8 filters.  Rebuilt from the oracle's binning of the
same positions (KAT-2 fixture) and the library's half-shell offset table, every neighbour ID, valid
bit and position equals the reference's (SHA-256 of the canonical stream)."""
import hashlib
import json

import numpy as np

import oracle
import sc2019_md_gb300 as m
from helpers import GOLDEN, kat2_positions, pair_stream_canon_from_cells


def test_halfshell_offsets_are_the_reference_filter_order():
    digits = ["".join(str(2 + int(v)) for v in o) for o in m.halfshell_offsets()]
    assert digits == ["222", "223", "231", "232", "233", "311", "312", "313", "321", "322", "323", "331",
                      "332", "333"]


def test_pair_stream_reproduces_reference_rtl_input():
    pos, _ = kat2_positions()
    cell_of, start, order, _ = oracle.bin_cells(pos, (7 * 8.5, 6 * 8.5, 6 * 8.5), (7, 6, 6))

    def cell_list(cx, cy, cz):
        c = ((cx - 1) * 6 + (cy - 1)) * 6 + (cz - 1)
        return order[start[c]:start[c + 1]]

    canon = pair_stream_canon_from_cells(pos, cell_list, (2, 2, 2), m.halfshell_offsets())
    expect = json.loads((GOLDEN / "pair_stream_222.json").read_text())
    assert len(canon) == expect["lines"] == 14040
    assert hashlib.sha256("\n".join(canon).encode()).hexdigest() == expect["sha256"]


def test_oracle_energy_matches_reference_golden_model_20k():
    """System-level pin: the FP64 oracle's LJ energy of the 20k LJArgon positions (sigma 2.1 A,
    eps 1.995996^2 kJ/mol, rc 8.5 A, periodic 59.5 x 51 x 51 A) equals the step-1 potential energy
    the reference's double-precision golden model printed (7 significant digits)."""
    pos, _ = kat2_positions()
    e = json.loads((GOLDEN / "energy_20k.json").read_text())
    pc64 = oracle.lb_coefficients([2.1], [1.995996 ** 2])
    s = oracle.System(pos, (7 * 8.5, 6 * 8.5, 6 * 8.5), (7, 6, 6), 8.5, pc64.astype(np.float32), eval=1,
                      pcoef64=pc64)
    _, st = s.force_direct64()
    ref = e["Double"]["potential"]
    assert abs(st["e_lj"] - ref) <= 1e-6 * abs(ref)
    # the single-precision and interpolated reference runs sit within their own FP32 / table error
    assert abs(e["Single"]["potential"] - ref) <= 5e-6 * abs(ref)
    assert abs(e["Interpolation"]["potential"] - ref) <= 2e-4 * abs(ref)
