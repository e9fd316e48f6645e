"""The C-ABI library loads and exports every function include/mdrl.h declares; host-only entry
points work without a GPU; the Python mirror's structures match the header (CPU only)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import sc2019_md_gb300 as m

ROOT = Path(__file__).resolve().parent.parent


def _declared_functions():
    text = (ROOT / "include" / "mdrl.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(n for n in names if n not in ("if", "while", "sizeof")))


def test_every_declared_symbol_is_exported():
    names = _declared_functions()
    assert "mdrl_force_eval" in names and "MD_Evaluation_Model" in names
    lib = C.CDLL(str(m.library_path()))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_binds_every_symbol():
    names = _declared_functions()
    src = (ROOT / "sc2019_md_gb300" / "__init__.py").read_text()
    unbound = [n for n in names if n not in src]
    assert not unbound, unbound


def test_struct_layouts_match_header():
    """Field order and count of mdrl_params / mdrl_stats / mdrl_replica in the header equal the
    mirror's."""
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "mdrl.h").read_text(), flags=re.S)
    for cname, cls in (("mdrl_params", m.Params), ("mdrl_stats", m.Stats), ("mdrl_replica", m.Replica),
                       ("mdrl_tile", m.Tile), ("mdrl_pme_params", m.PmeParams)):
        body = re.search(r"typedef struct \{((?:(?!typedef struct).)*?)\}\s*" + cname + ";", text, re.S).group(1)
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            for part in decl.split(",")[0:]:
                nm = re.findall(r"([A-Za-z_][A-Za-z0-9_]*)\s*(?:\[[^\]]*\])?\s*$", part.strip())
                fields.append(nm[0])
        assert fields == [f for f, _ in cls._fields_], (cname, fields)


def test_default_params():
    p = m.default_params()
    assert p.ntypes == 1 and p.sigma[0] == 3.4 and p.table_bins == 256 and p.dt_fs == 2.0
    assert p.accum == m.ACC_FIXED64 and p.integrator == m.INT_VELOCITY_VERLET
    assert m.lib().mdrl_version().decode().startswith("mdrl")


def test_fit_tables_host_only_and_validation():
    t = m.fit_tables(1, 4, 64, 0)
    x = 1.0 + 0.5 / 64        # segment 0, bin 0 middle
    v = t[0, 1, 0] * x + t[0, 0, 0]
    assert abs(v / x ** -7 - 1) < 1e-3
    with pytest.raises(m.MdrlError) as e:
        m.fit_tables(4, 4, 64, 0)
    assert e.value.status == 1 and "invalid" in str(e.value)


def test_null_context_calls_fail_cleanly():
    L = m.lib()
    assert L.mdrl_force_eval(None, 0, None, None, None, None, None, None, None, None, None, None) == 1
    assert L.mdrl_step(None, 1, None) == 1
    assert L.mdrl_destroy(None) == 0
    p = m.default_params(box=(-1.0, 1.0, 1.0))
    h = C.c_void_p()
    assert L.mdrl_create(C.byref(p), C.byref(h)) == 1
    assert b"box" in L.mdrl_last_error()


def test_batch_validation_before_any_device_call():
    """mdrl_batch_create rejects bad replicas and modes on the host, before touching a GPU."""
    L = m.lib()
    h = C.c_void_p()
    p = m.default_params(cutoff=10.0)
    reps = (m.Replica * 2)()
    reps[0].n, reps[1].n = 100, 100
    for d in range(3):
        reps[0].box[d] = 20.0
        reps[1].box[d] = 9.5          # not above the cutoff
    assert L.mdrl_batch_create(C.byref(p), 2, reps, C.byref(h)) == 3
    assert b"replica 1" in L.mdrl_last_error() and b"exceed the cutoff" in L.mdrl_last_error()
    for d in range(3):
        reps[1].box[d] = 20.0
    reps[1].n = 0
    assert L.mdrl_batch_create(C.byref(p), 2, reps, C.byref(h)) == 1
    reps[1].n = 100
    p.accum = m.ACC_FP32_ATOMIC
    assert L.mdrl_batch_create(C.byref(p), 2, reps, C.byref(h)) == 1
    assert b"fixed point" in L.mdrl_last_error()
    assert L.mdrl_batch_create(C.byref(p), 0, reps, C.byref(h)) == 1
    assert L.mdrl_batch_destroy(None) == 0
    assert L.mdrl_batch_step(None, 1, None) == 1
