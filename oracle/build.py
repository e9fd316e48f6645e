"""Build the CPU oracle (oracle/_build/liboracle.so) from oracle.cpp and bonded.cpp.

The oracle is test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm load it.  -ffp-contract=off keeps every float expression rounded once
per operation on x86-64 and aarch64 alike."""
from __future__ import annotations

import fcntl
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp"]


def _fresh(srcs) -> bool:
    return LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in srcs)


def build(force: bool = False) -> Path:
    srcs = [HERE / "oracle.cpp", HERE / "bonded.cpp", HERE / "oracle.h"]
    if not force and _fresh(srcs):
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    # processes that load the oracle at the same time (spawned test ranks) build it once
    with open(OUT / ".build.lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not force and _fresh(srcs):
            return LIB
        return _build_locked()


def _build_locked() -> Path:
    tmp = OUT / "liboracle.so.tmp"
    cmd = ["g++", *FLAGS, str(HERE / "oracle.cpp"), str(HERE / "bonded.cpp"), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
