"""Build libmdrl.so in-tree: nvcc for sm_103a (one -gencode), translation units compiled in
parallel, cudart linked statically; cuFFT (the PME transforms) linked dynamically with an rpath to
the toolkit that built the library."""
from __future__ import annotations

import concurrent.futures as cf
import fcntl
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libmdrl.so"
INCLUDE = HERE.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC"]


def nvcc_path() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return str(Path(cand) / "bin" / "nvcc")
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found: set CUDA_HOME")
    return found


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _deps() -> list[Path]:
    return _sources() + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "mdrl.h"]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def _compile(src: Path, ptxas_verbose: bool, out: Path = OUT, defines: tuple = ()) -> tuple[Path, str]:
    obj = out / (src.name + ".o")
    dflags = [f"-D{d}" for d in defines]
    if src.suffix == ".cu":
        cmd = [nvcc_path(), *ARCH, *NVCC_FLAGS, *dflags, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd = ["g++", *CXX_FLAGS, *dflags, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj, res.stdout + res.stderr


def build(force: bool = False, ptxas_verbose: bool = False, out_dir: Path | None = None,
          defines: tuple = ()) -> Path:
    """Compile every CUDA/C++ translation unit and link libmdrl.so; returns its path.  `out_dir`
    and `defines` (-D flags) build a variant elsewhere (tuning sweeps)."""
    out = OUT if out_dir is None else Path(out_dir)
    if out_dir is None and not defines and not force and not ptxas_verbose and up_to_date():
        return LIB
    out.mkdir(parents=True, exist_ok=True)
    # concurrent builds into one folder (processes started together) run one at a time
    with open(out / ".build.lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if out_dir is None and not defines and not force and not ptxas_verbose and up_to_date():
            return LIB
        return _build_locked(out, ptxas_verbose, defines)


def _build_locked(out: Path, ptxas_verbose: bool, defines: tuple) -> Path:
    lib = out / "libmdrl.so"
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose, out, defines), srcs))
    objs = [str(o) for o, _ in results]
    tmp = out / "libmdrl.so.tmp"
    cuda_lib = Path(nvcc_path()).resolve().parent.parent / "lib64"
    cmd = [nvcc_path(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(tmp), *objs, "-lcufft",
           "-Xlinker", "-rpath", "-Xlinker", str(cuda_lib)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)
    if ptxas_verbose:
        for _, log in results:
            if log.strip():
                print(log)
    return lib


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
