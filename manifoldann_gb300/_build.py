"""Build of the in-tree native artefacts.

* ``manifoldann_gb300/libmanngpu.so`` -- the GB300 (sm_103a) library behind
  ``include/mann.h``.  Every ``csrc/*.cu`` is compiled to an object in
  parallel and linked with the static CUDA runtime.
* ``oracle/liboracle.so`` -- the CPU oracle (test infrastructure) via its
  Makefile.

Nothing here needs a GPU: nvcc cross-compiles for sm_103a.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = ROOT / "_build" / "obj"
LIB = PKG / "libmanngpu.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "--expt-relaxed-constexpr",
    "-Xptxas",
    "-warn-spills",
]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = Path("/usr/local/cuda/bin/nvcc")
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False, ptxas_info: bool = False) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    objs = []
    jobs = []
    for src in sources:
        obj = OBJ / (src.stem + ".o")
        objs.append(obj)
        if ptxas_info or _stale(obj, [src] + headers):
            cmd = [nvcc()] + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + [
                "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
    if jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-cudart", "static"])
        os.replace(tmp, LIB)
    if verbose:
        for line in logs:
            if line.strip():
                print(line)
    return LIB


def build_oracle() -> Path:
    _run(["make", "-s", "-C", str(ORACLE_DIR)])
    return ORACLE_LIB


if __name__ == "__main__":
    import sys

    build_library(verbose=True, ptxas_info="-v" in sys.argv)
    build_oracle()
    print(LIB, ORACLE_LIB)
