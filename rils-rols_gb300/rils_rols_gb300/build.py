"""In-tree build of the native library librils_rols_gb300.so (sm_103a only).

Compiles the CUDA translation units with nvcc and the host C++ with g++ in
parallel, then links one shared library next to this file.  Runs on x86 (no
GPU needed: nvcc cross-compiles) and on the Arm GPU host alike.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent                      # rils-rols_gb300/
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
OUT = PKG / "librils_rols_gb300.so"
OBJ = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 fitness path needs the CUDA toolkit to build")


def sources() -> tuple[list[Path], list[Path]]:
    cu = sorted((CSRC / "device").glob("*.cu"))
    cpp = sorted((CSRC / "host").glob("*.cpp")) + sorted((CSRC / "common").glob("*.cpp"))
    return cu, cpp


def _digest(paths: list[Path]) -> str:
    h = hashlib.sha256()
    for p in sorted(paths):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(NVCC_FLAGS + CXX_FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    cu, cpp = sources()
    headers = list(CSRC.rglob("*.h")) + list(CSRC.rglob("*.cuh")) + list(INCLUDE.glob("*.h"))
    digest = _digest(cu + cpp + headers)
    stamp = OBJ / "digest"
    if not force and OUT.exists() and stamp.exists() and stamp.read_text() == digest:
        return OUT
    OBJ.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for src in cu:
        obj = OBJ / (src.stem + ".cu.o")
        jobs.append([nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = OBJ / (src.parent.name + "_" + src.stem + ".o")
        jobs.append(["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        return cmd[-1]

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(run, jobs))
    link = [nvcc, "-shared", *ARCH, "-o", str(OUT), *objs, "-Xcompiler", "-fPIC"]
    run(link)
    stamp.write_text(digest)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
