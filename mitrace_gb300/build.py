"""Builds the in-tree shared libraries.

* ``mitrace_gb300/libmitrace_gb300.so`` - the product: hand-written sm_103a
  kernels plus the C ABI of ``include/mitrace_gpu.h`` (nvcc, one -gencode).
* ``oracle/liboracle.so`` and ``oracle/liboracle_fast.so`` - the CPU oracle
  (test infrastructure: the checker and the timed CPU baseline).

Translation units compile in parallel; nothing is installed outside the tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "mitrace_gb300"
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "libmitrace_gb300.so"
ORACLE_DIR = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC,-ffp-contract=off,-Wall",
]
SOURCES = ["mt_api.cu", "mt_kernels.cu", "mt_bvh.cpp", "mt_noalloc.cu", "mt_adjoint.cu", "mt_nrc.cu", "mt_image.cu"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build mitrace_gb300")
    return cand


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(Path(d).stat().st_mtime <= t for d in deps)


def _run_parallel(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out.decode(errors="replace")))
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("build failed:\n" + msg)


def build_product(force: bool = False, verbose: bool = False) -> Path:
    """Compiles and links the library.  MT_NVCC_EXTRA (whitespace-separated
    flags, e.g. -DMT_TRAVERSE_MIN_BLOCKS=5) is appended for tuning builds."""
    nvcc = nvcc_path()
    extra = os.environ.get("MT_NVCC_EXTRA", "").split()
    if extra:
        force = True
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "mitrace_gpu.h"]
    objs, cmds = [], []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or not _newer(o, [s, *headers]):
            cmds.append([nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", str(s), "-o", str(o)])
    if cmds:
        if verbose:
            for c in cmds:
                print(" ".join(c))
        _run_parallel(cmds)
    if force or cmds or not _newer(LIB, objs):
        link = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        if verbose:
            print(" ".join(link))
        _run_parallel([link])
    return LIB


def build_oracle(force: bool = False) -> Path:
    cmd = ["make", "-s", "-C", str(ORACLE_DIR)]
    if force:
        subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "clean"], check=True)
    subprocess.run(cmd, check=True)
    return ORACLE_DIR / "liboracle.so"


def build_all(force: bool = False, verbose: bool = False):
    build_product(force=force, verbose=verbose)
    build_oracle(force=force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
