"""Build recipe of the native library (CUDA for sm_103a + C++ host side of the C-ABI).

The library is built in-tree into ``arbo_gpu_fit_gb300/_lib/libarbo_gb300.so``: each ``.cu``
translation unit is compiled in parallel with nvcc for ``sm_103a`` only, then linked as a
shared object. Floating-point contraction is off on both sides (``-fmad=false`` for device code,
``-ffp-contract=off`` for host code) so every float expression that feeds a decision is evaluated
exactly as written.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libarbo_gb300.so"
SOURCES = ["kernels.cu", "api.cu", "mcmc.cu", "mlp.cu", "selftest.cu"]
HEADERS = ["philox.cuh", "sim_internal.h", "tc.cuh"]
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-O2",
    "--expt-relaxed-constexpr", "-Xptxas", "-v",
]


def _nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build arbo_gpu_fit_gb300")
    return exe


def _fingerprint() -> str:
    h = hashlib.sha256()
    for name in SOURCES + HEADERS:
        h.update((CSRC / name).read_bytes())
    h.update((INCLUDE / "arbo.h").read_bytes())
    h.update(" ".join(NVCC_FLAGS).encode())
    return h.hexdigest()


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compile the library if sources or flags changed; returns the path of the .so."""
    LIB_DIR.mkdir(exist_ok=True)
    stamp = LIB_DIR / "build.stamp"
    fp = _fingerprint()
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return LIB
    nvcc = _nvcc()
    objs, procs = [], []
    for name in SOURCES:
        obj = LIB_DIR / (Path(name).stem + ".o")
        cmd = [nvcc, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(CSRC / name), "-o", str(obj)]
        procs.append((name, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(obj)
    logs = []
    for name, cmd, p in procs:
        out, _ = p.communicate()
        logs.append(f"== {name}\n{out}")
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {name}:\n{' '.join(cmd)}\n{out}")
    (LIB_DIR / "ptxas.log").write_text("\n".join(logs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}")
    os.replace(tmp, LIB)
    stamp.write_text(fp)
    if verbose:
        print("\n".join(logs), file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
