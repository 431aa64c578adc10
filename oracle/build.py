"""Build recipe of the serial CPU oracle (test infrastructure; see oracle.h).

Compiles ``oracle.c`` with gcc into ``oracle/_build/liboracle.so``. ``-ffp-contract=off`` keeps
every float expression un-fused (GCC contracts to FMA by default on aarch64), matching the
``-fmad=false`` device build.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
import threading
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
FLAGS = ["-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-Wall"]
_lock = threading.Lock()


def build_oracle(force: bool = False) -> Path:
    # Threads of one process build once; processes write their own temporary file and rename it.
    with _lock:
        return _build(force)


def _build(force: bool) -> Path:
    OUT.mkdir(exist_ok=True)
    h = hashlib.sha256()
    for f in ("oracle.c", "oracle.h"):
        h.update((HERE / f).read_bytes())
    h.update((HERE.parent / "include" / "arbo.h").read_bytes())
    h.update(" ".join(FLAGS).encode())
    stamp = OUT / "build.stamp"
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == h.hexdigest():
        return LIB
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found to build the oracle")
    tmp = LIB.with_suffix(f".so.{os.getpid()}.tmp")
    cmd = [cc, *FLAGS, "-o", str(tmp), str(HERE / "oracle.c"), "-lm"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}")
    os.replace(tmp, LIB)
    stamp.write_text(h.hexdigest())
    return LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
