"""Build recipe of the distribution-level checker: the reference's own CUDA kernels.

Test infrastructure only. Compiles the reference's kernel sources, unmodified and where they lie
in the reference checkout, into sm_103a cubins under ``oracle/_ref/`` (git-ignored; the cubins are
device code, so they run on any host CPU). Only the kernels are used: ``oracle/ref_kernels.py``
loads the cubins through the CUDA driver API and replays the reference's host launch sequence
(cpp/simulation.cpp:81-156) itself. Two shims in ``oracle/ref_shim/`` are put ahead of the
reference's include path: ``constant.h`` (four serotypes instead of the shipped one) and
``Parameter.h`` (case of cpp/parameter.h). ``ref_layout.cpp`` is compiled against the reference
headers with the host compiler to record the byte layout of the by-value kernel arguments
(``layout.json``). The reference's kernels are compiled with the device flags the reference
documents for its own build (README.md, "Compilation": ``-O2 -use_fast_math``), so ``powf`` and
``expf`` in its death tests take the fast approximate forms and FMA contraction stays on.

The reference checkout is read from ``$ARBO_REFERENCE_DIR``, else from ``REFERENCE_CHECKOUT``, the
one place this recipe names where the read-only checkout sits on the build machine. Where neither
exists (the GPU machine) the prebuilt files in ``oracle/_ref/`` are used as they are.
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SHIM = HERE / "ref_shim"
REF_SOURCES = ["setuprng", "demographicintial", "epidemicinitial", "ndemographic", "mdemographic",
               "nepidemic", "mepidemic", "epidemic", "datacollect"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FILES = [f"{n}.cubin" for n in REF_SOURCES] + ["harness.cubin", "layout.json"]
# Device flags of the reference's documented build (its README, "Compilation").
REF_FLAGS = ["-O2", "-use_fast_math"]


# Where the recipe finds the reference checkout on the build machine when $ARBO_REFERENCE_DIR is unset.
REFERENCE_CHECKOUT = "/root/reference"


def reference_dir() -> Path:
    return Path(os.environ.get("ARBO_REFERENCE_DIR") or REFERENCE_CHECKOUT)


def prebuilt() -> bool:
    return all((OUT / f).exists() for f in FILES)


def _nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found")
    return exe


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference kernel build failed:\n{' '.join(map(str, cmd))}\n{r.stdout}")
    return r.stdout


def build_reference_kernels(force: bool = False) -> Path | None:
    """Compile the cubins; returns ``oracle/_ref`` or None when neither sources nor a build exist."""
    src = reference_dir() / "cpp"
    if not src.is_dir():
        return OUT if prebuilt() else None
    OUT.mkdir(exist_ok=True)
    h = hashlib.sha256()
    for n in REF_SOURCES:
        h.update((src / f"{n}.cu").read_bytes())
    for f in sorted(src.glob("*.h")) + sorted(src.glob("*.cuh")):
        h.update(f.read_bytes())
    for f in [SHIM / "constant.h", SHIM / "Parameter.h", HERE / "ref_harness.cu", HERE / "ref_layout.cpp",
              Path(__file__)]:
        h.update(f.read_bytes())
    stamp = OUT / "build.stamp"
    if not force and prebuilt() and stamp.exists() and stamp.read_text() == h.hexdigest():
        return OUT
    nvcc = _nvcc()
    inc = ["-I", str(SHIM), "-I", str(src), "-include", str(SHIM / "constant.h"), "-include", "cstring",
           "-include", "cmath"]
    jobs = [[nvcc, "-cubin", *ARCH, *REF_FLAGS, *inc, str(src / f"{n}.cu"), "-o", str(OUT / f"{n}.cubin")]
            for n in REF_SOURCES]
    jobs.append([nvcc, "-cubin", *ARCH, "-O3", "-lineinfo", str(HERE / "ref_harness.cu"), "-o",
                 str(OUT / "harness.cubin")])
    cuda_inc = Path(nvcc).resolve().parent.parent / "include"
    layout_exe = OUT / "ref_layout"
    jobs.append([shutil.which("g++") or "c++", "-std=c++17", "-w", "-I", str(SHIM), "-I", str(src), "-I",
                 str(cuda_inc), "-include", "string", "-include", "cstring", "-include", "cmath",
                 str(HERE / "ref_layout.cpp"), "-o", str(layout_exe)])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        logs = list(ex.map(_run, jobs))
    layout = json.loads(_run([str(layout_exe)]))
    (OUT / "layout.json").write_text(json.dumps(layout, indent=1) + "\n")
    (OUT / "build.log").write_text("\n".join(logs))
    stamp.write_text(h.hexdigest())
    return OUT


if __name__ == "__main__":
    print(build_reference_kernels(force="--force" in sys.argv))
