"""FP64 serial check of a saved GPU fit (test infrastructure; run by hand after a fit).

Replays a subset of the exact (batched, equal to plain) chains of a fit saved by
``python -m arbo_gpu_fit_gb300.fit --save fit.npz`` with the serial double-precision program
(oracle/mcmc_serial.py: the oracle simulator, keyed draws, the same step schedule) and reports the
largest relative difference of the recorded states and the posterior means of the subset from both
runs with their relative error.

    python tests/mcmc_serial_check.py fit.npz --chains 4 --iters 20 [--threads 16]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from arbo_gpu_fit_gb300 import fit  # noqa: E402
from oracle import mcmc_serial  # noqa: E402


def check(path: str, chains: int, iters: int, threads: int, burn: int = 0) -> dict:
    z = np.load(path)
    population = str(z["population"])
    w = fit.workload(population)
    C = int(z["chains"])
    subset = list(range(min(chains, C)))
    gpu = z["batched_chain"][:iters, subset]
    t0 = time.perf_counter()
    ser, flags, _ = mcmc_serial.run(w, z["observed"], C, z["schedule"][:iters], int(z["mcmc_seed"]), iters,
                                    z["theta0"], replicates=int(z["replicates"]), subset=subset, threads=threads,
                                    chol=z["chol"][:iters] if "chol" in z.files else None)
    secs = time.perf_counter() - t0
    rel = np.abs(ser - gpu) / np.maximum(np.abs(ser), 1e-12)
    k = min(burn, iters - 1)
    mg, ms = gpu[k:].reshape(-1, gpu.shape[2]).mean(0), ser[k:].reshape(-1, ser.shape[2]).mean(0)
    return {"population": population, "chains": subset, "iters": iters, "replicates": int(z["replicates"]),
            "serial_seconds": secs, "threads": threads, "max_rel_state_diff": float(rel.max()),
            "accept_flags_equal": bool(np.array_equal(flags, z["batched_flags"][:iters, subset])),
            "mean_gpu": mg.tolist(), "mean_serial": ms.tolist(),
            "mean_rel_err": (np.abs(mg - ms) / np.abs(ms)).tolist()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("path")
    ap.add_argument("--chains", type=int, default=4)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--burn", type=int, default=0)
    a = ap.parse_args()
    print(json.dumps(check(a.path, a.chains, a.iters, a.threads, a.burn), indent=1))


if __name__ == "__main__":
    main()
