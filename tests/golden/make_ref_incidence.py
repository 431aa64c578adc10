"""Generates tests/golden/ref_weekly_incidence_plain_small.npz from the reference's own kernels.

Needs a GPU and the cubins that oracle/ref_build.py compiles from the reference sources. Runs the
small plain workload for seeds 0..199 through oracle.ref_kernels (the reference's kernels, driven
as cpp/simulation.cpp drives them) and stores, per seed, the weekly incidence per serotype and the
live mosquito count at the end of every week.

    python tests/golden/make_ref_incidence.py [--seeds 200] [--out tests/golden/ref_weekly_incidence_plain_small.npz]
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.ref_kernels import ReferenceKernels  # noqa: E402
from tests import distribution as D  # noqa: E402


def run_reference(seeds: int, verbose: bool = False):
    w = D.workload()
    sp = w.parameter.simulation
    T = w.max_time
    E = D.expected_series(sp, T)
    ref = ReferenceKernels(0)
    inc = np.zeros((seeds, D.WEEKS, int(sp.nStrains)), np.uint32)
    mweek = np.zeros((seeds, D.WEEKS + 1), np.uint32)
    t0 = time.time()
    for seed in range(seeds):
        out = ref.run(sp, w.network.loc, w.network.to, w.network.weight, E, int(sp.nSize), int(sp.mSize), T, seed,
                      strains=int(sp.nStrains))
        inc[seed] = D.weekly(out["incidence"])
        mweek[seed] = out["m_count"][0:7 * D.WEEKS + 1:7]
        if verbose and seed < 4:
            print(f"seed {seed}: incidence per serotype {out['incidence'].sum(0).tolist()}, "
                  f"mosquitoes t=0/91/182/273/364 {out['m_count'][[0, 91, 182, 273, 364]].tolist()}", flush=True)
    meta = dict(nsmid=ref.nsmid, nwarpid=ref.nwarpid, sm_count=ref.sm_count, seconds=time.time() - t0)
    return inc, mweek, meta


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seeds", type=int, default=D.SEEDS)
    ap.add_argument("--out", default=str(ROOT / "tests" / "golden" / D.FIXTURE))
    a = ap.parse_args()
    inc, mweek, meta = run_reference(a.seeds, verbose=True)
    np.savez_compressed(a.out, weekly_incidence=inc, weekly_mosquitoes=mweek, seeds=np.arange(a.seeds),
                        nsmid=meta["nsmid"], nwarpid=meta["nwarpid"])
    print(f"wrote {a.out}: {a.seeds} seeds in {meta['seconds']:.1f} s; yearly incidence mean per serotype "
          f"{inc.sum(1).mean(0).round(1).tolist()}; probe nsmid={meta['nsmid']} nwarpid={meta['nwarpid']} "
          f"SMs={meta['sm_count']}")


if __name__ == "__main__":
    main()
