"""The reference's simulation() entry point on top of the C-ABI (include/arbo_reference_compat.hpp).

A driver shaped like cpp/main.cpp's replicate loop (tests/compat/compat_driver.cpp) compiles and
links against the library with the reference's signature; on a GPU its outputs (the reference's
series, counters and community sizes, written into the caller's device buffers, and the nData
file) equal the library's own run of the same replicates."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
DRIVER = ROOT / "tests" / "compat" / "compat_driver.cpp"
GOLDEN_RATIO_64 = 0x9E3779B97F4A7C15


def build_driver(out_dir: Path) -> Path:
    from arbo_gpu_fit_gb300 import build as B

    lib = B.build_library()
    cuda = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parents[1]
    exe = out_dir / "compat_driver"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
           f"-I{cuda / 'include'}", str(DRIVER), "-o", str(exe), f"-L{lib.parent}", "-larbo_gb300",
           f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_compat_driver_builds(tmp_path):
    assert build_driver(tmp_path).exists()


@pytest.mark.gpu
def test_compat_simulation_equals_library(gpu, tmp_path):
    from arbo_gpu_fit_gb300.simulation import (Parameter, Simulation, SimulationParam, calc_cumulative_com_size,
                                               community_sizes, create_network)

    exe = build_driver(tmp_path)
    side, N, M, T, mcmc, runs = 4, 1200, 4800, 60, 3, 2
    P, S, R = side * side, 4, T + 1
    odir = tmp_path / "odir"
    odir.mkdir()
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(side), str(N), str(M), str(T), str(mcmc), str(runs), str(odir), str(out)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    base = int(r.stdout.split()[1])
    sizes = [R * S, R * S, R * S, R, R, P, P, P, P, R * S * P]
    raw = np.fromfile(out, np.uint32)
    assert raw.size == runs * sum(sizes)
    parts = np.split(raw, np.cumsum(sizes * runs)[:-1])
    assert (odir / f"nData{mcmc}.csv").exists()

    sp = SimulationParam(nSize=float(N), metaPop=float(P), bitingRate=0.9, mSize=M, nStrains=S, recordSpatial=1)
    net = create_network(side)

    def sizes_of(hetero, total):
        cum = calc_cumulative_com_size(net, hetero).astype(np.float64)
        return community_sizes(np.diff(np.concatenate([[0.0], cum])), total)

    ns, ms = sizes_of(sp.nHeteroPopSize, N), sizes_of(sp.mHeteroPopSize, M)
    seed = (base ^ (mcmc * GOLDEN_RATIO_64)) & (2**64 - 1)
    total_incidence = 0
    for run in range(runs):
        got = parts[run * len(sizes):(run + 1) * len(sizes)]
        with Simulation(Parameter(sp), net, ns, ms, max_time=T, seed=seed, instance=run) as sim:
            sim.init()
            sim.run()
            want = [sim.series("n_incidence"), sim.series("n_infected"), sim.series("one_subpop"),
                    sim.series("n_count"), sim.series("m_count"), sim.counters("n_subpop_count"),
                    sim.counters("m_subpop_count"), ns, ms, sim.series("infected_subpop")]
        names = ["nIncidence", "nInfectedCount", "nOneSubPopInfectedCount", "nCount", "mCount", "nSubPopCount",
                 "mSubPopCount", "nSubPopSize", "mSubPopSize", "nInfectedSubPopCountSeries"]
        for name, g, w in zip(names, got, want):
            assert np.array_equal(g, np.asarray(w, np.uint32).ravel()), f"run {run}: {name}"
        total_incidence += int(got[0].sum())
    assert total_incidence > 0
