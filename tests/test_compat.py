"""The reference's simulation() entry point on top of the C-ABI (include/arbo_reference_compat.hpp).

A driver shaped like cpp/main.cpp's replicate loop (tests/compat/compat_driver.cpp) compiles and
links against the library with the reference's signature; on a GPU its outputs (the reference's
series, counters, community sizes and end-of-run census, written into the caller's device buffers
in the reference's types, and the nData file) equal the library's own run of the same replicates,
converted to the reference's layouts by the restatements below (writeIncidence,
cpp/writeoutput.cpp:13-98; the census types of cpp/censustypedef.h:8-16)."""
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


def ndata_text(runs_series, S):
    """The text writeIncidence (cpp/writeoutput.cpp:13-98) leaves in nData<k>.csv after the given
    replicates: the header on replicate 0, then per replicate the rows t, popSize, incidence,
    prevalence and community-0 prevalence per serotype, and the replicate index."""
    head = "t,popSize" + "".join(f",incidence_DENV{k + 1}" for k in range(S))
    head += "".join(f",prevalence_DENV{k + 1}" for k in range(S))
    head += "".join(f",prevalence_DENV{k + 1}_random_community" for k in range(S)) + ",simRun"
    out = [head]
    for run, (inc, inf, one, cnt) in enumerate(runs_series):
        for t in range(len(cnt)):
            row = [t, int(cnt[t])] + [int(v) for v in inc[t]] + [int(v) for v in inf[t]] + [int(v) for v in one[t]] + [run]
            out.append(",".join(str(v) for v in row))
    return "\n".join(out)


def reference_census(sim, S):
    """The library's census in the reference's types and layouts (cpp/censustypedef.h:8-16), in the
    order the driver writes them: ages, exposed and recovery ages as uint16, history [s * N + i]
    (-1 naive, -2 immune), communities from the sorted ranges and the identity index."""
    N, M = sim.census("n_age").size, sim.census("m_age").size
    imm = sim.census("n_immunity").astype(np.int64)
    hist = np.where(((imm[None, :] >> np.arange(S)[:, None]) & 1) == 1, -2, -1).astype(np.int32).ravel()
    ncomm = np.repeat(np.arange(len(sim.counters("n_subpop_loc")) - 1), np.diff(sim.counters("n_subpop_loc")))
    mcomm = np.repeat(np.arange(len(sim.counters("m_subpop_loc")) - 1), np.diff(sim.counters("m_subpop_loc")))
    u16 = lambda a: (np.asarray(a, np.int64) & 0xFFFF).astype(np.uint16)  # noqa: E731
    return [u16(sim.census("n_age")), u16(sim.census("n_exposed")), hist, sim.census("n_status").astype(np.uint8),
            sim.census("n_ple").astype(np.float32), u16(sim.census("n_recovery")), sim.census("n_strain").astype(np.uint8),
            ncomm.astype(np.uint32), np.arange(N, dtype=np.uint32), u16(sim.census("m_age")),
            sim.census("m_dead").astype(np.uint8), u16(sim.census("m_exposed")), sim.census("m_status").astype(np.uint8),
            sim.census("m_ple").astype(np.float32), sim.census("m_strain").astype(np.uint8), mcomm.astype(np.uint32),
            np.arange(M, dtype=np.uint32)]


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

    sp = SimulationParam(nSize=float(N), metaPop=float(P), bitingRate=0.9, mSize=M, nStrains=S, recordSpatial=1)
    net = create_network(side)

    def sizes_of(hetero, total):
        cum = calc_cumulative_com_size(net, hetero).astype(np.float64)
        return community_sizes(np.diff(np.concatenate([[0.0], cum])), total)

    ns, ms = sizes_of(sp.nHeteroPopSize, N), sizes_of(sp.mHeteroPopSize, M)
    seed = (base ^ (mcmc * GOLDEN_RATIO_64)) & (2**64 - 1)
    total_incidence = 0
    census_raw = (tmp_path / "out.bin.census").read_bytes()
    pos, runs_series = 0, []
    for run in range(runs):
        got = parts[run * len(sizes):(run + 1) * len(sizes)]
        with Simulation(Parameter(sp), net, ns, ms, max_time=T, seed=seed, instance=run) as sim:
            sim.init()
            sim.run()
            want = [sim.series("n_incidence"), sim.series("n_infected"), sim.series("one_subpop"),
                    sim.series("n_count"), sim.series("m_count"), sim.counters("n_subpop_count"),
                    sim.counters("m_subpop_count"), ns, ms, sim.series("infected_subpop")]
            runs_series.append(want[:4])
            for k, w_ in enumerate(reference_census(sim, S)):
                g = np.frombuffer(census_raw, w_.dtype, w_.size, pos)
                pos += w_.nbytes
                assert np.array_equal(g, w_), f"run {run}: census field {k} in the reference's layout"
        names = ["nIncidence", "nInfectedCount", "nOneSubPopInfectedCount", "nCount", "mCount", "nSubPopCount",
                 "mSubPopCount", "nSubPopSize", "mSubPopSize", "nInfectedSubPopCountSeries"]
        for name, g, w in zip(names, got, want):
            assert np.array_equal(g, np.asarray(w, np.uint32).ravel()), f"run {run}: {name}"
        total_incidence += int(got[0].sum())
    assert total_incidence > 0
    assert pos == len(census_raw)
    assert (odir / f"nData{mcmc}.csv").read_text() == ndata_text(runs_series, S)
