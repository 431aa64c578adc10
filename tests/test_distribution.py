"""Distribution-level parity with the reference's own CUDA kernels.

The reference's kernels (compiled from its sources into cubins and driven as cpp/simulation.cpp
drives them, oracle/ref_kernels.py) ran the small plain workload for 200 seeds on a GB300; their
weekly incidence per serotype is the fixture tests/golden/ref_weekly_incidence_plain_small.npz
(tests/golden/make_ref_incidence.py). The reference's curand streams are indexed by hardware
thread slot, so only distributions can be compared: two-sample Kolmogorov-Smirnov tests on the
yearly incidence per serotype and on every (week, serotype) cell, with the acceptance rule of
tests.distribution.verdict (p > 0.01; Bonferroni over the 208 cells).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import ref_build
from tests import distribution as D

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def reference():
    return np.load(GOLDEN / D.FIXTURE)


def test_reference_fixture_is_sane(reference):
    inc, mos = reference["weekly_incidence"], reference["weekly_mosquitoes"]
    assert inc.shape == (D.SEEDS, D.WEEKS, 4) and mos.shape == (D.SEEDS, D.WEEKS + 1)
    assert np.all(inc[:, 0] == 0)  # nothing becomes infectious in the first week
    assert 4000 < inc.sum(1).mean() < 8000
    # Live mosquitoes: capped at the 40,000 slots around the seasonal peak, ~20,000 at the trough.
    assert mos.max() <= 40_000 and np.all(mos[:, 0] == 40_000)
    trough = mos.min(axis=1)
    assert np.all((19_000 < trough) & (trough < 21_000))


def test_oracle_matches_reference_kernels_in_distribution(reference):
    r = D.ks_report(D.run_oracle(D.SEEDS), reference["weekly_incidence"])
    assert D.verdict(r) == [], D.verdict(r)


def test_planted_rate_error_is_detected(reference):
    # A 4 % lower mosquito-to-human transmission probability, planted in the oracle, must fail
    # the same rule: the comparison has the power to see a change of this size.
    sp = D.workload().parameter.simulation
    r = D.ks_report(D.run_oracle(D.SEEDS, mnBitingSuccess=float(sp.mnBitingSuccess) * 0.96),
                    reference["weekly_incidence"])
    assert D.verdict(r) != []


def test_reference_build_layout():
    if not (ref_build.reference_dir() / "cpp").is_dir() and not ref_build.prebuilt():
        pytest.skip("neither reference sources nor prebuilt reference cubins are present")
    out = ref_build.build_reference_kernels()
    layout = json.loads((out / "layout.json").read_text())
    # Parameter {ArchitectureParam; IOParam (4 std::string); SimulationParam (33 floats)}.
    assert layout["sizeof_SimulationParam"] == 33 * 4
    assert layout["sizeof_ArchitectureParam"] == 12
    assert layout["off_simulation"] == layout["off_io"] + layout["sizeof_IOParam"]
    assert layout["sizeof_curandState"] == 48
    from oracle.ref_kernels import KERNELS

    for key, (mod, sym) in KERNELS.items():
        assert sym.encode() in (out / f"{mod}.cubin").read_bytes(), key


@pytest.mark.gpu
def test_library_matches_reference_kernels_in_distribution(gpu, reference):
    ours = D.run_library(D.SEEDS)
    r = D.ks_report(ours, reference["weekly_incidence"])
    assert D.verdict(r) == [], D.verdict(r)


@pytest.mark.gpu
def test_library_matches_live_reference_kernels(gpu):
    # Both sides live on this GPU: the reference's kernels through the driver API, this library
    # through its C-ABI.
    if not ref_build.prebuilt():
        pytest.skip("reference cubins not built (oracle/ref_build.py needs the reference sources)")
    import sys

    sys.path.insert(0, str(GOLDEN))
    from make_ref_incidence import run_reference

    ref, mos, meta = run_reference(D.SEEDS)
    assert meta["nsmid"] >= meta["sm_count"]
    assert np.all(mos[:, 0] == 40_000)
    r = D.ks_report(D.run_library(D.SEEDS), ref)
    assert D.verdict(r) == [], D.verdict(r)
