"""C-ABI boundary checks that need no GPU: symbols, struct layouts, host helpers."""
import re
from pathlib import Path

import numpy as np
import pytest

from arbo_gpu_fit_gb300 import _native
from arbo_gpu_fit_gb300.simulation import (SimulationParam, calc_cumulative_com_size, community_sizes,
                                           create_network)

HEADER = Path(__file__).resolve().parents[1] / "include" / "arbo.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(arbo_[a-z0-9_]+)\s*\(", text)))


def struct_fields(name):
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    body = re.search(r"typedef struct " + name + r" \{(.*?)\}", text, flags=re.S).group(1)
    return re.findall(r"\b(\w+)\s*;", body)


def test_library_exports_every_declared_symbol(native):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, missing
    assert set(names) == set(_native.SIGNATURES), set(names) ^ set(_native.SIGNATURES)


@pytest.mark.parametrize("cname, pystruct", [
    ("arbo_sim_param", _native.SimParamStruct),
    ("arbo_arch_param", _native.ArchParamStruct),
    ("arbo_io_param", _native.IOParamStruct),
    ("arbo_csr", _native.CSRStruct),
    ("arbo_mcmc_config", _native.McmcConfigStruct),
    ("arbo_census_export", _native.CensusExportStruct),
])
def test_struct_layout_matches_header(cname, pystruct):
    assert [f for f, _ in pystruct._fields_] == struct_fields(cname)


def test_version(native):
    assert b"sm_103a" in native.arbo_version()


def test_batch_setter_rejects_bad_arguments(native):
    # Checked before any device call: no batch, or neither parameters nor seeds.
    assert native.arbo_batch_set_params(None, None, None, None, None) == _native.ARBO_ERR_INVALID
    assert b"arbo_batch_set_params" in native.arbo_last_error()


def test_defaults_are_reference_constructor_values():
    p = SimulationParam()
    # cpp/SimulationParam.cpp:11-47
    assert p.nSize == 100000.0 and p.metaPop == 10000.0
    assert p.bitingRate == 0.25 and p.mnBitingSuccess == 0.5 and p.nmBitingSuccess == 0.5
    assert p.recovery == 4.0 and p.mExposed == 6.0 and p.nExposed == 7.0
    assert p.externalInfection == 5.0 and p.noDistance == 0.75
    assert abs(p.longDistance - 0.01) < 1e-9
    assert p.mScaleLifeExpectancy == 23.0 and p.mShapeLifeExpectancy == 4.0
    assert p.nMaxInitialAgeYears == 150 and p.mMaxInitialAge == 300 and p.maxIntroAttempt == 1000
    assert p.nStrains == 4 and p.quirks == _native.QUIRKS_REFERENCE


@pytest.mark.parametrize("side", [1, 2, 3, 10, 50])
def test_lattice_csr(side):
    net = create_network(side)
    P = side * side
    assert net.loc.size == P + 1 and net.nnz == 4 * side * (side - 1)
    deg = net.degrees()
    for v in range(P):
        x, y = v % side, v // side
        expect = (x > 0) + (x < side - 1) + (y > 0) + (y < side - 1)
        assert deg[v] == expect
        row = net.to[net.loc[v]:net.loc[v + 1]]
        assert list(row) == sorted(row)
        for u in row:
            ux, uy = int(u) % side, int(u) // side
            assert abs(ux - x) + abs(uy - y) == 1
            assert v in net.to[net.loc[u]:net.loc[u + 1]]
    assert np.all(net.weight == 1.0)
    if side > 2:
        assert set(np.unique(deg)) == {2, 3, 4}


def test_cumulative_com_size():
    net = create_network(5)
    out = calc_cumulative_com_size(net, 1.0)
    deg = net.degrees().astype(np.float64)
    np.testing.assert_allclose(out, np.cumsum(deg) / deg.sum(), rtol=1e-6)
    assert out[-1] == 1.0
    flat = calc_cumulative_com_size(net, 0.0)
    np.testing.assert_allclose(flat, np.arange(1, 26) / 25.0, rtol=1e-6)


def test_community_sizes():
    rng = np.random.default_rng(1)
    w = np.exp(0.8 * rng.standard_normal(2500))
    for total in (0, 1, 2499, 1_000_000, 6_000_000):
        s = community_sizes(w, total)
        assert int(s.sum()) == total
        q = total * w / w.sum()
        assert np.all(np.abs(s - q) < 1.0 + 1e-9)
    np.testing.assert_array_equal(community_sizes(np.ones(4), 10), [3, 3, 2, 2])
