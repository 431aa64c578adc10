"""The serial oracle on its own (no GPU): random stream, seeding bijection, model invariants,
and the committed golden fixtures that pin its outputs."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from arbo_gpu_fit_gb300 import configs
from oracle import binding as ob
from tests.helpers import CENSUS_FIELDS, SERIES_KINDS, recount, small_case

GOLDEN = Path(__file__).resolve().parent / "golden"


def philox_py(ctr, key):
    """Philox4x32-10 written out independently (Salmon et al., SC'11)."""
    c = [x & 0xFFFFFFFF for x in ctr]
    k0, k1 = key[0] & 0xFFFFFFFF, key[1] & 0xFFFFFFFF
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF, ((p0 >> 32) ^ c[3] ^ k1) & 0xFFFFFFFF,
             p0 & 0xFFFFFFFF]
        k0 = (k0 + 0x9E3779B9) & 0xFFFFFFFF
        k1 = (k1 + 0xBB67AE85) & 0xFFFFFFFF
    return c


def test_philox_matches_independent_restatement():
    rng = np.random.default_rng(7)
    for _ in range(200):
        ctr = [int(x) for x in rng.integers(0, 2**32, 4, dtype=np.uint64)]
        key = [int(x) for x in rng.integers(0, 2**32, 2, dtype=np.uint64)]
        assert ob.philox(ctr, key) == philox_py(ctr, key)
    assert ob.philox([0, 0, 0, 0], [0, 0]) == philox_py([0, 0, 0, 0], [0, 0])


def test_draw_counter_layout():
    seed = 0x0123456789ABCDEF
    got = ob.draw4(seed, 7, 18, 1234, 56, 0x123456, 0x89)
    want = philox_py([1234, 56, (18 << 24) | 0x123456, (0x89 << 16) | 7], [seed & 0xFFFFFFFF, seed >> 32])
    assert got == want


def test_uniform_and_bounded_statistics():
    vals = np.array([ob.draw4(99, 0, 5, e, 3) for e in range(20000)], np.uint64).ravel()
    u = ((vals >> 8) + 1).astype(np.float64) / 2**24
    assert u.min() > 0.0 and u.max() <= 1.0
    hist = np.histogram(u, bins=20, range=(0, 1))[0]
    expect = vals.size / 20
    chi2 = ((hist - expect) ** 2 / expect).sum()
    assert chi2 < 50.0  # 19 dof; p ~ 1e-4
    b = (vals * 7) >> 32
    assert set(np.unique(b)) == set(range(7))


@pytest.mark.parametrize("n", [1, 2, 3, 17, 1000, 4097])
def test_seed_perm_is_bijection(n):
    out = [ob.perm(42, 3, 1, n, j) for j in range(n)]
    assert sorted(out) == list(range(n))


def _run_checked(w, steps, quirks):
    sp = w.parameter.simulation
    sp.quirks = quirks
    o = ob.OracleSim(sp, w.network, w.n_sizes, w.m_sizes, w.max_time, w.seed)
    o.init()
    S, P = int(sp.nStrains), w.network.subPopTotal
    N, M = int(sp.nSize), int(sp.mSize)
    prev_imm = None
    for t in range(steps):
        infh, infm, mcnt = recount(o, S, P)
        assert np.array_equal(infh, o.counters("n_infected_subpop")), t
        if quirks == 0:
            assert np.array_equal(infm, o.counters("m_infected_subpop")), t
        assert np.array_equal(mcnt, o.counters("m_subpop_count")), t
        assert o.series("n_count")[t] == N
        assert o.series("m_count")[t] == mcnt.sum()
        assert np.all(o.counters("m_dead_count") >= 0)
        st = o.census("n_status")
        imm = o.census("n_immunity")
        # an infected or infectious human is immune to the serotype it carries
        sel = st > 0
        assert np.all((imm[sel] >> o.census("n_strain")[sel]) & 1)
        if prev_imm is not None:
            # immunity only grows, except for newborns (age 0)
            born = o.census("n_age") == 0
            assert np.all(((prev_imm & ~imm) == 0) | born)
        prev_imm = imm
        o.step(1)
    return o


@pytest.mark.parametrize("quirks", [0, 3])
def test_oracle_invariants(quirks):
    w = small_case(n=1500, m=5000, side=4, T=30, seed=99)
    o = _run_checked(w, 30, quirks)
    assert o.series("n_incidence").sum() > 0
    assert o.series("m_infected")[1:].sum() > 0


def test_oracle_plain_small_runs_and_seasonality():
    w = configs.plain_small()
    o = ob.OracleSim(w.parameter.simulation, w.network, w.n_sizes, w.m_sizes, w.max_time, w.seed)
    o.init()
    o.run()
    mc = o.series("m_count")
    E = o.table(4)
    assert mc[0] == 40000 and E[0] == 40000.0
    # alive mosquitoes track the capped seasonal target within a few percent
    rel = np.abs(mc[30:].astype(float) - E[30:]) / E[30:]
    assert np.median(rel) < 0.05
    assert np.all(o.series("n_count") == 10000)
    assert o.series("n_incidence").sum() > 1000


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


@pytest.mark.parametrize("name", ["small_epidemic", "plain_small_60"])
def test_golden_fixtures(name):
    from tests.golden.make_golden import CASES, run_case
    ref = np.load(GOLDEN / f"{name}.npz")
    out = run_case(CASES[name])
    for k in ref.files:
        if k.startswith("census_"):
            assert str(ref[k]) == out[k], k
        else:
            np.testing.assert_array_equal(ref[k], out[k], err_msg=k)
