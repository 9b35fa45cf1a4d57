"""The oracle (C restatement of the reference path) against the reference's own goldens.

Everything here runs on the CPU: it pins the oracle before any GPU result is
compared with it.
"""

import math

import numpy as np
import pytest


def test_rate_lma_known_answers(O, goldens):
    # src/gillespie.rs:448-472: every case, dense and sparse forms.
    assert len(goldens["rate_lma"]) == 16
    for case in goldens["rate_lma"]:
        S = len(case["species"])
        dense = O.OracleNet(S).add_lma(case["rate"], case["exponents"], [0] * S)
        pairs = [(i, e) for i, e in enumerate(case["exponents"]) if e > 0]
        sparse = O.OracleNet(S).add_lma_sparse(case["rate"], pairs, [0] * S)
        assert dense.rate(0, case["species"]) == case["expected"], case["where"]
        assert sparse.rate(0, case["species"]) == case["expected"], case["where"]


def test_jump_affect_known_answer(O, goldens):
    # src/gillespie.rs:484-494
    case = goldens["jump_affect"][0]
    S = len(case["species"])
    net = O.OracleNet(S).add_lma(1.0, [0] * S, case["differences"])
    assert net.affect(0, case["species"]).tolist() == case["expected"]


def test_fixed_seed_golden(O, goldens):
    # tests/test_rebop.py:30-36: SIR, rng=42 -> final (S, I, R) = (0, 227, 773).
    fs = goldens["fixed_seed"]
    seed = O.numpy_seed(fs["rng"])
    assert seed == fs["numpy_seed"]
    net = O.sir_net()
    x0 = [fs["init"].get(s, 0) for s in ("S", "I", "R")]
    out, ev, tot, _ = net.run_ensemble(x0, [seed], fs["tmax"], fs["nb_steps"])
    final = out[-1, :, 0].tolist()
    assert final == [fs["final"]["S"], fs["final"]["I"], fs["final"]["R"]]


def test_rng_stream_properties(O):
    # xoshiro256++ / SplitMix64 seeding: distinct seeds give distinct streams,
    # the state is never all zero, and Exp1 draws have mean ~1 and var ~1.
    a = O.draw_u64(0, 1000)
    b = O.draw_u64(1, 1000)
    assert len(set(a.tolist())) == 1000 and not np.array_equal(a, b)
    assert all(int(w) != 0 for w in O.seed_state(0))
    e = O.draw_exp1(12345, 400_000)
    assert e.min() > 0
    assert abs(e.mean() - 1) < 0.01 and abs(e.var() - 1) < 0.02
    # tail beyond the ziggurat base (R = 7.697): P = exp(-R)
    assert abs((e > 7.69711747013105).mean() - math.exp(-7.69711747013105)) < 2e-4


def test_zig_tables_zignor(O):
    x, f = O.zig_tables()
    assert x[1] == 7.69711747013104972 and x[256] == 0.0
    assert np.all(np.diff(x[1:]) < 0)                       # decreasing abscissae
    assert all(f[i] == math.exp(-x[i]) for i in range(257))  # f = exp(-x), libm exp
    # ZIGNOR: every layer above the base has area v = x[i-1] * (f[i] - f[i-1])
    v = 0.0039496598225815571993
    areas = x[1:255] * (f[2:256] - f[1:255])
    assert np.allclose(areas, v, rtol=1e-9)


def test_gillespie_sir_conservation(O):
    # src/gillespie.rs:504-516
    net = (O.OracleNet(3).add_lma(0.1 / 10000.0, [1, 1, 0], [-1, 1, 0])
           .add_lma(0.01, [0, 1, 0], [0, -1, 1]))
    out, _, _, _ = net.run_ensemble([9999, 1, 0], np.arange(4, dtype=np.uint64), 250.0, 250)
    assert np.all(out.sum(axis=1) == 10000)


def test_gillespie_dimers(O):
    # src/gillespie.rs:518-530
    out, _, _, _ = O.dimer_net().run_ensemble([1, 0, 0, 0], np.arange(8, dtype=np.uint64), 1.0, 1)
    final = out[-1]
    assert np.all(final[0] == 1) and np.all(final[2] > 1000) and np.all(final[3] < 10000)


@pytest.mark.parametrize("seed", range(10))
def test_sir_invariants(O, seed):
    # tests/test_rebop.py:15-27
    net = O.sir_net()
    out, _, _, _ = net.run_ensemble([999, 1, 0], [O.numpy_seed(seed)], 250.0, 250)
    S, I, R = out[:, 0, 0], out[:, 1, 0], out[:, 2, 0]
    assert np.all(S >= 0) and np.all(I >= 0) and np.all(R >= 0)
    assert np.all(S <= 999) and np.all(I <= 1000) and np.all(R <= 1000)
    assert np.all(S + I + R == 1000)


@pytest.mark.parametrize("seed", range(10))
def test_all_reactions_invariants(O, seed):
    # tests/test_rebop.py:39-52 (nb_steps = 0)
    times, out = O.sir_net().run_all_events([999, 1, 0], O.numpy_seed(seed), 250.0)
    assert times[0] == 0 and times[-1] > 250
    assert np.all(np.diff(times) > 0)
    if np.isinf(times[-1]):
        out = out[:-1]
    d = np.diff(out, axis=0)
    assert set(d[:, 0].tolist()) <= {-1, 0}
    assert set(d[:, 1].tolist()) <= {-1, 1}
    assert set(d[:, 2].tolist()) <= {0, 1}


def test_dense_vs_sparse(O):
    # tests/test_rebop.py:55-65: the representation does not change results.
    dense = O.sir_net()
    sparse = (O.OracleNet(3).add_lma_sparse(1e-4, [(0, 1), (1, 1)], [-1, 1, 0])
              .add_lma_sparse(0.01, [(1, 1)], [0, -1, 1]))
    seeds = np.arange(16, dtype=np.uint64)
    a = dense.run_ensemble([999, 1, 0], seeds, 250.0, 250)[0]
    b = sparse.run_ensemble([999, 1, 0], seeds, 250.0, 250)[0]
    assert np.array_equal(a, b)


def test_macro_semantics(O):
    # src/gillespie_macro.rs:176-253 with the macro's arithmetic.
    sir = (O.OracleNet(3, macro=True).add_macro(0.1 / 10000.0, [(0, 1), (1, 1)], [-1, 1, 0])
           .add_macro(0.01, [(1, 1)], [0, -1, 1]))
    out = sir.run_ensemble([9999, 1, 0], np.arange(4, dtype=np.uint64), 1000.0, 1)[0]
    assert np.all(out[-1].sum(axis=0) == 10000)
    dim = (O.OracleNet(4, macro=True).add_macro(25.0, [(0, 1)], [0, 1, 0, 0])
           .add_macro(1000.0, [(1, 1)], [0, 0, 1, 0]).add_macro(0.001, [(2, 2)], [0, 0, -2, 1])
           .add_macro(0.1, [(1, 1)], [0, -1, 0, 0]).add_macro(1.0, [(2, 1)], [0, 0, -1, 0]))
    out = dim.run_ensemble([1, 0, 0, 0], np.arange(4, dtype=np.uint64), 1.0, 1)[0]
    assert np.all(out[-1, 0] == 1) and np.all((out[-1, 3] > 1000) & (out[-1, 3] < 10000))
    bd = O.OracleNet(1, macro=True).add_macro(10.0, [], [1]).add_macro(0.1, [(0, 1)], [-1])
    out = bd.run_ensemble([0], np.arange(4, dtype=np.uint64), 100.0, 1)[0]
    assert np.all((out[-1, 0] > 50) & (out[-1, 0] < 200))
    # forgotten parameter: NaN rate -> no reaction at all
    bd_nan = O.OracleNet(1, macro=True).add_macro(10.0, [], [1]).add_macro(math.nan, [(0, 1)], [-1])
    out = bd_nan.run_ensemble([0], [7], 100.0, 1)[0]
    assert out[-1, 0, 0] == 0
    # no reactions: counts unchanged up to t = 1e20
    none = O.OracleNet(3, macro=True)
    out = none.run_ensemble([42, 1337, 0], [1], 1e20, 1)[0]
    assert out[-1, :, 0].tolist() == [42, 1337, 0]


def test_macro_vs_api_order2_rounding(O):
    # The macro multiplies rate * (n(n-1)) (integer factorial), the API rate *
    # (n-1) * n: both are computed as the reference does.
    api = O.OracleNet(1).add_lma(0.001, [2], [-2])
    mac = O.OracleNet(1, macro=True).add_macro(0.001, [(0, 2)], [-2])
    for n in (2, 3, 1000, 12345):
        assert api.rate(0, [n]) == (0.001 * (n - 1)) * n
        assert mac.rate(0, [n]) == 0.001 * float(n * (n - 1))


def test_oracle_rejects_out_of_range_sparse_index(O):
    # src/gillespie.rs:496-502 (issue 85): the reference panics.
    net = O.OracleNet(1).add_lma_sparse(1.0, [(10, 1)], [0])
    assert not net.validate()


def test_advance_until_is_resumable(O):
    # Gillespie state = (species, t, rng): two advance_until calls equal the
    # sampled run at the same times.
    net = O.dimer_net()
    st = O.seed_state(99)
    sp, t, st, ev0, _, _ = net.advance_until([1, 0, 0, 0], 0.0, st, 0.0)
    sp, t, st, ev1, _, _ = net.advance_until(sp, t, st, 0.5)
    sp, t, st, ev2, _, _ = net.advance_until(sp, t, st, 1.0)
    out = net.run_ensemble([1, 0, 0, 0], [99], 1.0, 2)[0]
    assert sp.tolist() == out[-1, :, 0].tolist() and t == 1.0


def test_birth_death_matches_poisson_law(O):
    # Statistical check independent of any stream: for births at k1 and
    # deaths at k2 * n from n = 0, n(t) is Poisson with mean
    # k1 / k2 * (1 - exp(-k2 t)) at every t.  Means, variances and the KS
    # distance to that law, at every sample time, within 5 standard errors.
    from scipy import stats

    k1, k2, n_traj = 20.0, 1.0, 4000
    net = O.OracleNet(1).add_lma(k1, [0], [1]).add_lma(k2, [1], [-1])
    seeds = np.random.default_rng(77).integers(np.iinfo(np.uint64).max, size=n_traj, dtype=np.uint64)
    out, _, _, _ = net.run_ensemble([0], seeds, 5.0, 10, n_threads=4)
    for i in range(1, 11):
        t = 0.5 * i
        m = k1 / k2 * (1.0 - math.exp(-k2 * t))
        x = out[i, 0, :].astype(float)
        assert abs(x.mean() - m) < 5 * math.sqrt(m / n_traj), (t, x.mean(), m)
        assert abs(x.var() - m) < 5 * math.sqrt((m + 2 * m * m) / n_traj), (t, x.var(), m)
        vals = np.arange(0, int(x.max()) + 1)
        ecdf = np.searchsorted(np.sort(x), vals, side="right") / n_traj
        assert np.max(np.abs(ecdf - stats.poisson.cdf(vals, m))) < 1.63 / math.sqrt(n_traj) * 1.5, t


def test_generator_step_back_inverts_the_state_update(O):
    # The float-pair step draws ahead and steps the generator back when it
    # commits fewer draws (xo_prev in rebop_gb300/csrc/rng.cuh): restated here
    # on the oracle's own stream, stepping forward n times and back n times
    # returns the seeded state, and every output in between is the oracle's.
    M = (1 << 64) - 1

    def rotl(x, k):
        return ((x << k) | (x >> (64 - k))) & M

    def step(s):
        s0, s1, s2, s3 = s
        out = (rotl((s0 + s3) & M, 23) + s0) & M
        t = (s1 << 17) & M
        s2 ^= s0
        s3 ^= s1
        s1 ^= s2
        s0 ^= s3
        s2 ^= t
        return out, [s0, s1, s2, rotl(s3, 45)]

    def back(s):
        d1 = rotl(s[3], 19)
        y = s[1] ^ s[2]
        b = (y ^ (y << 17) ^ (y << 34) ^ (y << 51)) & M
        a = s[0] ^ d1
        return [a, b, s[1] ^ b ^ a, d1 ^ b]

    for seed in (0, 1, 42, 2**63 + 5):
        st0 = [int(w) for w in O.seed_state(seed)]
        ref = O.draw_u64(seed, 64)
        s, states = st0, [st0]
        for k in range(64):
            out, s = step(s)
            assert out == int(ref[k])
            states.append(s)
        for k in range(64, 0, -1):
            s = back(s)
            assert s == states[k - 1]
