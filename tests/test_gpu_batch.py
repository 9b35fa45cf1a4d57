"""Heterogeneous batches (one CUDA graph) against individual ensemble runs.

Every item of a batch must give exactly what Network.run_ensemble gives for
the same network, inputs and seeds -- which the parity tests pin to the
oracle -- whether it ran as thread units or a warp per trajectory in the
persistent launch, merged with other parameter sets, or alone; and again when
the captured graph is replayed with new seeds.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rb():
    import rebop_gb300

    return rebop_gb300


def _mm(rb):
    n = rb.Network(4)  # E, S, ES, P
    n.add_reaction(rb.Rate.lma(0.01, [1, 1, 0, 0]), [-1, -1, 1, 0])
    n.add_reaction(rb.Rate.lma(0.1, [0, 0, 1, 0]), [1, 1, -1, 0])
    n.add_reaction(rb.Rate.lma(0.05, [0, 0, 1, 0]), [1, 0, -1, 1])
    return n


def _check(b, k, net, x0, seeds, tmax, nb, rates=None, save=None):
    ref = net.run_ensemble(x0, seeds, tmax, nb, rates=rates, save=save)
    np.testing.assert_array_equal(b.counts(k), ref.counts)
    np.testing.assert_array_equal(b.events(k), ref.events)


def test_batch_matches_individual_runs(rb):
    import bench
    from rebop_gb300 import expr as E

    rng = np.random.default_rng(5)
    b = rb.Batch()
    specs = []
    mm = _mm(rb)
    for k in range(40):  # Michaelis-Menten parameter sets
        rates = 10 ** rng.uniform(-3, 1, 3)
        x0 = [int(rng.integers(10, 101)), int(rng.integers(100, 1001)), 0, 0]
        seeds = rng.integers(np.iinfo(np.uint64).max, size=8, dtype=np.uint64)
        specs.append((b.add(mm, x0, seeds, 5.0, 10, rates=rates), mm, x0, seeds, 5.0, 10, rates, None))
    for k, (S, R) in enumerate([(8, 16), (24, 80), (64, 256), (40, 120)]):  # random networks
        reactions, _ = bench.random_network(100 + k, S, R)
        net = rb.Network(S)
        for kk, e, d in reactions:
            net.add_reaction(rb.Rate.lma(kk, e), d)
        x0 = rng.integers(0, 501, size=S).tolist()
        seeds = rng.integers(np.iinfo(np.uint64).max, size=16, dtype=np.uint64)
        save = list(range(0, S, 3))
        specs.append((b.add(net, x0, seeds, 2e-3, 6, save=save), net, x0, seeds, 2e-3, 6, None, save))
    # a rate expression and per-trajectory rates: launches of their own
    en = rb.Network(2)
    en.add_reaction(rb.Rate.expression(E.parse("3 + A / 4").to_expr({"A": 0}, {})), [1, 0])
    en.add_reaction(rb.Rate.lma(0.5, [1, 0]), [-1, 1])
    seeds = rng.integers(np.iinfo(np.uint64).max, size=32, dtype=np.uint64)
    specs.append((b.add(en, [0, 0], seeds, 4.0, 8), en, [0, 0], seeds, 4.0, 8, None, None))
    per = np.stack([10 ** rng.uniform(-3, 1, 32) for _ in range(3)], axis=1)
    seeds = rng.integers(np.iinfo(np.uint64).max, size=32, dtype=np.uint64)
    specs.append((b.add(mm, [30, 300, 0, 0], seeds, 5.0, 10, rates=per), mm, [30, 300, 0, 0], seeds, 5.0, 10,
                  per, None))
    n_own, n_persistent = b.plan()
    # one persistent launch: the Michaelis-Menten sets, the per-trajectory-rate
    # item and the 8-species 16-reaction network as thread units, the larger
    # networks a warp per trajectory; the rate expression runs alone
    assert n_own == 1 and n_persistent == 45
    st = b.run()
    assert st["mapping"] == 6 and st["events"] > 0 and st["kernel_launches"] == 2
    for k, net, x0, seeds, tmax, nb, rates, save in specs:
        _check(b, k, net, x0, seeds, tmax, nb, rates, save)
    assert {b.mapping(k) for k in list(range(41)) + [45]} == {7}
    assert {b.mapping(k) for k in range(41, 44)} == {5}
    assert b.mapping(44) == 0
    # replay the captured graph with new seeds
    for k, net, x0, seeds, tmax, nb, rates, save in specs:
        b.seeds(k)[:] = rng.integers(np.iinfo(np.uint64).max, size=b.seeds(k).size, dtype=np.uint64)
    st2 = b.run()
    for k, net, x0, seeds, tmax, nb, rates, save in specs:
        _check(b, k, net, x0, b.seeds(k), tmax, nb, rates, save)


def _macro_dsl(rng, S, R):
    """A define_system! body over species s0..s{S-1} with R reactions of order
    <= 2 and numeric rates, and its oracle (macro arithmetic) copy."""
    from oracle import oracle as O

    lines = [";", "Net { " + ", ".join(f"s{i}" for i in range(S)) + " }"]
    onet = O.OracleNet(S, macro=True)
    for k in range(R):
        a = int(rng.integers(S))
        factors = [(a, 2)] if rng.random() < 0.3 else [(a, 1)] + ([(int(rng.integers(S)), 1)] if rng.random() < 0.5 else [])
        if len(factors) == 2 and factors[0][0] == factors[1][0]:
            factors = [(factors[0][0], 2)]
        prods = [int(p) for p in rng.integers(S, size=int(rng.integers(0, 3)))]
        rate = float(10 ** rng.uniform(-3, -1))
        lhs = " + ".join(f"{n} s{sp}" if n > 1 else f"s{sp}" for sp, n in factors)
        rhs = " + ".join(f"s{sp}" for sp in prods)
        lines.append(f"r{k} : {lhs} => {rhs} @ {rate!r}")
        d = [0] * S
        for sp, n in factors:
            d[sp] -= n
        for sp in prods:
            d[sp] += 1
        onet.add_macro(rate, factors, d)
    return "\n".join(lines), onet


def test_batch_of_define_system_networks(rb):
    # define_system! arithmetic (falling factorials in integers, the first-match
    # choice) inside the persistent launch: dimer parameter sets as thread
    # units, 20-species 40-reaction networks a warp per trajectory; every item
    # against the oracle's macro arithmetic
    from oracle import oracle as O

    rng = np.random.default_rng(12)
    b = rb.Batch()
    specs = []
    dim = rb.Network.from_dsl("""
        ;
        Dimers { gene, mRNA, protein, dimer }
        transcription : gene => gene + mRNA @ 25.0
        translation : mRNA => mRNA + protein @ 1000.0
        dimerization : 2 protein => dimer @ 0.001
        decay_mRNA : mRNA => @ 0.1
        decay_prot : protein => @ 1.0
    """)
    for k in range(12):
        rates = np.array([25.0, 1000.0, 0.001, 0.1, 1.0]) * 10 ** rng.uniform(-0.5, 0.5, 5)
        seeds = rng.integers(np.iinfo(np.uint64).max, size=8, dtype=np.uint64)
        o = (O.OracleNet(4, macro=True).add_macro(rates[0], [(0, 1)], [0, 1, 0, 0])
             .add_macro(rates[1], [(1, 1)], [0, 0, 1, 0]).add_macro(rates[2], [(2, 2)], [0, 0, -2, 1])
             .add_macro(rates[3], [(1, 1)], [0, -1, 0, 0]).add_macro(rates[4], [(2, 1)], [0, 0, -1, 0]))
        specs.append((b.add(dim, [1, 0, 0, 0], seeds, 0.3, 6, rates=rates), o, [1, 0, 0, 0], seeds, 0.3, 6))
    for k in range(3):
        text, o = _macro_dsl(rng, 20, 40)
        net = rb.Network.from_dsl(text)
        x0 = rng.integers(20, 80, size=20).tolist()
        seeds = rng.integers(np.iinfo(np.uint64).max, size=16, dtype=np.uint64)
        specs.append((b.add(net, x0, seeds, 0.05, 5), o, x0, seeds, 0.05, 5))
    assert b.plan() == (0, 15)  # one persistent launch in macro arithmetic
    b.run()
    for k, o, x0, seeds, tmax, nb in specs:
        ref, ev, _, _ = o.run_ensemble(x0, seeds, tmax, nb)
        assert ev.sum() > 100
        np.testing.assert_array_equal(b.counts(k), ref)
        np.testing.assert_array_equal(b.events(k), ev)
    assert {b.mapping(k) for k in range(12)} == {7} and {b.mapping(k) for k in range(12, 15)} == {5}


@pytest.mark.parametrize("mode", ["persistent", "merged"])
def test_batch_results_in_place(rb, monkeypatch, mode):
    # Items added without output arrays: their results are read where the
    # batch keeps them (the staging buffer, or the batch's own copy for a
    # merged class) and equal the copied results of the same items, before and
    # after a replay with new seeds.
    import bench

    monkeypatch.setenv("RB_BATCH_MODE", mode)
    if mode == "merged":
        monkeypatch.setenv("RB_BATCH_MIN_THREAD", "1")
    rng = np.random.default_rng(13)
    mm = _mm(rb)
    reactions, _ = bench.random_network(130, 30, 90)
    net = rb.Network(30)
    for kk, e, d in reactions:
        net.add_reaction(rb.Rate.lma(kk, e), d)
    specs = []
    for k in range(6):
        specs.append((mm, [int(rng.integers(10, 101)), 500, 0, 0], 10 ** rng.uniform(-3, 1, 3), 3.0, 8, [1, 3]))
    specs.append((net, rng.integers(0, 501, size=30).tolist(), None, 2e-3, 5, None))
    seeds = [rng.integers(np.iinfo(np.uint64).max, size=24, dtype=np.uint64) for _ in specs]
    a, v = rb.Batch(), rb.Batch()
    for (n, x0, rates, tmax, nb, save), sd in zip(specs, seeds):
        a.add(n, x0, sd.copy(), tmax, nb, rates=rates, save=save)
        v.add(n, x0, sd.copy(), tmax, nb, rates=rates, save=save, copy=False)
    for rep in range(2):
        a.run()
        v.run()
        for k in range(len(specs)):
            np.testing.assert_array_equal(v.counts(k), a.counts(k))
            np.testing.assert_array_equal(v.events(k), a.events(k))
        for k in range(len(specs)):
            fresh = rng.integers(np.iinfo(np.uint64).max, size=24, dtype=np.uint64)
            a.seeds(k)[:] = fresh
            v.seeds(k)[:] = fresh


def test_batch_merges_parameter_sets(rb, monkeypatch):
    # The merged plan: with every class worth a launch, parameter sets of one
    # network run as one thread-per-trajectory ensemble with per-trajectory
    # rates and counts.
    monkeypatch.setenv("RB_BATCH_MODE", "merged")
    monkeypatch.setenv("RB_BATCH_MIN_THREAD", "1")
    rng = np.random.default_rng(6)
    b = rb.Batch()
    mm = _mm(rb)
    specs = []
    for k in range(30):
        rates = 10 ** rng.uniform(-3, 1, 3)
        x0 = [int(rng.integers(10, 101)), int(rng.integers(100, 1001)), 0, 0]
        seeds = rng.integers(np.iinfo(np.uint64).max, size=int(rng.integers(1, 20)), dtype=np.uint64)
        specs.append((b.add(mm, x0, seeds, 3.0, 12, rates=rates, save=[1, 3]), x0, seeds, rates))
    assert b.plan() == (1, 0)
    b.run()
    for k, x0, seeds, rates in specs:
        _check(b, k, mm, x0, seeds, 3.0, 12, rates, [1, 3])
        assert b.mapping(k) in (2, 3, 4)


def test_batch_of_networks_beyond_256_reactions(rb):
    # Warp batch items whose lanes own more than 8 reactions each: their chunk
    # sums are longer sequential chains, which the error bound must count.
    import bench

    rng = np.random.default_rng(9)
    b = rb.Batch()
    specs = []
    for k, (S, R) in enumerate([(50, 400), (30, 300)]):
        reactions, _ = bench.random_network(200 + k, S, R)
        net = rb.Network(S)
        for kk, e, d in reactions:
            net.add_reaction(rb.Rate.lma(kk, e), d)
        x0 = rng.integers(0, 501, size=S).tolist()
        seeds = rng.integers(np.iinfo(np.uint64).max, size=24, dtype=np.uint64)
        specs.append((b.add(net, x0, seeds, 1e-3, 5), net, x0, seeds, 1e-3, 5, None, None))
    n_own, n_persistent = b.plan()
    assert n_persistent == 2 and n_own == 0
    st = b.run()
    assert st["events"] > 0
    for k, net, x0, seeds, tmax, nb, rates, save in specs:
        _check(b, k, net, x0, seeds, tmax, nb, rates, save)
        assert b.mapping(k) == 5


def test_bench_batch_against_oracle(rb, O):
    # The bench's whole heterogeneous batch (4096 Michaelis-Menten parameter
    # sets and 1024 random networks of 8-64 species and 16-256 reactions, 64
    # trajectories each) runs once; every 16th parameter set, every 8th random
    # network and every random network of 240 reactions or more are compared
    # with the oracle, bit for bit, before and after a replay with new seeds.
    import bench

    items = bench.batch_items()
    b, _ = bench.make_batch(rb, items, want_events=True)
    n_mm = bench.BATCH["n_mm"]
    pick = [j for j in range(len(items))
            if (j < n_mm and j % 16 == 0) or (j >= n_mm and ((j - n_mm) % 8 == 0 or len(items[j][1]) >= 240))]
    assert len(pick) > 400
    for step in range(2):
        if step:
            for j in range(len(items)):
                b.seeds(j)[:] = bench.batch_seeds(1, j)
        st = b.run()
        assert st["events"] > 0
        for j in pick:
            net, tmax = bench.batch_oracle_net(O, items[j])
            ref, ev, _, _ = net.run_ensemble(items[j][2], b.seeds(j), tmax, bench.BATCH["nb_steps"])
            np.testing.assert_array_equal(b.counts(j), ref, err_msg=f"item {j} (step {step})")
            np.testing.assert_array_equal(b.events(j), ev, err_msg=f"item {j} (step {step})")
