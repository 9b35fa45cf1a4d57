"""Heterogeneous batches (one CUDA graph) against individual ensemble runs.

Every item of a batch must give exactly what Network.run_ensemble gives for
the same network, inputs and seeds -- which the parity tests pin to the
oracle -- whether it ran merged with other parameter sets, in the warp
kernel's batch mode, or alone; and again when the captured graph is replayed
with new seeds.
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
    n_thread, n_warp = b.plan()
    # the 8-species network and both Michaelis-Menten forms run on thread
    # kernels, the expression alone; three random networks share the warp batch
    assert n_warp == 3 and n_thread == 3
    st = b.run()
    assert st["mapping"] == 6 and st["events"] > 0
    for k, net, x0, seeds, tmax, nb, rates, save in specs:
        _check(b, k, net, x0, seeds, tmax, nb, rates, save)
    # thread classes: generated kernels from 4096 trajectories up, below that
    # the descriptor kernels
    assert {b.mapping(k) for k in range(41)} <= {2, 3, 4}
    assert {b.mapping(k) for k in range(41, 44)} == {5}
    assert b.mapping(44) == 0 and b.mapping(45) in (2, 3, 4)
    # replay the captured graph with new seeds
    for k, net, x0, seeds, tmax, nb, rates, save in specs:
        b.seeds(k)[:] = rng.integers(np.iinfo(np.uint64).max, size=b.seeds(k).size, dtype=np.uint64)
    st2 = b.run()
    for k, net, x0, seeds, tmax, nb, rates, save in specs:
        _check(b, k, net, x0, b.seeds(k), tmax, nb, rates, save)
