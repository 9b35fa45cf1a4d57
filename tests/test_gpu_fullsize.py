"""Parity at the benchmark configurations' full sizes.

The kernels schedule differently at full occupancy (slots rotated over lanes,
warps refilled from the trajectory queue), so each configuration runs at its
full size here.  Trajectories are independent and keyed by their seeds: any
subset the oracle can afford must match bit for bit, and size-independent
properties (conservation laws, non-negative counts, event totals) must hold
for every trajectory.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rb():
    import rebop_gb300

    return rebop_gb300


def _seeds(n, salt):
    return np.random.default_rng(777 + salt).integers(np.iinfo(np.uint64).max, size=n, dtype=np.uint64)


def test_dimer_full_size(rb, O):
    # 1e5 trajectories, tmax 1, 101 samples: the bench's workload
    import bench

    w = bench.DIMER
    net = rb.Network(4)
    for k, e, d in w["reactions"]:
        net.add_reaction(rb.Rate.lma(k, e), d)
    seeds = _seeds(100_000, 1)
    res = net.run_ensemble(w["x0"], seeds, 1.0, 100)
    assert res.stats["mapping"] == 4
    # every trajectory (about 1.7e9 events) against the oracle
    ref, ev, _, _ = O.dimer_net().run_ensemble(w["x0"], seeds, 1.0, 100)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    c = res.counts
    assert (c >= 0).all()
    assert (c[:, 0, :] == 1).all()  # the gene is never consumed
    assert res.total_events == int(res.events.sum())


def test_sir_full_size(rb, O):
    # tests/test_rebop.py:15-27 conservation, at 1e4 trajectories, all compared
    import bench

    w = bench.SIR
    net = rb.Network(3)
    for k, e, d in w["reactions"]:
        net.add_reaction(rb.Rate.lma(k, e), d)
    seeds = _seeds(10_000, 2)
    res = net.run_ensemble(w["x0"], seeds, 250.0, 250)
    ref, ev, _, _ = O.sir_net().run_ensemble(w["x0"], seeds, 250.0, 250)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    assert (res.counts.sum(axis=1) == 1000).all()


def test_large_network_full_size(rb, O):
    # 200 species x 1000 reactions, 1e4 trajectories of ~1e5 events on the warp
    # kernel; 256 of them (about 2.5e7 events) against the oracle
    import bench

    w = bench.LARGE
    net = rb.Network(w["S"])
    onet = O.OracleNet(w["S"])
    for k, e, d in w["reactions"]:
        net.add_reaction(rb.Rate.lma(k, e), d)
        onet.add_lma_sparse(k, [(i, x) for i, x in enumerate(e) if x], d)
    seeds = _seeds(10_000, 3)
    res = net.run_ensemble(w["x0"], seeds, w["tmax"], w["nb_steps"])
    assert res.stats["mapping"] == 5
    assert res.events.mean() > 5e4
    pick = np.unique(np.concatenate([np.arange(0, 10_000, 38), [1, 9998, 9999]]))
    assert pick.size >= 256
    ref, ev, _, _ = onet.run_ensemble(w["x0"], seeds[pick], w["tmax"], w["nb_steps"])
    np.testing.assert_array_equal(res.counts[:, :, pick], ref)
    np.testing.assert_array_equal(res.events[pick], ev)
    assert (res.counts >= 0).all()
