"""The autotuner on the GPU: pilot runs, the remembered winner, and runs that
use it -- bit-exact with the oracle whichever kernel wins."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tune_then_run_with_the_winner(O, tmp_path, monkeypatch):
    import rebop_gb300 as rb
    from rebop_gb300._lib import lib

    monkeypatch.setenv("RB_TUNE_CACHE", str(tmp_path / "tune.txt"))
    lib.rb_tune_clear(0)
    try:
        net = rb.Network(4)
        for k, e, d in [(25.0, [1, 0, 0, 0], [0, 1, 0, 0]), (1000.0, [0, 1, 0, 0], [0, 0, 1, 0]),
                        (0.001, [0, 0, 2, 0], [0, 0, -2, 1]), (0.1, [0, 1, 0, 0], [0, -1, 0, 0]),
                        (1.0, [0, 0, 1, 0], [0, 0, -1, 0])]:
            net.add_reaction(rb.Rate.lma(k, e), d)
        n = 20_000  # above the spreading threshold: block sizes are tuned too
        r = net.tune([1, 0, 0, 0], n, 0.3, 12)
        best, trials = r["best"], r["trials"]
        timed = [t for t in trials if t["ms"] >= 0]
        assert {t["mapping"] for t in trials} >= {4, 3, 2}
        assert any(t["block"] == 512 for t in trials)
        assert best["ms"] == min(t["ms"] for t in timed)
        assert (tmp_path / "tune.txt").exists()
        assert net.tuned(n) == best
        seeds = np.random.default_rng(11).integers(np.iinfo(np.uint64).max, size=n, dtype=np.uint64)
        res = net.run_ensemble([1, 0, 0, 0], seeds, 0.3, 12)
        assert res.stats["mapping"] == best["mapping"]
        ref, ev, _, _ = O.dimer_net().run_ensemble([1, 0, 0, 0], seeds, 0.3, 12)
        np.testing.assert_array_equal(res.counts, ref)
        np.testing.assert_array_equal(res.events, ev)
    finally:
        lib.rb_tune_clear(1)
