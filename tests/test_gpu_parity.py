"""GPU parity: the engine's kernels against the oracle, bit for bit.

Integer counts, event counts and reaction sequences must be identical; the
random stream is the reference's (xoshiro256++ / ziggurat Exp1) keyed by the
same seed on both sides.
"""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rb():
    import rebop_gb300

    return rebop_gb300


def _sir(rb, k1=1e-4, k2=0.01):
    n = rb.Network(3)
    n.add_reaction(rb.Rate.lma(k1, [1, 1, 0]), [-1, 1, 0])
    n.add_reaction(rb.Rate.lma(k2, [0, 1, 0]), [0, -1, 1])
    return n


def _dimer(rb):
    n = rb.Network(4)
    n.add_reaction(rb.Rate.lma(25.0, [1, 0, 0, 0]), [0, 1, 0, 0])
    n.add_reaction(rb.Rate.lma(1000.0, [0, 1, 0, 0]), [0, 0, 1, 0])
    n.add_reaction(rb.Rate.lma(0.001, [0, 0, 2, 0]), [0, 0, -2, 1])
    n.add_reaction(rb.Rate.lma(0.1, [0, 1, 0, 0]), [0, -1, 0, 0])
    n.add_reaction(rb.Rate.lma(1.0, [0, 0, 1, 0]), [0, 0, -1, 0])
    return n


def _seeds(n, salt=0):
    return np.random.default_rng(1234 + salt).integers(np.iinfo(np.uint64).max, size=n, dtype=np.uint64)


def test_fixed_seed_golden_through_dropin(rb, goldens):
    # tests/test_rebop.py:30-36 through the Python drop-in, on the GPU.
    fs = goldens["fixed_seed"]
    sir = rb.Gillespie()
    sir.add_reaction(1e-4, ["S", "I"], ["I", "I"])
    sir.add_reaction(0.01, ["I"], ["R"])
    ds = sir.run(fs["init"], tmax=fs["tmax"], nb_steps=fs["nb_steps"], rng=fs["rng"])
    np.testing.assert_array_equal(np.asarray(ds.time), np.arange(251))
    assert [int(ds[s][-1]) for s in ("S", "I", "R")] == [fs["final"][s] for s in ("S", "I", "R")]


def test_dense_vs_sparse_through_dropin(rb, O, goldens):
    # tests/test_rebop.py:55-65: sparse=None / False / True at rng=42 give the
    # same dataset.  The drop-in runs all three on the GPU; the oracle runs the
    # reference's dense (Rate::lma) and sparse (Rate::lma_sparse) forms with
    # the seed the reference's wrapper derives from rng=42.
    sir = rb.Gillespie()
    sir.add_reaction(1e-4, ["S", "I"], ["I", "I"])
    sir.add_reaction(0.01, ["I"], ["R"])
    init, tmax, nb_steps, seed = {"S": 999, "I": 1}, 250, 250, 42
    ds_auto = sir.run(init, tmax=tmax, nb_steps=nb_steps, rng=seed, sparse=None)
    ds_dense = sir.run(init, tmax=tmax, nb_steps=nb_steps, rng=seed, sparse=False)
    ds_sparse = sir.run(init, tmax=tmax, nb_steps=nb_steps, rng=seed, sparse=True)
    for s in ("S", "I", "R"):
        np.testing.assert_array_equal(np.asarray(ds_dense[s]), np.asarray(ds_auto[s]))
        np.testing.assert_array_equal(np.asarray(ds_dense[s]), np.asarray(ds_sparse[s]))
    np.testing.assert_array_equal(np.asarray(ds_dense.time), np.asarray(ds_sparse.time))
    s64 = O.numpy_seed(seed)
    dense, _, _, _ = O.sir_net().run_ensemble([999, 1, 0], [s64], float(tmax), nb_steps)
    sp = (O.OracleNet(3).add_lma_sparse(1e-4, [(0, 1), (1, 1)], [-1, 1, 0])
          .add_lma_sparse(0.01, [(1, 1)], [0, -1, 1]))
    sparse, _, _, _ = sp.run_ensemble([999, 1, 0], [s64], float(tmax), nb_steps)
    np.testing.assert_array_equal(dense, sparse)
    for k, s in enumerate(("S", "I", "R")):
        np.testing.assert_array_equal(np.asarray(ds_dense[s]), dense[:, k, 0])
    fs = goldens["fixed_seed"]
    assert [int(ds_sparse[s][-1]) for s in ("S", "I", "R")] == [fs["final"][s] for s in ("S", "I", "R")]


def test_sir_ensemble_bit_exact(rb, O):
    seeds = _seeds(1000)
    res = _sir(rb).run_ensemble([999, 1, 0], seeds, 250.0, 250)
    ref, ev, tot, _ = O.sir_net().run_ensemble([999, 1, 0], seeds, 250.0, 250)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    assert res.total_events == tot
    np.testing.assert_array_equal(res.times, np.arange(251.0))


def test_dimer_ensemble_bit_exact(rb, O):
    seeds = _seeds(1500, 1)
    res = _dimer(rb).run_ensemble([1, 0, 0, 0], seeds, 1.0, 100, want_final=True)
    ref, ev, tot, fin = O.dimer_net().run_ensemble([1, 0, 0, 0], seeds, 1.0, 100, want_final=True)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    np.testing.assert_array_equal(res.final, fin)
    assert res.total_events == tot > 1500 * 10_000


def test_per_trajectory_x0_rates_and_saved_subset(rb, O):
    n = 700
    rng = np.random.default_rng(5)
    x0 = np.stack([rng.integers(500, 1500, n), rng.integers(1, 20, n), np.zeros(n, np.int64)], axis=1)
    rates = np.stack([10 ** rng.uniform(-5, -3, n), 10 ** rng.uniform(-3, -1, n)], axis=1)
    seeds = _seeds(n, 2)
    res = _sir(rb).run_ensemble(x0, seeds, 100.0, 37, rates=rates, save=[2, 0])
    ref, ev, _, _ = O.sir_net().run_ensemble(x0, seeds, 100.0, 37, save_idx=[2, 0], rates=rates)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)


def test_sparse_pairs_in_caller_order(rb, O):
    # Rate::lma_sparse multiplies its pairs in the given order (gillespie.rs:79-86);
    # a repeated index multiplies twice.
    net = rb.Network(3)
    net.add_reaction(rb.Rate.lma_sparse(3e-4, [(1, 1), (0, 1)]), [-1, 1, 0])
    net.add_reaction(rb.Rate.lma_sparse(1e-6, [(1, 1), (1, 1)]), [0, -1, 1])
    net.add_reaction(rb.Rate.lma(0.02, [0, 1, 0]), [0, -1, 1])
    o = (O.OracleNet(3).add_lma_sparse(3e-4, [(1, 1), (0, 1)], [-1, 1, 0])
         .add_lma_sparse(1e-6, [(1, 1), (1, 1)], [0, -1, 1]).add_lma(0.02, [0, 1, 0], [0, -1, 1]))
    seeds = _seeds(300, 3)
    res = net.run_ensemble([900, 5, 0], seeds, 60.0, 30)
    ref, ev, _, _ = o.run_ensemble([900, 5, 0], seeds, 60.0, 30)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)


DIMER_DSL = """
    rtx rtl rdi rdm rdp;
    Dimers { gene, mRNA, protein, dimer }
    transcription   : gene      => gene + mRNA      @ rtx
    translation     : mRNA      => mRNA + protein   @ rtl
    dimerization    : 2 protein => dimer            @ rdi
    decay_mRNA      : mRNA      =>                  @ rdm
    decay_prot      : protein   =>                  @ rdp
"""


def test_define_system_bit_exact(rb, O):
    D = rb.define_system(DIMER_DSL)
    d = D.with_parameters(25.0, 1000.0, 0.001, 0.1, 1.0)
    d.gene = 1
    seeds = _seeds(400, 4)
    res = d.run_ensemble(seeds, 1.0, 20)
    o = (O.OracleNet(4, macro=True).add_macro(25.0, [(0, 1)], [0, 1, 0, 0])
         .add_macro(1000.0, [(1, 1)], [0, 0, 1, 0]).add_macro(0.001, [(2, 2)], [0, 0, -2, 1])
         .add_macro(0.1, [(1, 1)], [0, -1, 0, 0]).add_macro(1.0, [(2, 1)], [0, 0, -1, 0]))
    ref, ev, _, _ = o.run_ensemble([1, 0, 0, 0], seeds, 1.0, 20)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    # the struct API: seed + advance_until, gillespie_macro.rs:192-208
    d2 = D.with_parameters(25.0, 1000.0, 0.001, 0.1, 1.0)
    d2.gene = 1
    d2.seed(int(seeds[0]))
    d2.advance_until(1.0)
    assert d2.t == 1.0 and d2.gene == 1 and 1000 < d2.dimer < 10000


def test_define_system_forgotten_parameter_and_no_reactions(rb):
    BD = rb.define_system("r_birth r_death; BirthDeath { A } birth: => A @ r_birth death: A => @ r_death")
    bd = BD.new()
    bd.r_birth = 10.0
    bd.advance_until(100.0)  # r_death is NaN: no reaction (gillespie_macro.rs:225-238)
    assert bd.t == 100.0 and bd.A == 0
    F = rb.define_system("; FooBarBuz { Foo, Bar, Buz }")
    f = F.new()
    f.Foo, f.Bar = 42, 1337
    f.advance_until(1e20)
    assert f.t == 1e20 and (f.Foo, f.Bar, f.Buz) == (42, 1337, 0)


def test_rust_api_stateful_trajectory(rb, O):
    # Gillespie::new_with_seed + repeated advance_until (gillespie.rs:301-344).
    g = rb.api.Gillespie.new_with_seed([1, 0, 0, 0], False, 777)
    g.add_reaction(rb.Rate.lma(25.0, [1, 0, 0, 0]), [0, 1, 0, 0])
    g.add_reaction(rb.Rate.lma(1000.0, [0, 1, 0, 0]), [0, 0, 1, 0])
    g.add_reaction(rb.Rate.lma(0.001, [0, 0, 2, 0]), [0, 0, -2, 1])
    g.add_reaction(rb.Rate.lma(0.1, [0, 1, 0, 0]), [0, -1, 0, 0])
    g.add_reaction(rb.Rate.lma(1.0, [0, 0, 1, 0]), [0, 0, -1, 0])
    assert g.get_time() == 0.0 and g.get_species(3) == 0
    net = O.dimer_net()
    sp, t, st = [1, 0, 0, 0], 0.0, O.seed_state(777)
    for tm in (0.1, 0.25, 0.25, 0.7, 1.0):
        g.advance_until(tm)
        sp, t, st, _, _, _ = net.advance_until(sp, t, st, tm)
        assert g.get_time() == t == tm
        assert [g.get_species(s) for s in range(4)] == sp.tolist()
    # set_species / set_time then continue
    g.set_species([1, 5, 5, 5])
    g.set_time(2.0)
    g.advance_until(2.5)
    sp, t, st, _, _, _ = net.advance_until([1, 5, 5, 5], 2.0, st, 2.5)
    assert [g.get_species(s) for s in range(4)] == sp.tolist()
    with pytest.raises(ValueError):
        g.get_species(4)


def test_advance_one_reaction_and_every_event_mode(rb, O):
    net = _sir(rb)
    for seed in (3, 11, 2024):
        times, out = net.run_all_events([999, 1, 0], seed, 250.0)
        rt, ro = O.sir_net().run_all_events([999, 1, 0], seed, 250.0)
        np.testing.assert_array_equal(times, rt)
        np.testing.assert_array_equal(out, ro)
    # absorbing state: the last record has t = +inf (tests/test_rebop.py:47-48)
    dead = rb.Network(1)
    dead.add_reaction(rb.Rate.lma(1.0, [1]), [-1])
    times, out = dead.run_all_events([3], 5, 1e9)
    assert np.isinf(times[-1]) and out[-1, 0] == 0 and len(times) == 5
    rt, ro = O.sir_net().run_all_events([999, 1, 0], 3, 250.0)
    g = rb.api.Gillespie.new_with_seed([999, 1, 0], False, 3)
    g.add_reaction(rb.Rate.lma(1e-4, [1, 1, 0]), [-1, 1, 0])
    g.add_reaction(rb.Rate.lma(0.01, [0, 1, 0]), [0, -1, 1])
    for k in range(1, 6):
        g.advance_one_reaction()
        assert g.get_time() == rt[k]
        assert [g.get_species(s) for s in range(3)] == ro[k].tolist()


def test_dropin_every_event_and_var_names(rb, O):
    sir = rb.Gillespie()
    sir.add_reaction(1e-4, ["S", "I"], ["I", "I"])
    sir.add_reaction(0.01, ["I"], ["R"])
    ds = sir.run({"S": 999, "I": 1}, tmax=250, nb_steps=0, rng=4)
    rt, ro = O.sir_net().run_all_events([999, 1, 0], O.numpy_seed(4), 250.0)
    np.testing.assert_array_equal(np.asarray(ds.time), rt)
    np.testing.assert_array_equal(np.asarray(ds.R), ro[:, 2])
    full = sir.run({"S": 999, "I": 1}, tmax=250, nb_steps=250, rng=0)
    sub = sir.run({"S": 999, "I": 1}, tmax=250, nb_steps=250, rng=0, var_names=["S", "I"])
    assert "R" not in sub and "S" in sub
    np.testing.assert_array_equal(np.asarray(full.S), np.asarray(sub.S))
    ens = sir.run_ensemble({"S": 999, "I": 1}, 250, 250, 64, rng=0)
    np.testing.assert_array_equal(np.asarray(ens.S)[0], np.asarray(full.S))


def test_edge_cases(rb, O):
    # no reactions: counts constant; the clock jumps to each sample time
    empty = rb.Network(2)
    res = empty.run_ensemble([3, 4], _seeds(33), 10.0, 10)
    assert np.all(res.counts[:, 0] == 3) and np.all(res.counts[:, 1] == 4) and res.total_events == 0
    # no species at all (tests/test_rebop.py:148-152)
    none = rb.Gillespie()
    ds = none.run({}, tmax=10, nb_steps=10)
    assert len(ds) == 0
    np.testing.assert_array_equal(np.asarray(ds.time), np.linspace(0, 10, 11))
    # NaN and negative rates: !(0 < total) absorbs, as the reference does
    nan = rb.Network(1)
    nan.add_reaction(rb.Rate.lma(math.nan, [1]), [-1])
    assert np.all(nan.run_ensemble([5], _seeds(3), 1.0, 4).counts == 5)
    neg = rb.Network(1)
    neg.add_reaction(rb.Rate.lma(-1.0, [1]), [-1])
    assert np.all(neg.run_ensemble([5], _seeds(3), 1.0, 4).counts == 5)
    # zero trajectories
    z = _sir(rb).run_ensemble([999, 1, 0], np.zeros(0, np.uint64), 1.0, 3)
    assert z.counts.shape == (4, 3, 0)
    # trajectory counts that are not a multiple of the block size, large counts
    big = rb.Network(2)
    big.add_reaction(rb.Rate.lma(1e-18, [2, 0]), [-2, 1])
    big.add_reaction(rb.Rate.lma(1e3, [0, 0]), [1, 0])
    ob = O.OracleNet(2).add_lma(1e-18, [2, 0], [-2, 1]).add_lma(1e3, [0, 0], [1, 0])
    seeds = _seeds(129, 9)
    res = big.run_ensemble([3_000_000_000, 0], seeds, 0.5, 5)
    ref, ev, _, _ = ob.run_ensemble([3_000_000_000, 0], seeds, 0.5, 5)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    # more sample rows than the kernels count for streaming (65 536): every
    # row is copied after the launch, and every one is the oracle's
    seeds = _seeds(48, 10)
    res = _sir(rb).run_ensemble([999, 1, 0], seeds, 250.0, 70_000)
    ref, ev, _, _ = O.sir_net().run_ensemble([999, 1, 0], seeds, 250.0, 70_000)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)


def test_device_entry_point_matches_host_entry_point(rb, O):
    torch = pytest.importorskip("torch")
    net = _dimer(rb)
    n = 777
    seeds = _seeds(n, 6)
    d_seeds = torch.from_numpy(seeds.view(np.int64)).cuda()
    d_x0 = torch.tensor([1, 0, 0, 0], dtype=torch.int64, device="cuda")
    d_out = torch.empty((11, 4, n), dtype=torch.int64, device="cuda")
    d_ev = torch.empty(n, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    net.run_ensemble_device(n, d_x0.data_ptr(), False, d_seeds.data_ptr(), 0.5, 10, d_out.data_ptr(),
                            events_ptr=d_ev.data_ptr(), stream=stream)
    total = net.last_events()
    torch.cuda.synchronize()
    ref, ev, tot, _ = O.dimer_net().run_ensemble([1, 0, 0, 0], seeds, 0.5, 10)
    np.testing.assert_array_equal(d_out.cpu().numpy(), ref)
    np.testing.assert_array_equal(d_ev.cpu().numpy().view(np.uint64), ev)
    assert total == tot


def test_page_locked_results_written_in_place(rb, O):
    # Page-locked result buffers written by the kernel directly (no staging
    # copy): the results and the byte counts match the staged path.
    torch = pytest.importorskip("torch")
    net = _dimer(rb)
    n = 1234
    seeds = _seeds(n, 8)
    pin_out = torch.empty((21, 4, n), dtype=torch.int64, pin_memory=True).numpy()
    pin_ev = torch.empty(n, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    pin_out[...] = -7
    res = _with_env("RB_ZERO_COPY", "1",
                    lambda: net.run_ensemble([1, 0, 0, 0], seeds, 0.5, 20, out=pin_out, events=pin_ev))
    ref, ev, tot, _ = O.dimer_net().run_ensemble([1, 0, 0, 0], seeds, 0.5, 20)
    np.testing.assert_array_equal(pin_out, ref)
    np.testing.assert_array_equal(pin_ev, ev)
    assert res.total_events == tot
    staged = _with_env("RB_ZERO_COPY", "0", lambda: net.run_ensemble([1, 0, 0, 0], seeds, 0.5, 20))
    np.testing.assert_array_equal(staged.counts, ref)
    assert res.stats["d2h_bytes"] == staged.stats["d2h_bytes"]


def _with_kernel(kind, fn):
    import os

    old = os.environ.get("RB_SSA_KERNEL")
    os.environ["RB_SSA_KERNEL"] = kind
    try:
        return fn()
    finally:
        if old is None:
            del os.environ["RB_SSA_KERNEL"]
        else:
            os.environ["RB_SSA_KERNEL"] = old


def test_fast_and_generic_kernels_match_oracle(rb, O):
    # The lockstep integer-binary64 kernel and the generic kernel against the oracle.
    cases = []
    cases.append((_dimer(rb), O.dimer_net(), [1, 0, 0, 0], 0.5, 25, None))
    cases.append((_sir(rb), O.sir_net(), [999, 1, 0], 250.0, 50, None))
    n = 300
    rng = np.random.default_rng(11)
    rates = np.stack([10 ** rng.uniform(-5, -3, n), 10 ** rng.uniform(-3, -1, n)], axis=1)
    cases.append((_sir(rb), O.sir_net(), [999, 1, 0], 100.0, 20, rates))
    for net, onet, x0, tmax, nb, r in cases:
        seeds = _seeds(n, 21)
        spec = _with_kernel("spec", lambda: net.run_ensemble(x0, seeds, tmax, nb, rates=r))
        fast = _with_kernel("fast", lambda: net.run_ensemble(x0, seeds, tmax, nb, rates=r))
        gen = _with_kernel("generic", lambda: net.run_ensemble(x0, seeds, tmax, nb, rates=r))
        ref, ev, _, _ = onet.run_ensemble(x0, seeds, tmax, nb, rates=r)
        assert spec.stats["mapping"] == 3 and fast.stats["mapping"] == 2 and gen.stats["mapping"] == 0
        np.testing.assert_array_equal(spec.counts, ref)
        np.testing.assert_array_equal(fast.counts, ref)
        np.testing.assert_array_equal(gen.counts, ref)
        np.testing.assert_array_equal(spec.events, ev)
        np.testing.assert_array_equal(fast.events, ev)


def test_spec_kernel_stress_against_oracle(rb, O):
    # Speculative float-pair kernel: bit-exact counts and event numbers over
    # many trajectories, including long sample intervals (the clock's error
    # bound grows with the events of an interval) and order-2 reactions.
    seeds = _seeds(4000, 41)
    res = _with_kernel("spec", lambda: _dimer(rb).run_ensemble([1, 0, 0, 0], seeds, 1.0, 25))
    ref, ev, _, _ = O.dimer_net().run_ensemble([1, 0, 0, 0], seeds, 1.0, 25)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    assert res.stats["exact_reruns"] < 4000 * 26 // 100
    # dimers2 (benchmarks/benches/my_benchmark.rs:74-105): 2A <-> A_A -> AA with 1e5 A
    net = rb.Network(3)
    for k, e, d in [(1.0, [1, 0, 0], [-1, 0, 0]), (1 / 500, [2, 0, 0], [-2, 1, 0]),
                    (0.5, [0, 1, 0], [2, -1, 0]), (1 / 25, [0, 1, 0], [0, -1, 1])]:
        net.add_reaction(rb.Rate.lma(k, e), d)
    onet = O.OracleNet(3)
    for k, e, d in [(1.0, [1, 0, 0], [-1, 0, 0]), (1 / 500, [2, 0, 0], [-2, 1, 0]),
                    (0.5, [0, 1, 0], [2, -1, 0]), (1 / 25, [0, 1, 0], [0, -1, 1])]:
        onet.add_lma(k, e, d)
    seeds = _seeds(256, 42)
    res = _with_kernel("spec", lambda: net.run_ensemble([5000, 0, 0], seeds, 2.0, 4))
    ref, ev, _, _ = onet.run_ensemble([5000, 0, 0], seeds, 2.0, 4)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)


def test_fast_kernel_native_fallback_paths(rb, O):
    # Steps outside the integer emulation's domain are redone in native binary64.
    seeds = _seeds(200, 31)
    # NaN / negative rate constants for some trajectories (per-trajectory rates)
    rates = np.tile([1e-4, 0.01], (200, 1))
    rates[::7, 1] = np.nan
    rates[::11, 0] = -1e-4
    net, onet = _sir(rb), O.sir_net()
    fast = _with_kernel("fast", lambda: net.run_ensemble([999, 1, 0], seeds, 100.0, 10, rates=rates))
    ref, ev, _, _ = onet.run_ensemble([999, 1, 0], seeds, 100.0, 10, rates=rates)
    np.testing.assert_array_equal(fast.counts, ref)
    np.testing.assert_array_equal(fast.events, ev)
    # counts that go negative: A is consumed at a rate set by B, and A is a reactant too
    net = rb.Network(2)
    net.add_reaction(rb.Rate.lma(1.0, [0, 1]), [-1, 0])
    net.add_reaction(rb.Rate.lma(0.5, [1, 0]), [0, 1])
    onet = O.OracleNet(2).add_lma(1.0, [0, 1], [-1, 0]).add_lma(0.5, [1, 0], [0, 1])
    fast = _with_kernel("fast", lambda: net.run_ensemble([3, 5], seeds, 3.0, 6))
    ref, ev, _, _ = onet.run_ensemble([3, 5], seeds, 3.0, 6)
    np.testing.assert_array_equal(fast.counts, ref)
    np.testing.assert_array_equal(fast.events, ev)
    # counts at and beyond 2^53 (the reference's `as f64` rounds them)
    net = rb.Network(2)
    net.add_reaction(rb.Rate.lma(1e-16, [1, 0]), [-1, 1])
    onet = O.OracleNet(2).add_lma(1e-16, [1, 0], [-1, 1])
    x0 = [2 ** 53 + 7, 0]
    fast = _with_kernel("fast", lambda: net.run_ensemble(x0, seeds[:50], 0.02, 4))
    ref, ev, _, _ = onet.run_ensemble(x0, seeds[:50], 0.02, 4)
    np.testing.assert_array_equal(fast.counts, ref)
    np.testing.assert_array_equal(fast.events, ev)
    # macro arithmetic through the fast kernel
    D = rb.define_system(DIMER_DSL)
    d = D.with_parameters(25.0, 1000.0, 0.001, 0.1, 1.0)
    d.gene = 1
    res = _with_kernel("fast", lambda: d.run_ensemble(seeds, 0.3, 5))
    o = (O.OracleNet(4, macro=True).add_macro(25.0, [(0, 1)], [0, 1, 0, 0])
         .add_macro(1000.0, [(1, 1)], [0, 0, 1, 0]).add_macro(0.001, [(2, 2)], [0, 0, -2, 1])
         .add_macro(0.1, [(1, 1)], [0, -1, 0, 0]).add_macro(1.0, [(2, 1)], [0, 0, -1, 0]))
    ref, ev, _, _ = o.run_ensemble([1, 0, 0, 0], seeds, 0.3, 5)
    np.testing.assert_array_equal(res.counts, ref)


def _with_env(name, value, fn):
    import os

    old = os.environ.get(name)
    os.environ[name] = value
    try:
        return fn()
    finally:
        if old is None:
            del os.environ[name]
        else:
            os.environ[name] = old


def test_generated_network_kernel_matches_oracle(rb, O):
    # Networks compiled at run time (counts in registers, reactions unrolled)
    # against the oracle, bit for bit, and against the descriptor kernel.
    seeds = _seeds(3000, 51)
    jit = _with_env("RB_JIT", "1", lambda: _dimer(rb).run_ensemble([1, 0, 0, 0], seeds, 1.0, 20))
    ref, ev, _, _ = O.dimer_net().run_ensemble([1, 0, 0, 0], seeds, 1.0, 20)
    assert jit.stats["mapping"] == 4
    np.testing.assert_array_equal(jit.counts, ref)
    np.testing.assert_array_equal(jit.events, ev)
    # per-trajectory rates, with some outside the float-pair range (exact re-runs)
    n = 500
    rng = np.random.default_rng(5)
    rates = np.stack([10 ** rng.uniform(-5, -3, n), 10 ** rng.uniform(-3, -1, n)], axis=1)
    rates[::50, 0] = 1e-30
    rates[::77, 1] = np.nan
    jit = _with_env("RB_JIT", "1", lambda: _sir(rb).run_ensemble([999, 1, 0], seeds[:n], 200.0, 40, rates=rates))
    ref, ev, _, _ = O.sir_net().run_ensemble([999, 1, 0], seeds[:n], 200.0, 40, rates=rates)
    assert jit.stats["mapping"] == 4
    np.testing.assert_array_equal(jit.counts, ref)
    np.testing.assert_array_equal(jit.events, ev)
    # counts that go negative (A consumed at a rate set by B)
    net = rb.Network(2)
    net.add_reaction(rb.Rate.lma(1.0, [0, 1]), [-1, 0])
    net.add_reaction(rb.Rate.lma(0.5, [1, 0]), [0, 1])
    onet = O.OracleNet(2).add_lma(1.0, [0, 1], [-1, 0]).add_lma(0.5, [1, 0], [0, 1])
    jit = _with_env("RB_JIT", "1", lambda: net.run_ensemble([3, 5], seeds[:400], 3.0, 6))
    ref, ev, _, _ = onet.run_ensemble([3, 5], seeds[:400], 3.0, 6)
    np.testing.assert_array_equal(jit.counts, ref)
    np.testing.assert_array_equal(jit.events, ev)
    # macro arithmetic
    D = rb.define_system(DIMER_DSL)
    d = D.with_parameters(25.0, 1000.0, 0.001, 0.1, 1.0)
    d.gene = 1
    res = _with_env("RB_JIT", "1", lambda: d.run_ensemble(seeds[:600], 0.5, 10))
    o = (O.OracleNet(4, macro=True).add_macro(25.0, [(0, 1)], [0, 1, 0, 0])
         .add_macro(1000.0, [(1, 1)], [0, 0, 1, 0]).add_macro(0.001, [(2, 2)], [0, 0, -2, 1])
         .add_macro(0.1, [(1, 1)], [0, -1, 0, 0]).add_macro(1.0, [(2, 1)], [0, 0, -1, 0]))
    ref, ev, _, _ = o.run_ensemble([1, 0, 0, 0], seeds[:600], 0.5, 10)
    np.testing.assert_array_equal(res.counts, ref)


def _random_net(rb, O, seed, S, R, x0_mean):
    import bench

    reactions, x0 = bench.random_network(seed, S, R, x0_mean=x0_mean)
    net = rb.Network(S)
    onet = O.OracleNet(S)
    for k, e, d in reactions:
        net.add_reaction(rb.Rate.lma(k, e), d)
        onet.add_lma_sparse(k, [(i, x) for i, x in enumerate(e) if x], d)
    return net, onet, x0


def test_warp_kernel_dependency_updates_match_full_passes(rb, O):
    # After a reaction fires the warp kernel re-evaluates only the propensities
    # that read a species it changed; results equal full re-evaluation and the
    # oracle, over networks whose lists are short (64 x 400) and long (a
    # species read by every reaction makes some lists cover the network).
    for seed, S, R, tmax in ((71, 64, 400, 2e-2), (72, 30, 300, 1e-2)):
        net, onet, x0 = _random_net(rb, O, seed, S, R, 80.0)
        if seed == 72:  # species 0 becomes a catalyst of every reaction
            net = rb.Network(S + 1)
            onet = O.OracleNet(S + 1)
            import bench

            reactions, x0 = bench.random_network(seed, S, R, x0_mean=80.0)
            for k, e, d in reactions:
                net.add_reaction(rb.Rate.lma(k, list(e) + [1]), list(d) + [0])
                onet.add_lma_sparse(k, [(i, x) for i, x in enumerate(list(e) + [1]) if x], list(d) + [0])
            net.add_reaction(rb.Rate.lma(5.0, [0] * S + [0]), [0] * S + [1])
            onet.add_lma_sparse(5.0, [], [0] * S + [1])
            x0 = list(x0) + [3]
        seeds = _seeds(96, seed)
        res = _with_kernel("warp", lambda: net.run_ensemble(x0, seeds, tmax, 10))
        full = _with_env("RB_WARP_DEPS", "0", lambda: _with_kernel("warp", lambda: net.run_ensemble(x0, seeds, tmax, 10)))
        ref, ev, _, _ = onet.run_ensemble(x0, seeds, tmax, 10)
        assert res.stats["mapping"] == 5 and ev.min() > 100
        np.testing.assert_array_equal(res.counts, ref)
        np.testing.assert_array_equal(res.events, ev)
        np.testing.assert_array_equal(full.counts, ref)


def test_warp_kernel_exact_choice_path(rb, O):
    # Every choice taken by the exact lane-by-lane fold (the path of a close
    # float-pair comparison), with dependency updates resuming after it, in
    # both arithmetics.
    net, onet, x0 = _random_net(rb, O, 73, 48, 200, 60.0)
    seeds = _seeds(64, 73)
    res = _with_env("RB_WARP_EXACT_CHOICE", "1",
                    lambda: _with_kernel("warp", lambda: net.run_ensemble(x0, seeds, 5e-3, 5)))
    ref, ev, _, _ = onet.run_ensemble(x0, seeds, 5e-3, 5)
    assert res.stats["mapping"] == 5 and ev.min() > 50
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    D = rb.define_system(DIMER_DSL)
    d = D.with_parameters(25.0, 1000.0, 0.001, 0.1, 1.0)
    d.gene = 1
    res = _with_env("RB_WARP_EXACT_CHOICE", "1",
                    lambda: _with_kernel("warp", lambda: d.run_ensemble(seeds, 0.2, 4)))
    o = (O.OracleNet(4, macro=True).add_macro(25.0, [(0, 1)], [0, 1, 0, 0])
         .add_macro(1000.0, [(1, 1)], [0, 0, 1, 0]).add_macro(0.001, [(2, 2)], [0, 0, -2, 1])
         .add_macro(0.1, [(1, 1)], [0, -1, 0, 0]).add_macro(1.0, [(2, 1)], [0, 0, -1, 0]))
    ref, ev, _, _ = o.run_ensemble([1, 0, 0, 0], seeds, 0.2, 4)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)


def test_warp_kernel_wide_jump_deltas(rb, O):
    # A jump delta beyond 16 bits (a burst of 40 000 molecules) in a network the
    # warp kernel runs: its block tables keep 16-bit deltas and read wider ones
    # from the descriptor.
    import bench

    reactions, x0 = bench.random_network(74, 12, 40, x0_mean=50.0)
    net, onet = rb.Network(12), O.OracleNet(12)
    for k, e, d in reactions:
        net.add_reaction(rb.Rate.lma(k, e), d)
        onet.add_lma_sparse(k, [(i, x) for i, x in enumerate(e) if x], d)
    burst = [0] * 12
    burst[3] = 40_000
    net.add_reaction(rb.Rate.lma(20.0, [0] * 12), burst)
    onet.add_lma_sparse(20.0, [], burst)
    seeds = _seeds(64, 74)
    res = net.run_ensemble(x0, seeds, 1e-2, 8)
    ref, ev, _, _ = onet.run_ensemble(x0, seeds, 1e-2, 8)
    assert res.stats["mapping"] == 5
    assert ref[:, 3].max() >= 40_000  # some trajectories took the burst
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)


def test_warp_kernel_matches_oracle(rb, O):
    # Warp per trajectory: a random network beyond the thread kernels (chosen
    # by the dispatcher), then small networks forced onto it.
    net, onet, x0 = _random_net(rb, O, 7, 40, 120, 60.0)
    seeds = _seeds(64, 61)
    res = net.run_ensemble(x0, seeds, 2e-2, 12)
    ref, ev, tot, _ = onet.run_ensemble(x0, seeds, 2e-2, 12)
    assert res.stats["mapping"] == 5
    assert ev.min() > 200
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    assert res.total_events == tot
    seeds = _seeds(300, 62)
    res = _with_kernel("warp", lambda: _dimer(rb).run_ensemble([1, 0, 0, 0], seeds, 0.3, 6))
    ref, ev, _, _ = O.dimer_net().run_ensemble([1, 0, 0, 0], seeds, 0.3, 6)
    assert res.stats["mapping"] == 5
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    # per-trajectory rates, some outside the float-pair range (exact intervals)
    rng = np.random.default_rng(12)
    rates = np.stack([10 ** rng.uniform(-5, -3, 300), 10 ** rng.uniform(-3, -1, 300)], axis=1)
    rates[::40, 0] = 1e-25
    rates[::55, 1] = np.nan
    res = _with_kernel("warp", lambda: _sir(rb).run_ensemble([999, 1, 0], seeds, 150.0, 15, rates=rates))
    ref, ev, _, _ = O.sir_net().run_ensemble([999, 1, 0], seeds, 150.0, 15, rates=rates)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    # counts that go negative
    n2 = rb.Network(2)
    n2.add_reaction(rb.Rate.lma(1.0, [0, 1]), [-1, 0])
    n2.add_reaction(rb.Rate.lma(0.5, [1, 0]), [0, 1])
    o2 = O.OracleNet(2).add_lma(1.0, [0, 1], [-1, 0]).add_lma(0.5, [1, 0], [0, 1])
    res = _with_kernel("warp", lambda: n2.run_ensemble([3, 5], seeds[:100], 3.0, 6))
    ref, ev, _, _ = o2.run_ensemble([3, 5], seeds[:100], 3.0, 6)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    # macro arithmetic
    D = rb.define_system(DIMER_DSL)
    d = D.with_parameters(25.0, 1000.0, 0.001, 0.1, 1.0)
    d.gene = 1
    res = _with_kernel("warp", lambda: d.run_ensemble(seeds[:200], 0.3, 5))
    o = (O.OracleNet(4, macro=True).add_macro(25.0, [(0, 1)], [0, 1, 0, 0])
         .add_macro(1000.0, [(1, 1)], [0, 0, 1, 0]).add_macro(0.001, [(2, 2)], [0, 0, -2, 1])
         .add_macro(0.1, [(1, 1)], [0, -1, 0, 0]).add_macro(1.0, [(2, 1)], [0, 0, -1, 0]))
    ref, ev, _, _ = o.run_ensemble([1, 0, 0, 0], seeds[:200], 0.3, 5)
    np.testing.assert_array_equal(res.counts, ref)
