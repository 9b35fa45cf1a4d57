"""Rate::Expr (src/expr.rs) propensities: postfix programs, oracle, engine.

CPU tests pin the postfix compiler and the oracle's program evaluation to the
resolved-tree evaluation (itself pinned to the reference's golden values in
test_host.py); GPU tests run Expr networks on the engine against the oracle.
Operations +, -, *, /, max, min and negation are IEEE binary64 on both sides,
so trajectories are identical bit for bit; exp and powf come from CUDA's math
library on the device and the C library on the host, which may differ in the
last place.
"""

import math
import warnings

import numpy as np
import pytest


@pytest.fixture(scope="module")
def rb():
    import rebop_gb300

    return rebop_gb300


def _E():
    from rebop_gb300 import expr

    return expr


EXPRESSIONS = [
    "0.2 * B * C / (5 + C)",
    "k1 * A - B / 3 + 7",
    "max(A, B) - min(A, 2.5) * -C",
    "exp(-A / 50) * 3 + B ^ 2 / 100",
    "A ^ 0.5 + exp(B / (C + 1))",
    "(A + B) * (A - B) / (1 + C * C)",
    "max(min(A, 10), B / 2) ^ 2",
]
SPECIES = {"A": 0, "B": 1, "C": 2}
PARAMS = {"k1": 0.125}


def _postfix_eval(code, consts, sp):
    # a stack machine over the tree's own operation semantics
    E = _E()
    names = {2: "neg", 3: "add", 4: "sub", 5: "mul", 6: "div", 7: "pow", 8: "max", 9: "min", 10: "exp"}
    st = []
    for w in code:
        op, arg = w & 0xFF, w >> 8
        if op == 0:
            st.append(consts[arg])
        elif op == 1:
            st.append(float(sp[arg]))
        elif op in (2, 10):
            st.append(E.Expr(names[op], a=E.Expr("const", value=st.pop())).eval([]))
        else:
            y, x = st.pop(), st.pop()
            st.append(E.Expr(names[op], a=E.Expr("const", value=x), b=E.Expr("const", value=y)).eval([]))
    assert len(st) == 1
    return st[0]


def test_postfix_program_equals_tree():
    E = _E()
    rng = np.random.default_rng(3)
    for text in EXPRESSIONS:
        e = E.parse(text).to_expr(SPECIES, PARAMS)
        code, consts = e.to_program()
        for sp in rng.integers(0, 200, size=(50, 3)):
            assert _postfix_eval(code, consts, sp) == e.eval(sp)


def test_oracle_expr_equals_tree(O):
    E = _E()
    rng = np.random.default_rng(4)
    for text in EXPRESSIONS:
        e = E.parse(text).to_expr(SPECIES, PARAMS)
        code, consts = e.to_program()
        net = O.OracleNet(3).add_expr(code, consts, [0, 0, 0])
        assert net.validate()
        for sp in rng.integers(0, 200, size=(50, 3)):
            a, b = net.rate(0, sp), e.eval(sp)
            assert a == b or (math.isnan(a) and math.isnan(b))


def test_engine_rejects_malformed_programs(rb):
    net = rb.Network(2)
    for code, consts in [([5], []), ([0], []), ([1 | (2 << 8)], []), ([0, 0], [1.0]), ([11], []), ([], [])]:
        with pytest.raises(ValueError):
            net.add_reaction(rb.Rate.expression(_Prog(code, consts)), [1, 0])
    with pytest.raises(ValueError):  # one difference per species
        net.add_reaction(rb.Rate.expression(_Prog([0], [1.0])), [1])
    deep = [0] * 17 + [3] * 16
    with pytest.raises(ValueError):
        net.add_reaction(rb.Rate.expression(_Prog(deep, [1.0])), [1, 0])
    net.add_reaction(rb.Rate.expression(_Prog([0] * 16 + [3] * 15, [1.0])), [1, 0])
    assert net.nb_reactions == 1


class _Prog:
    def __init__(self, code, consts):
        self.code, self.consts = code, consts

    def to_program(self):
        return list(self.code), list(self.consts)


def test_dropin_expression_errors(rb):
    # tests/test_rebop.py:92-97
    s = rb.Gillespie()
    with pytest.raises(ValueError, match="Rate expression not understood"):
        s.add_reaction("+", [], ["A"])
    with pytest.raises(ValueError, match="Rate expression not understood"):
        s.add_reaction("1+", [], ["A"])
    s = rb.Gillespie()
    s.add_reaction("k * A", [], ["A"])
    with pytest.raises(ValueError, match="Parameter k should have a value"):
        s.run({"A": 1}, tmax=1, nb_steps=1)


# ---------------------------------------------------------------- GPU
def _mm(rb, O, E):
    """Michaelis-Menten with a rate expression for the product step, written
    both ways: mass action for binding, Expr for catalysis (examples/mm.py)."""
    sp = {"E": 0, "S": 1, "ES": 2, "P": 3}
    cat = E.parse("kcat * ES * S / (Km + S)").to_expr(sp, {"kcat": 0.3, "Km": 40.0})
    code, consts = cat.to_program()
    net = rb.Network(4)
    net.add_reaction(rb.Rate.lma(0.01, [1, 1, 0, 0]), [-1, -1, 1, 0])
    net.add_reaction(rb.Rate.lma(0.1, [0, 0, 1, 0]), [1, 1, -1, 0])
    net.add_reaction(rb.Rate.expression(cat), [1, 0, -1, 1])
    onet = (O.OracleNet(4).add_lma(0.01, [1, 1, 0, 0], [-1, -1, 1, 0]).add_lma(0.1, [0, 0, 1, 0], [1, 1, -1, 0])
            .add_expr(code, consts, [1, 0, -1, 1]))
    return net, onet


@pytest.mark.gpu
def test_expr_network_bit_exact(rb, O):
    E = _E()
    net, onet = _mm(rb, O, E)
    seeds = np.random.default_rng(9).integers(np.iinfo(np.uint64).max, size=600, dtype=np.uint64)
    res = net.run_ensemble([50, 500, 0, 0], seeds, 60.0, 30)
    ref, ev, tot, _ = onet.run_ensemble([50, 500, 0, 0], seeds, 60.0, 30)
    assert res.stats["mapping"] == 0
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
    assert res.total_events == tot
    # every-event mode through the events kernel
    times, out = net.run_all_events([50, 500, 0, 0], int(seeds[0]), 20.0)
    rt, ro = onet.run_all_events([50, 500, 0, 0], int(seeds[0]), 20.0)
    np.testing.assert_array_equal(times, rt)
    np.testing.assert_array_equal(out, ro)


@pytest.mark.gpu
def test_expr_with_exp_and_pow(rb, O):
    # exp and powf: device and host libraries may differ in the last place, so
    # a trajectory may part ways when a choice falls within that; nearly all agree.
    E = _E()
    sp = {"A": 0, "B": 1}
    e1 = E.parse("3 * exp(-A / 40) + B ^ 0.5").to_expr(sp, {})
    e2 = E.parse("0.05 * A * max(B, 1) ^ 0.25").to_expr(sp, {})
    net = rb.Network(2)
    onet = O.OracleNet(2)
    for e, d in [(e1, [1, 0]), (e2, [-1, 1])]:
        code, consts = e.to_program()
        net.add_reaction(rb.Rate.expression(e), d)
        onet.add_expr(code, consts, d)
    seeds = np.random.default_rng(10).integers(np.iinfo(np.uint64).max, size=400, dtype=np.uint64)
    res = net.run_ensemble([0, 0], seeds, 50.0, 25)
    ref, ev, _, _ = onet.run_ensemble([0, 0], seeds, 50.0, 25)
    same = np.all(res.counts == ref, axis=(0, 1))
    assert same.mean() >= 0.99
    assert abs(res.counts[-1].mean() - ref[-1].mean()) <= 0.05 * ref[-1].mean() + 1


@pytest.mark.gpu
def test_reference_arbitrary_rate_tests(rb):
    # tests/test_rebop.py:92-145 through the drop-in
    s = rb.Gillespie()
    s.add_reaction("B", [], ["A"])
    with pytest.warns(UserWarning, match="species are not involved in any reaction"):
        ds = s.run({"B": 1}, tmax=10, nb_steps=100)
    assert ds.A[-1] >= 1
    np.testing.assert_equal(np.asarray(ds.B.values), [1] * 101)
    s = rb.Gillespie()
    s.add_reaction("B", [], ["A"])
    s.add_reaction(1, [], ["B"])
    assert s.run({}, tmax=10, nb_steps=100).A[-1] >= 1
    # crossed
    s = rb.Gillespie()
    s.add_reaction("B", [], ["A"])
    s.add_reaction("A", [], ["B"])
    ds = s.run({}, tmax=10, nb_steps=10)
    np.testing.assert_equal(np.asarray(ds.A.values), [0] * 11)
    np.testing.assert_equal(np.asarray(ds.B.values), [0] * 11)
    np.testing.assert_allclose(np.asarray(ds.time), np.linspace(0, 10, 11))
    ds = s.run({"A": 1}, tmax=10, nb_steps=10)
    assert ds.A[-1] > 1 and ds.B[-1] > 0
    ds = s.run({"B": 1}, tmax=10, nb_steps=10)
    assert ds.A[-1] > 0 and ds.B[-1] > 1
    # arbitrary rates 2: conservation B + C + D
    s = rb.Gillespie()
    s.add_reaction(14, [], ["A"])
    s.add_reaction(0.1, ["A", "B"], ["C"], 0.01)
    s.add_reaction("0.2 * B * C / (5 + C)", ["B"], ["D"])
    ds = s.run({"B": 1000}, tmax=100, nb_steps=100)
    assert (np.asarray(ds.B) + np.asarray(ds.C) + np.asarray(ds.D) == 1000).all()
    assert ds.D[-1] >= 1


@pytest.mark.gpu
def test_expr_rust_api_and_ensemble_dropin(rb, O):
    E = _E()
    e = E.parse("2 + A / 10").to_expr({"A": 0}, {})
    code, consts = e.to_program()
    onet = O.OracleNet(1).add_expr(code, consts, [1])
    # Rust API: Gillespie::new_with_seed + add_reaction(Rate::expr) + advance_until
    g = rb.api.Gillespie.new_with_seed([0], False, 77)
    g.add_reaction(rb.Rate.expression(e), [1])
    g.advance_until(3.0)
    sp, t, _, _, _, _ = onet.advance_until([0], 0.0, O.seed_state(77), 3.0)
    assert g.get_species(0) == sp[0] and g.get_time() == t
    # ensembles, through the network API and the drop-in
    net = rb.Network(1)
    net.add_reaction(rb.Rate.expression(e), [1])
    seeds = np.random.default_rng(11).integers(np.iinfo(np.uint64).max, size=300, dtype=np.uint64)
    res = net.run_ensemble([0], seeds, 5.0, 5)
    ref, ev, _, _ = onet.run_ensemble([0], seeds, 5.0, 5)
    np.testing.assert_array_equal(res.counts, ref)
    s = rb.Gillespie()
    s.add_reaction("2 + A / 10", [], ["A"])
    ds = s.run_ensemble({}, tmax=5.0, nb_steps=5, n_trajectories=300, seeds=seeds)
    np.testing.assert_array_equal(np.asarray(ds.A), ref[:, 0, :].T)
