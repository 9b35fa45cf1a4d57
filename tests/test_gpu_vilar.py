"""The reference's Vilar oscillator benchmark on the GPU, bit for bit against the oracle.

The model and its run arguments come from the golden extract of
benchmarks/benches/vilar/vilar.py (run-time API) and, for the macro form,
the define_system! text of benchmarks/benches/vilar/vilar.rs.  A trajectory
to tmax = 200 is about 5.5e5 events, so this is the longest-running parity
case per trajectory.
"""

import os

import numpy as np
import pytest

from test_host import VILAR

pytestmark = pytest.mark.gpu

GREEK = {"α": "alpha", "β": "beta", "γ": "gamma", "δ": "delta", "θ": "theta"}


def _seeds(n, salt=0):
    return np.random.default_rng(4321 + salt).integers(np.iinfo(np.uint64).max, size=n, dtype=np.uint64)


def _runtime_model(rb, O, vil):
    g = rb.Gillespie()
    for r in vil["reactions"]:
        g.add_reaction(r["rate"], r["reactants"], r["products"])
    names = list(g._species)
    onet = O.OracleNet(len(names))
    for r in vil["reactions"]:
        e = [r["reactants"].count(s) for s in names]
        onet.add_lma(r["rate"], e, [r["products"].count(s) - x for s, x in zip(names, e)])
    return g, names, onet


def _with_env(name, value, fn):
    old = os.environ.get(name)
    os.environ[name] = value
    try:
        return fn()
    finally:
        if old is None:
            del os.environ[name]
        else:
            os.environ[name] = old


def test_vilar_runtime_api_bit_exact(goldens, O):
    import rebop_gb300 as rb

    vil = goldens["vilar"]
    run = vil["run"]
    g, names, onet = _runtime_model(rb, O, vil)
    assert names == ["Da", "A", "Dpa", "Dr", "Dpr", "Ma", "Mr", "R", "C"]
    n = 256
    seeds = _seeds(n)
    x0 = [run["init"].get(s, 0) for s in names]
    ref, ev, tot, _ = onet.run_ensemble(x0, seeds, run["tmax"], run["nb_steps"])
    assert tot > n * 100_000  # the oscillator's event count, ~5.5e5 per trajectory
    for jit in ("0", "1"):
        ds = _with_env("RB_JIT", jit, lambda: g.run_ensemble(run["init"], run["tmax"], run["nb_steps"], n,
                                                             seeds=seeds))
        np.testing.assert_array_equal(np.asarray(ds.time), np.arange(run["nb_steps"] + 1, dtype=float))
        for k, s in enumerate(names):
            np.testing.assert_array_equal(ds[s].values, ref[:, k, :].T, err_msg=f"species {s}, RB_JIT={jit}")


def test_vilar_macro_form_bit_exact(goldens, O):
    import rebop_gb300 as rb

    vil = goldens["vilar"]
    V = rb.define_system(VILAR)
    sp = list(V._species)
    values = []
    for p in V._params:
        key = "".join(GREEK.get(c, c) for c in p)
        values.append(vil["params"][key])
    v = V.with_parameters(*values)
    v.Da, v.Dr = 1, 1
    onet = O.OracleNet(len(sp), macro=True)
    for r in vil["reactions"]:
        facs = []
        for s in r["reactants"]:
            i = sp.index(s)
            if facs and facs[-1][0] == i:
                facs[-1] = (i, facs[-1][1] + 1)
            else:
                facs.append((i, 1))
        d = [r["products"].count(s) - r["reactants"].count(s) for s in sp]
        onet.add_macro(r["rate"], facs, d)
    x0 = [1 if s in ("Da", "Dr") else 0 for s in sp]
    seeds = _seeds(128, 1)
    res = v.run_ensemble(seeds, 200.0, 200)
    ref, ev, _, _ = onet.run_ensemble(x0, seeds, 200.0, 200)
    np.testing.assert_array_equal(res.counts, ref)
    np.testing.assert_array_equal(res.events, ev)
