"""Host-side logic and the C ABI surface, on the CPU (no kernel runs here)."""

import ctypes
import re
import warnings
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def rb():
    import rebop_gb300

    return rebop_gb300


def _header_symbols():
    text = (ROOT / "include" / "rebop_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rb_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol(rb):
    from rebop_gb300 import build

    lib = ctypes.CDLL(str(build.LIB))
    syms = _header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_channel(rb):
    from rebop_gb300._lib import last_error, lib

    assert re.match(r"\d+\.\d+\.\d+", lib.rb_version().decode())
    h = ctypes.c_void_p()
    assert lib.rb_network_create(-1, ctypes.byref(h)) == 1
    assert "negative" in last_error()


def test_add_reaction_shape_asserts(rb):
    # src/gillespie.rs:227-237: exponent and difference vectors need S entries.
    n = rb.Network(3)
    with pytest.raises(ValueError, match="assertion failed"):
        n.add_reaction(rb.Rate.lma(1.0, [1, 0]), [0, 0, 0])
    with pytest.raises(ValueError, match="assertion failed"):
        n.add_reaction(rb.Rate.lma(1.0, [1, 0, 0]), [0, 0])
    n.add_reaction(rb.Rate.lma(1.0, [1, 0, 0]), [-1, 0, 1])
    assert n.nb_reactions == 1 and n.nb_species == 3


def test_issue85_out_of_range_sparse_index(rb):
    # src/gillespie.rs:496-502: the reference panics; the ABI returns RB_ERR_INVALID.
    g = rb.api.Gillespie.new_with_seed([1], True, 0)
    with pytest.raises(ValueError, match="assertion failed"):
        g.add_reaction(rb.Rate.lma_sparse(1.0, [(10, 1)]), [0])
    assert g.nb_reactions() == 0


def test_rate_and_jump_conversions(rb, goldens):
    # src/gillespie.rs:421-446 and :474-482
    Rate, Jump = rb.api.Rate, rb.api.Jump
    for case in goldens["rate_sparse"]:
        r = Rate.lma(case["rate"], case["dense"])
        assert r.sparse() == Rate.lma_sparse(case["rate"], [tuple(p) for p in case["sparse"]])
    r = Rate.lma(2.0, [3])
    assert r.dense() == r and r.sparse().dense() == r
    r = Rate.lma_sparse(2.0, [(0, 1), (3, 2)])
    assert r.dense() == Rate.lma(2.0, [1, 0, 0, 2]) and r.dense().sparse() == r
    dj, sj = Jump.new([-1, 0, 3, -2]), Jump.new_sparse([(0, -1), (2, 3), (3, -2)])
    assert dj.sparse() == sj and sj.dense() == dj and dj.dense() == dj and sj.sparse() == sj


VILAR = """
    αA αpA αR αpR βA βR δMA δMR δA δR γA γR γC θA θR;
    Vilar { Da, Dr, Dpa, Dpr, Ma, Mr, A, R, C }
    r_activation_a      : Da + A    => Dpa      @ γA
    r_activation_r      : Dr + A    => Dpr      @ γR
    r_deactivation_a    : Dpa       => Da + A   @ θA
    r_deactivation_r    : Dpr       => Dr + A   @ θR
    r_transcription_a   : Da        => Da + Ma  @ αA
    r_transcription_r   : Dr        => Dr + Mr  @ αR
    r_transcription_p_a : Dpa       => Dpa + Ma @ αpA
    r_transcription_p_r : Dpr       => Dpr + Mr @ αpR
    r_translation_a     : Ma        => Ma + A   @ βA
    r_translation_r     : Mr        => Mr + R   @ βR
    r_complexation      : A + R     => C        @ γC
    r_decomplexation    : C         => R        @ δA
    r_decay_mRNA_a      : Ma        =>          @ δMA
    r_decay_mRNA_r      : Mr        =>          @ δMR
    r_decay_prot_a      : A         =>          @ δA
    r_decay_prot_r      : R         =>          @ δR
"""


def test_dsl_lowering(rb):
    # benchmarks/benches/vilar/vilar.rs:6-25 (Greek identifiers included)
    net = rb.Network.from_dsl(VILAR)
    assert net.name == "Vilar" and net.nb_species == 9 and net.nb_reactions == 16
    assert net.params[0] == "αA" and net.species[-1] == "C"
    assert np.isnan(net.reaction_rate(0))  # parameters start as NaN
    net.set_param("γA", 1.0)
    assert net.reaction_rate(0) == 1.0
    n2 = rb.Network.from_dsl("k; X { A } r: 2 A => A @ k * 0.5 / 2")
    n2.set_param("k", 8.0)
    assert n2.reaction_rate(0) == 2.0
    for bad in ("k; X { A } r: B => A @ k", "k; X { A } r: 0 A => A @ k", "k; X { A } r: A => A @ q",
                "X { A }", "k; X { A } r: A => A @ A"):
        with pytest.raises(ValueError):
            rb.Network.from_dsl(bad)


def test_vilar_dsl_agrees_with_runtime_extract(rb, goldens):
    # The reference states the Vilar benchmark twice: define_system! in
    # benchmarks/benches/vilar/vilar.rs and the run-time API in vilar.py.  The
    # DSL lowering with the extracted parameter values must give the extracted
    # reactions, in the same order, with the same rates and net changes.
    vil = goldens["vilar"]
    greek = {"α": "alpha", "β": "beta", "γ": "gamma", "δ": "delta", "θ": "theta"}
    net = rb.Network.from_dsl(VILAR)
    for p in net.params:
        net.set_param(p, vil["params"]["".join(greek.get(c, c) for c in p)])
    assert net.nb_reactions == len(vil["reactions"]) == 16
    for i, r in enumerate(vil["reactions"]):
        assert net.reaction_rate(i) == r["rate"]
    assert vil["run"]["n_traj"] == 100 and vil["run"]["nb_steps"] == 200 and vil["run"]["tmax"] == 200.0
    assert vil["run"]["init"] == {"Da": 1, "Dr": 1}


def test_expr_parser_goldens(rb, goldens):
    from rebop_gb300 import expr

    for case in goldens["expr_eval"]:
        e = expr.parse(case["expr"]).to_expr(case["species_index"], {})
        assert e.eval(case["species"]) == case["expected"], case["where"]
    for bad in ("+", "1+", " 1", "1 ", "2e", "a^b^c", "max(1)", "(1"):
        with pytest.raises(expr.ParseError):
            expr.parse(bad)
    assert str(expr.parse("V * A / (Km + A)")) == "((V * A) / (Km + A))"
    assert str(expr.parse("1e-5*x")) == "(0.00001 * x)"
    assert expr.parse("maximum").op == "var" and expr.parse("inf").op == "var"


def test_dropin_python_errors_and_text(rb):
    # tests/test_rebop.py:92-97 and :155-159; pyo3_gillespie.rs:239-252
    s = rb.Gillespie()
    with pytest.raises(ValueError, match="Rate expression not understood"):
        s.add_reaction("+", [], ["A"])
    with pytest.raises(ValueError, match="Rate expression not understood"):
        s.add_reaction("1+", [], ["A"])
    s = rb.Gillespie()
    s.add_reaction(4, ["A"], ["B"])
    with pytest.raises(ValueError, match="Species B cannot also be a parameter"):
        s.run({}, 10, 10, params={"B": 4.2})
    s = rb.Gillespie()
    s.add_reaction(0.1, ["A", "B"], ["C"], 0.01)
    s.add_reaction(14, [], ["A"])
    assert s.nb_reactions() == 3 and s.nb_species() == 3
    assert str(s) == ("3 species and 3 reactions\nA + B --> C @ LMA(0.1)\nC --> A + B @ LMA(0.01)\n"
                      " --> A @ LMA(14)\n")


def test_dropin_set_init_warning_adds_species(rb):
    s = rb.Gillespie()
    s.add_reaction(1.0, [], ["A"])
    assert s.set_init({"B": 1}) is True
    assert s.nb_species() == 2


def test_partition_independence_of_seeds():
    # Trajectory j's stream depends only on its own seed, so any split of the
    # trajectory range across ranks reproduces the unsplit ensemble.
    from oracle import oracle as O

    net = O.sir_net()
    seeds = np.random.default_rng(0).integers(np.iinfo(np.uint64).max, size=40, dtype=np.uint64)
    full = net.run_ensemble([999, 1, 0], seeds, 50.0, 10)[0]
    parts = [net.run_ensemble([999, 1, 0], seeds[a:b], 50.0, 10)[0] for a, b in ((0, 13), (13, 27), (27, 40))]
    assert np.array_equal(np.concatenate(parts, axis=2), full)


def test_product_zig_tables_equal_oracle(rb, O):
    x, f = rb.api.zig_tables()
    ox, of = O.zig_tables()
    assert np.array_equal(x.view(np.uint64), ox.view(np.uint64))
    assert np.array_equal(f.view(np.uint64), of.view(np.uint64))


def test_no_oracle_import_in_product():
    for p in (ROOT / "rebop_gb300").rglob("*"):
        if p.suffix in (".py", ".cpp", ".cu", ".cuh", ".hpp", ".h"):
            text = p.read_text(encoding="utf-8")
            assert "oracle" not in text.lower() or p.name == "build.py", p


def _dimer_net(rb):
    net = rb.Network(4)
    for k, e, d in [(25.0, [1, 0, 0, 0], [0, 1, 0, 0]), (1000.0, [0, 1, 0, 0], [0, 0, 1, 0]),
                    (0.001, [0, 0, 2, 0], [0, 0, -2, 1]), (0.1, [0, 1, 0, 0], [0, -1, 0, 0]),
                    (1.0, [0, 0, 1, 0], [0, 0, -1, 0])]:
        net.add_reaction(rb.Rate.lma(k, e), d)
    return net


def test_generated_network_source(rb):
    # The generator unrolls every reaction (falling factorial in the written
    # order) and turns each jump into per-species selects.
    import ctypes as C
    import importlib

    L = importlib.import_module("rebop_gb300._lib").lib
    buf = C.create_string_buffer(1 << 17)
    net = _dimer_net(rb)
    assert L.rbg_internal_jit_source(net._h, buf, 1 << 17) == 0
    src = buf.value.decode()
    assert "kMaxR = 5" in src and "float n[4]" in src
    assert "fmaxf(__fadd_rn(c.n[2], -1.0f), 0.0f)" in src
    assert "c.n[2] += (idx == 1 ? 1.0f : 0.0f) + (idx == 2 ? -2.0f : 0.0f) + (idx == 4 ? -1.0f : 0.0f);" in src
    # the exact binary64 choice multiplies the reference's factors n-1, then n
    assert "acc = __dmul_rn(acc, (double)((long long)cn[2] - 1));\n    acc = __dmul_rn(acc, (double)((long long)cn[2] - 0));" in src
    big = rb.Network(40)
    big.add_reaction(rb.Rate.lma(1.0, [1] + [0] * 39), [-1] + [0] * 39)
    assert L.rbg_internal_jit_source(big._h, buf, 1 << 17) == 5  # RB_ERR_UNSUPPORTED


def test_generated_network_compiles(rb, tmp_path, monkeypatch):
    # NVRTC compiles the generated kernel for sm_103a without a GPU.
    import ctypes as C
    import importlib
    import shutil

    if shutil.which("nvcc") is None:
        pytest.skip("no CUDA toolkit")
    monkeypatch.setenv("RB_JIT_CACHE", str(tmp_path))
    L = importlib.import_module("rebop_gb300._lib").lib
    n = C.c_uint64()
    net = _dimer_net(rb)
    rc = L.rbg_internal_jit_compile(net._h, C.byref(n))
    assert rc == 0, importlib.import_module("rebop_gb300._lib").last_error()
    assert n.value > 10000
    assert len(list(tmp_path.glob("net_*.cubin"))) == 1


def test_batch_results_in_place_need_a_run(rb):
    # An item added without output arrays (copy=False) has no results to read
    # before the batch has run: the entry point says so instead of handing out
    # a pointer; its shape and the plan are known without a GPU.
    b = rb.Batch()
    n = rb.Network(2)
    n.add_reaction(rb.Rate.lma(1.0, [1, 0]), [-1, 1])
    k = b.add(n, [10, 0], np.arange(4, dtype=np.uint64), 1.0, 3, copy=False)
    assert b.plan() == (0, 1)
    with pytest.raises(ValueError, match="has not run"):
        b.counts(k)
    with pytest.raises(ValueError, match="out of range"):
        b._view(5)


def test_batch_plan_groups_by_structure(rb, monkeypatch):
    # The persistent plan: small networks (at most 16 species and reactions)
    # become thread units, larger ones a warp per trajectory, rate expressions
    # and define_system! networks of the other arithmetic launches of their
    # own.  The merged plan: parameter sets of one network merge into one
    # thread-per-trajectory launch.
    import bench

    from rebop_gb300 import expr as E

    b = rb.Batch()
    mm = rb.Network(4)  # E + S <-> ES -> E + P
    mm.add_reaction(rb.Rate.lma(0.01, [1, 1, 0, 0]), [-1, -1, 1, 0])
    mm.add_reaction(rb.Rate.lma(0.1, [0, 0, 1, 0]), [1, 1, -1, 0])
    mm.add_reaction(rb.Rate.lma(0.05, [0, 0, 1, 0]), [1, 0, -1, 1])
    seeds = np.arange(8, dtype=np.uint64)
    for k in range(3):
        assert b.add(mm, [50, 500, 0, 0], seeds, 10.0, 5, rates=[0.01 * (k + 1), 0.1, 0.05]) == k
    b.add(mm, [50, 500, 0, 0], seeds, 20.0, 5)
    reactions, x0 = bench.random_network(3, 20, 60)
    big = rb.Network(20)
    for k, e, d in reactions:
        big.add_reaction(rb.Rate.lma(k, e), d)
    b.add(big, x0, seeds, 0.01, 4)
    b.add(big, x0, seeds, 0.02, 4)
    ex = rb.Network(2)
    ex.add_reaction(rb.Rate.expression(E.parse("3 + A / 4").to_expr({"A": 0}, {})), [1, 0])
    b.add(ex, [0, 0], seeds, 1.0, 4)
    d = rb.Network.from_dsl("k; Bd { A } r: A => @ k")
    d.set_param("k", 1.0)
    b.add(d, [5], seeds, 1.0, 4)
    assert b.plan() == (2, 6)
    assert [b.mapping(k) for k in range(8)] == [7, 7, 7, 7, 5, 5, 0, 0]
    monkeypatch.setenv("RB_BATCH_MODE", "merged")
    # parameter sets merge by structure and horizon; classes below
    # RB_BATCH_MIN_THREAD trajectories join the warp batch
    b1 = rb.Batch()
    for k in range(3):
        b1.add(mm, [50, 500, 0, 0], seeds, 10.0, 5, rates=[0.01 * (k + 1), 0.1, 0.05])
    b1.add(mm, [50, 500, 0, 0], seeds, 20.0, 5)
    b1.add(big, x0, seeds, 0.01, 4)
    b1.add(big, x0, seeds, 0.02, 4)
    assert b1.plan() == (0, 6)
    assert [b1.mapping(k) for k in range(6)] == [5] * 6
    monkeypatch.setenv("RB_BATCH_MIN_THREAD", "1")
    b2 = rb.Batch()
    for k in range(3):
        b2.add(mm, [50, 500, 0, 0], seeds, 10.0, 5, rates=[0.01 * (k + 1), 0.1, 0.05])
    b2.add(mm, [50, 500, 0, 0], seeds, 20.0, 5)
    b2.add(big, x0, seeds, 0.01, 4)
    assert b2.plan() == (2, 1)
    assert [b2.mapping(k) for k in range(5)] == [4, 4, 4, 4, 5]
    with pytest.raises(ValueError):
        b.add(mm, [1, 2, 3], seeds, 1.0, 2)


def test_warp_dependency_table(rb):
    # Row j of the warp kernel's dependency table lists, at lane-major
    # positions, exactly the reactions whose propensity reads a species that
    # reaction j changes; more than 31 of them mark the row for a full pass.
    import bench
    from rebop_gb300._lib import lib as L

    for seed, S, R in ((3, 20, 90), (4, 200, 1000), (5, 6, 300)):
        reactions, _ = bench.random_network(seed, S, R)
        net = rb.Network(S)
        for k, e, d in reactions:
            net.add_reaction(rb.Rate.lma(k, e), d)
        tab = np.zeros(R * 32, dtype=np.uint16)
        assert L.rbg_internal_warp_dep_table(net._h, tab.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)),
                                             tab.size) == 0
        tab = tab.reshape(R, 32)
        C = (R + 31) // 32
        readers = [{r for r, (_, e, _) in enumerate(reactions) if e[s] > 0} for s in range(S)]
        for j, (_, _, d) in enumerate(reactions):
            deps = set().union(*[readers[s] for s in range(S) if d[s] != 0]) if any(d) else set()
            pos = {(r % C) * 32 + r // C for r in deps}
            if len(pos) > 31:
                assert tab[j, 0] == 0xFFFF
            else:
                assert tab[j, 0] == len(pos)
                assert set(tab[j, 1:1 + len(pos)].tolist()) == pos


def _build_cpp_mirror(tmp_path):
    import shutil
    import subprocess

    from rebop_gb300 import build

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "rust_api_mirror"
    lib = Path(build.LIB)
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(ROOT / "tests/cpp/rust_api_mirror.cpp"),
                    "-o", str(exe), "-L", str(lib.parent), "-l:" + lib.name, "-Wl,-rpath," + str(lib.parent)],
                   check=True)
    return exe


def test_cpp_mirror_of_the_rust_api(rb, tmp_path):
    # include/rebop_gb300.hpp: constructors, asserts as exceptions, accessors.
    import subprocess

    exe = _build_cpp_mirror(tmp_path)
    r = subprocess.run([str(exe), "cpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
