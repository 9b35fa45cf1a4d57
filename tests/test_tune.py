"""The autotuner's candidate shapes, cache key and cache file (no GPU).

rb_ensemble_tune times pilot runs of the candidate kernels and launch shapes
on the GPU (tests/test_gpu_tune.py); which candidates it tries for a network
and ensemble, how it keys what it learned and how the cache file keeps it
are host logic, checked here.
"""

import ctypes as C

import pytest

GB300 = (152, 232448, b"NVIDIA GB300")


def _dimer(rb):
    n = rb.Network(4)
    for k, e, d in [(25.0, [1, 0, 0, 0], [0, 1, 0, 0]), (1000.0, [0, 1, 0, 0], [0, 0, 1, 0]),
                    (0.001, [0, 0, 2, 0], [0, 0, -2, 1]), (0.1, [0, 1, 0, 0], [0, -1, 0, 0]),
                    (1.0, [0, 0, 1, 0], [0, 0, -1, 0])]:
        n.add_reaction(rb.Rate.lma(k, e), d)
    return n


def _cands(lib, TuneResult, net, n_traj, stage, best=(4, 0, 0, -1), nb_steps=100, tmax=1.0, rpt=0):
    out = (TuneResult * 32)()
    n = C.c_int32()
    b = TuneResult(*best, 0.0)
    assert lib.rbg_internal_tune_candidates(net._h, GB300[0], GB300[1], n_traj, nb_steps, tmax, rpt, stage,
                                            C.byref(b), out, 32, C.byref(n)) == 0
    return [(out[k].mapping, out[k].block, out[k].phase_steps, out[k].sched) for k in range(n.value)]


@pytest.fixture(scope="module")
def tl():
    import rebop_gb300 as rb
    from rebop_gb300._lib import TuneResult, lib

    return rb, lib, TuneResult


def test_candidates_follow_the_network_and_ensemble(tl):
    import bench

    rb, lib, TR = tl
    dimer = _dimer(rb)
    # kernels: generated, descriptor speculative, lockstep exact (no warp kernel for 5 reactions)
    assert [c[0] for c in _cands(lib, TR, dimer, 100_000, 0)] == [4, 3, 2]
    # block sizes of the generated kernel for a full-size ensemble ...
    assert [c[1] for c in _cands(lib, TR, dimer, 100_000, 1)] == [256, 320, 416, 448, 512]
    # ... not for a small one, which is spread over 128-lane blocks
    assert _cands(lib, TR, dimer, 1_000, 1) == []
    # phase lengths and the other scheduler around the best shape
    assert _cands(lib, TR, dimer, 100_000, 2, best=(4, 416, 0, -1)) == [(4, 416, 64, -1), (4, 416, 256, -1),
                                                                        (4, 416, 0, 1)]
    assert _cands(lib, TR, dimer, 100_000, 1, best=(2, 0, 0, -1)) == []
    # 200 species x 1000 reactions: only a warp per trajectory covers it
    big = rb.Network(bench.LARGE["S"])
    for k, e, d in bench.LARGE["reactions"]:
        big.add_reaction(rb.Rate.lma(k, e), d)
    assert _cands(lib, TR, big, 10_000, 0) == [(5, 0, 0, -1)]
    # 64 reactions: the warp kernel, the lockstep kernel's 32-reaction limit passed
    mid = rb.Network(20)
    for k, e, d in bench.random_network(3, 20, 64)[0]:
        mid.add_reaction(rb.Rate.lma(k, e), d)
    assert [c[0] for c in _cands(lib, TR, mid, 10_000, 0)] == [5]
    # a rate expression: only the generic exact kernel
    from rebop_gb300 import expr as E

    ex = rb.Network(2)
    ex.add_reaction(rb.Rate.expression(E.parse("3 + A / 4").to_expr({"A": 0}, {})), [1, 0])
    assert _cands(lib, TR, ex, 1000, 0) == [(0, 0, 0, -1)]


def test_key_separates_network_shape_size_and_gpu(tl):
    rb, lib, _ = tl
    buf = C.create_string_buffer(512)

    def key(net, n, gpu=GB300[2], sm=GB300[0], rpt=0):
        assert lib.rbg_internal_tune_key(net._h, sm, gpu, n, rpt, buf, 512) == 0
        return buf.value.decode()

    d = _dimer(rb)
    k = key(d, 100_000)
    assert k == "S=4 R=5 M=2 O=2 macro=0 expr=0 log2n=16 rpt=0 sm=152 gpu=NVIDIA GB300"
    assert key(d, 70_000) == k                       # same power of two
    assert key(d, 200_000) != k                      # next power of two
    assert key(d, 100_000, rpt=1) != k
    assert key(d, 100_000, gpu=b"other", sm=132) != k
    assert key(_dimer(rb), 100_000) == k             # same shape, another network object


def test_cache_file_round_trip(tl, tmp_path, monkeypatch):
    rb, lib, TR = tl
    path = tmp_path / "tune.txt"
    monkeypatch.setenv("RB_TUNE_CACHE", str(path))
    lib.rb_tune_clear(1)
    buf = C.create_string_buffer(1024)
    assert lib.rb_tune_cache_path(buf, 1024) == len(str(path)) and buf.value.decode() == str(path)
    out = TR()
    assert lib.rbg_internal_tune_get(b"S=4 R=5 key", C.byref(out)) != 0
    assert lib.rbg_internal_tune_store(b"S=4 R=5 key", C.byref(TR(4, 416, 64, 0, 27.5))) == 0
    assert lib.rbg_internal_tune_store(b"S=3 R=2 other", C.byref(TR(2, 0, 0, -1, 1.5))) == 0
    assert path.exists() and len(path.read_text().splitlines()) == 2
    lib.rb_tune_clear(0)  # forget the memory copy: the next lookup reads the file
    assert lib.rbg_internal_tune_get(b"S=4 R=5 key", C.byref(out)) == 0
    assert (out.mapping, out.block, out.phase_steps, out.sched, out.ms) == (4, 416, 64, 0, 27.5)
    lib.rb_tune_clear(1)
    assert not path.exists()
    assert lib.rbg_internal_tune_get(b"S=4 R=5 key", C.byref(out)) != 0
