"""How far the Exp1 ziggurat is pinned to the reference's bits.

The reference draws Exp1 from rand_distr 0.6.0 (Cargo.lock:596), whose ZIGNOR
tables are committed constants of that crate, absent here.  The engine and the
oracle rebuild them from the published recurrence (Doornik 2005) in binary64
with the host libm.  This test rebuilds the same recurrence with correctly
rounded exp and log (mpmath at 160 bits, rounded to nearest), lists the table
entries where the libm-built double differs, and bounds the probability that a
draw's accept/reject decision depends on a bit that is not pinned:

  * a table entry that differs from the correctly rounded recurrence, and
  * the run-time exp(-x) of the wedge test (CUDA's exp on the GPU, glibc's in
    the oracle; both within 1 ulp of exp(-x), so at most 2 ulp apart) and the
    tail's ln U (it moves the draw by an ulp, which matters only when the clock
    lands within an ulp of a sample time).

The bound is per Exp1 draw (one per event, plus one discarded draw per sample
time); the figure is quoted beside the engine's parity claims.
"""

import math

import pytest

ZIG_R = 7.69711747013104972
ZIG_V = 0.0039496598225815571993


def _cr(mp, y):
    """Nearest binary64 to the mpf y."""
    d = float(y)
    for n in (math.nextafter(d, -math.inf), math.nextafter(d, math.inf)):
        if abs(mp.mpf(n) - y) < abs(mp.mpf(d) - y):
            d = n
    return d


def correctly_rounded_tables(mp):
    X = [0.0] * 257
    X[0] = ZIG_V / _cr(mp, mp.exp(mp.mpf(-ZIG_R)))
    X[1] = ZIG_R
    for i in range(2, 256):
        X[i] = -_cr(mp, mp.log(mp.mpf(ZIG_V / X[i - 1] + _cr(mp, mp.exp(mp.mpf(-X[i - 1]))))))
    X[256] = 0.0
    F = [_cr(mp, mp.exp(mp.mpf(-x))) for x in X]
    return X, F


def unpinned_decision_bound(X, F, table_diff_f):
    """Upper bound on P(an Exp1 draw's decision depends on an unpinned bit).

    Layer i (1..255) is picked with probability 1/256 and its fast test fails
    with probability 1 - X[i+1]/X[i]; the wedge test then compares
    L = F[i+1] + (F[i] - F[i+1]) U, spread evenly over [F[i], F[i+1]], with
    exp(-x).  L falls within w ulp of exp(-x) with probability at most
    (w + 1) ulp(F[i+1]) / (F[i+1] - F[i]).  w = 2 for the run-time exp; a table
    entry F[j] that may be off by one ulp moves L by at most one ulp in the two
    layers that read it."""
    p = 0.0
    for i in range(1, 256):
        p_layer = (1 / 256) * (1 - X[i + 1] / X[i])
        width = F[i + 1] - F[i]
        p += p_layer * 3 * math.ulp(F[i + 1]) / width
        if i in table_diff_f or i + 1 in table_diff_f:
            p += p_layer * 2 * math.ulp(F[i + 1]) / width
    # tail, R - ln U: an ulp of the draw matters only if the clock lands within
    # an ulp of the next sample time (below 2^-50 of the draws)
    p += (1 / 256) * (1 - X[1] / X[0]) * 2.0 ** -50
    return p


def test_ziggurat_tables_against_correctly_rounded_recurrence(O):
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 160
    X, F = correctly_rounded_tables(mp)
    x_lib, f_lib = O.zig_tables()
    diff_x = [i for i in range(257) if X[i] != x_lib[i]]
    diff_f = [i for i in range(257) if F[i] != f_lib[i]]
    # every abscissa is the correctly rounded recurrence's; of the 257
    # exp(-x) values glibc rounds one (f[87]) the other way
    assert diff_x == []
    assert set(diff_f) <= {87}
    for i in diff_f:
        assert abs(F[i] - f_lib[i]) <= math.ulp(F[i])
    p = unpinned_decision_bound(X, F, set(diff_f) | {87})
    assert p < 1e-15
    print(f"P(unpinned decision) per Exp1 draw <= {p:.2e}; table entries off by one ulp: f{diff_f}")


def test_engine_tables_equal_oracle_tables(O):
    # the engine and the oracle build the same tables
    rb = pytest.importorskip("rebop_gb300")
    x_e, f_e = rb.api.zig_tables()
    x_o, f_o = O.zig_tables()
    assert list(x_e) == list(x_o) and list(f_e) == list(f_o)
