"""ctypes front of the C oracle (ssa_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline / reference arm, never by the product package.

``OracleNet`` holds a reaction network exactly as the reference stores it
(rebop src/gillespie.rs:12-19, 95-100, 157-163): per reaction a rate constant,
either a dense LMA exponent vector (``Rate::lma``) or a sparse
(index, exponent) list kept in the caller's order (``Rate::lma_sparse``), and a
dense jump vector (``add_reaction``'s ``differences``).
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "libssa_oracle.so"


def compile_flags() -> list[str]:
    """gcc flags of the oracle: optimised for the host CPU it runs on (the
    CPU baseline is timed there), never contracting a*b+c or reassociating,
    so results stay the reference's binary64 results on any host."""
    import platform

    tune = "-mcpu=native" if platform.machine().lower() in ("aarch64", "arm64") else "-march=native"
    return ["-O3", tune, "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> Path:
    """Compile ssa_oracle.c into a shared library (gcc, compile_flags())."""
    src = HERE / "ssa_oracle.c"
    stamp = BUILD_DIR / "flags.txt"
    flags = compile_flags()
    if (LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= src.stat().st_mtime
            and stamp.exists() and stamp.read_text() == " ".join(flags)):
        return LIB_PATH
    BUILD_DIR.mkdir(exist_ok=True)
    tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["gcc", *flags, "-fPIC", "-shared", "-pthread", "-o", str(tmp), str(src), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    stamp.write_text(" ".join(flags))
    return LIB_PATH


class _Net(C.Structure):
    _fields_ = [
        ("n_species", C.c_int32),
        ("n_reactions", C.c_int32),
        ("rate", C.POINTER(C.c_double)),
        ("rate_kind", C.POINTER(C.c_int32)),
        ("lma", C.POINTER(C.c_uint32)),
        ("sp_off", C.POINTER(C.c_int32)),
        ("sp_idx", C.POINTER(C.c_uint32)),
        ("sp_exp", C.POINTER(C.c_uint32)),
        ("jump", C.POINTER(C.c_int64)),
        ("macro_mode", C.c_int32),
        ("mfac_off", C.POINTER(C.c_int32)),
        ("mfac_idx", C.POINTER(C.c_uint32)),
        ("mfac_ord", C.POINTER(C.c_uint32)),
        ("ex_off", C.POINTER(C.c_int32)),
        ("ex_code", C.POINTER(C.c_int32)),
        ("ex_const", C.POINTER(C.c_double)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        P = C.POINTER
        L.orc_validate.argtypes = [P(_Net)]
        L.orc_validate.restype = C.c_int
        L.orc_rate.argtypes = [P(_Net), C.c_int, P(C.c_int64)]
        L.orc_rate.restype = C.c_double
        L.orc_affect.argtypes = [P(_Net), C.c_int, P(C.c_int64)]
        L.orc_affect.restype = None
        L.orc_advance_until.argtypes = [P(_Net), P(C.c_int64), P(C.c_double), P(C.c_uint64), C.c_double,
                                        P(C.c_int32), P(C.c_double), C.c_int64, P(C.c_int64)]
        L.orc_advance_until.restype = C.c_int64
        L.orc_seed_state.argtypes = [C.c_uint64, P(C.c_uint64)]
        L.orc_seed_state.restype = None
        L.orc_draw_u64.argtypes = [C.c_uint64, P(C.c_uint64), C.c_int64]
        L.orc_draw_u64.restype = None
        L.orc_draw_exp1.argtypes = [C.c_uint64, P(C.c_double), C.c_int64]
        L.orc_draw_exp1.restype = None
        L.orc_zig_tables.argtypes = [P(C.c_double), P(C.c_double)]
        L.orc_zig_tables.restype = None
        L.orc_run_ensemble.argtypes = [P(_Net), P(C.c_double), C.c_int64, P(C.c_int64), C.c_int64,
                                       P(C.c_uint64), C.c_int64, C.c_double, C.c_int64, P(C.c_int32),
                                       C.c_int32, P(C.c_int64), P(C.c_int64), P(C.c_uint64), C.c_int32]
        L.orc_run_ensemble.restype = C.c_int64
        L.orc_run_all_events.argtypes = [P(_Net), P(C.c_int64), C.c_uint64, C.c_double, P(C.c_int32),
                                         C.c_int32, P(C.c_double), P(C.c_int64), C.c_int64]
        L.orc_run_all_events.restype = C.c_int64
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None, ct):
    if a is None:
        return C.POINTER(ct)()
    return a.ctypes.data_as(C.POINTER(ct))


class OracleNet:
    """A reaction network in the reference's own representation."""

    def __init__(self, n_species: int, macro: bool = False):
        self.S = int(n_species)
        self.macro = bool(macro)
        self.rates: list[float] = []
        self.kinds: list[int] = []
        self.dense: list[list[int]] = []
        self.sparse: list[list[tuple[int, int]]] = []
        self.jumps: list[list[int]] = []
        self.mfac: list[list[tuple[int, int]]] = []
        self.programs: list[tuple[list[int], list[float]]] = []

    # Gillespie::add_reaction(Rate::lma(rate, exps), differences)
    def add_lma(self, rate: float, exponents, differences) -> "OracleNet":
        assert len(exponents) == self.S and len(differences) == self.S
        self.rates.append(float(rate))
        self.kinds.append(0)
        self.dense.append([int(e) for e in exponents])
        self.sparse.append([])
        self.jumps.append([int(d) for d in differences])
        self.mfac.append([(s, int(e)) for s, e in enumerate(exponents) if e > 0])
        self.programs.append(([], []))
        return self

    # Gillespie::add_reaction(Rate::expr(expr), differences): the expression as
    # a postfix program (words op | arg << 8, see ssa_oracle.c) and its constants
    def add_expr(self, code, consts, differences) -> "OracleNet":
        assert len(differences) == self.S
        self.rates.append(0.0)
        self.kinds.append(2)
        self.dense.append([0] * self.S)
        self.sparse.append([])
        self.jumps.append([int(d) for d in differences])
        self.mfac.append([])
        self.programs.append(([int(c) for c in code], [float(c) for c in consts]))
        return self

    # Gillespie::add_reaction(Rate::lma_sparse(rate, pairs), differences)
    def add_lma_sparse(self, rate: float, pairs, differences) -> "OracleNet":
        assert len(differences) == self.S
        self.rates.append(float(rate))
        self.kinds.append(1)
        self.dense.append([0] * self.S)
        self.sparse.append([(int(i), int(e)) for i, e in pairs])
        self.jumps.append([int(d) for d in differences])
        self.mfac.append([(int(i), int(e)) for i, e in pairs])
        self.programs.append(([], []))
        return self

    # define_system! reaction: reactant factors (species, literal) in written order
    def add_macro(self, rate: float, factors, differences) -> "OracleNet":
        self.rates.append(float(rate))
        self.kinds.append(0)
        d = [0] * self.S
        for s, k in factors:
            d[s] += k
        self.dense.append(d)
        self.sparse.append([])
        self.jumps.append([int(x) for x in differences])
        self.mfac.append([(int(s), int(k)) for s, k in factors])
        self.programs.append(([], []))
        return self

    @property
    def R(self) -> int:
        return len(self.rates)

    def _pack(self, rates=None):
        S, R = self.S, self.R
        keep = {}
        keep["rate"] = np.ascontiguousarray(np.asarray(self.rates if rates is None else rates, dtype=np.float64).reshape(-1)) if R else np.zeros(1)
        keep["kind"] = np.asarray(self.kinds or [0], dtype=np.int32)
        keep["lma"] = np.asarray(self.dense, dtype=np.uint32).reshape(-1) if R and S else np.zeros(1, np.uint32)
        off = [0]
        idx, ex = [], []
        for lst in self.sparse:
            for i, e in lst:
                idx.append(i)
                ex.append(e)
            off.append(len(idx))
        keep["sp_off"] = np.asarray(off, dtype=np.int32)
        keep["sp_idx"] = np.asarray(idx or [0], dtype=np.uint32)
        keep["sp_exp"] = np.asarray(ex or [0], dtype=np.uint32)
        keep["jump"] = np.asarray(self.jumps, dtype=np.int64).reshape(-1) if R and S else np.zeros(1, np.int64)
        moff = [0]
        midx, mord = [], []
        for lst in self.mfac:
            for i, e in lst:
                midx.append(i)
                mord.append(e)
            moff.append(len(midx))
        keep["mfac_off"] = np.asarray(moff, dtype=np.int32)
        keep["mfac_idx"] = np.asarray(midx or [0], dtype=np.uint32)
        keep["mfac_ord"] = np.asarray(mord or [0], dtype=np.uint32)
        eoff, ecode, econst = [0], [], []
        for code, consts in self.programs:
            base = len(econst)
            for w in code:
                op, arg = w & 0xFF, w >> 8
                ecode.append(op | ((arg + base) << 8) if op == 0 else w)  # constants: global index
            econst.extend(consts)
            eoff.append(len(ecode))
        keep["ex_off"] = np.asarray(eoff, dtype=np.int32)
        keep["ex_code"] = np.asarray(ecode or [0], dtype=np.int32)
        keep["ex_const"] = np.asarray(econst or [0.0], dtype=np.float64)
        n = _Net(S, R, _ptr(keep["rate"], C.c_double), _ptr(keep["kind"], C.c_int32),
                 _ptr(keep["lma"], C.c_uint32), _ptr(keep["sp_off"], C.c_int32),
                 _ptr(keep["sp_idx"], C.c_uint32), _ptr(keep["sp_exp"], C.c_uint32),
                 _ptr(keep["jump"], C.c_int64), int(self.macro), _ptr(keep["mfac_off"], C.c_int32),
                 _ptr(keep["mfac_idx"], C.c_uint32), _ptr(keep["mfac_ord"], C.c_uint32),
                 _ptr(keep["ex_off"], C.c_int32), _ptr(keep["ex_code"], C.c_int32),
                 _ptr(keep["ex_const"], C.c_double))
        return n, keep

    def validate(self) -> bool:
        n, keep = self._pack()
        return lib().orc_validate(C.byref(n)) == 0

    def rate(self, r: int, species) -> float:
        n, keep = self._pack()
        sp = np.asarray(species, dtype=np.int64)
        return lib().orc_rate(C.byref(n), r, _ptr(sp, C.c_int64))

    def affect(self, r: int, species) -> np.ndarray:
        n, keep = self._pack()
        sp = np.array(species, dtype=np.int64)
        lib().orc_affect(C.byref(n), r, _ptr(sp, C.c_int64))
        return sp

    def run_ensemble(self, x0, seeds, tmax: float, nb_steps: int, save_idx=None, rates=None,
                     n_threads: int | None = None, want_final: bool = False):
        """Sampled runs; returns (out[nb_steps+1][n_save][n_traj], events[n_traj], total, final)."""
        S, R = self.S, self.R
        seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(-1))
        n_traj = seeds.size
        x0 = np.ascontiguousarray(np.asarray(x0, dtype=np.int64))
        x0_stride = S if x0.ndim == 2 else 0
        if save_idx is None:
            save_idx = list(range(S))
        save = np.asarray(save_idx or [0], dtype=np.int32)
        n_save = len(save_idx)
        rates_arr, rstride = None, 0
        if rates is not None:
            rates_arr = np.ascontiguousarray(np.asarray(rates, dtype=np.float64))
            rstride = R if rates_arr.ndim == 2 else 0
        out = np.zeros((nb_steps + 1, max(n_save, 1), n_traj), dtype=np.int64)
        ev = np.zeros(n_traj, dtype=np.uint64)
        final = np.zeros((n_traj, max(S, 1)), dtype=np.int64) if want_final else None
        n, keep = self._pack()
        if n_threads is None:
            n_threads = os.cpu_count() or 1
        tot = lib().orc_run_ensemble(C.byref(n), _ptr(rates_arr, C.c_double), rstride, _ptr(x0, C.c_int64),
                                     x0_stride, _ptr(seeds, C.c_uint64), n_traj, float(tmax), int(nb_steps),
                                     _ptr(save, C.c_int32), n_save, _ptr(out, C.c_int64),
                                     _ptr(final, C.c_int64), _ptr(ev, C.c_uint64), int(n_threads))
        if tot < 0:
            raise ValueError("oracle rejected the network or arguments")
        return out[:, :n_save, :], ev, int(tot), final

    def advance_until(self, species, t: float, rng_state, tmax: float, log_cap: int = 0):
        """One stateful advance_until; returns (species, t, rng_state, events, log_r, log_t)."""
        n, keep = self._pack()
        sp = np.array(species, dtype=np.int64)
        tt = C.c_double(t)
        st = np.array(rng_state, dtype=np.uint64)
        lr = np.zeros(max(log_cap, 1), dtype=np.int32)
        lt = np.zeros(max(log_cap, 1), dtype=np.float64)
        ln = C.c_int64(0)
        ev = lib().orc_advance_until(C.byref(n), _ptr(sp, C.c_int64), C.byref(tt), _ptr(st, C.c_uint64),
                                     float(tmax), _ptr(lr, C.c_int32), _ptr(lt, C.c_double), int(log_cap),
                                     C.byref(ln))
        k = min(ln.value, log_cap)
        return sp, tt.value, st, int(ev), lr[:k], lt[:k]

    def run_all_events(self, x0, seed: int, tmax: float, save_idx=None, cap: int = 1 << 20):
        S = self.S
        if save_idx is None:
            save_idx = list(range(S))
        save = np.asarray(save_idx or [0], dtype=np.int32)
        n_save = len(save_idx)
        x0 = np.ascontiguousarray(np.asarray(x0, dtype=np.int64))
        n, keep = self._pack()
        while True:
            times = np.zeros(cap, dtype=np.float64)
            out = np.zeros((cap, max(n_save, 1)), dtype=np.int64)
            k = lib().orc_run_all_events(C.byref(n), _ptr(x0, C.c_int64), C.c_uint64(int(seed)), float(tmax),
                                         _ptr(save, C.c_int32), n_save, _ptr(times, C.c_double),
                                         _ptr(out, C.c_int64), cap)
            if k < 0:
                raise ValueError("oracle rejected the network")
            if k <= cap:
                return times[:k], out[:k, :n_save]
            cap = int(k)


def seed_state(seed: int) -> np.ndarray:
    st = np.zeros(4, dtype=np.uint64)
    lib().orc_seed_state(C.c_uint64(int(seed)), _ptr(st, C.c_uint64))
    return st


def draw_u64(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.uint64)
    lib().orc_draw_u64(C.c_uint64(int(seed)), _ptr(out, C.c_uint64), n)
    return out


def draw_exp1(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float64)
    lib().orc_draw_exp1(C.c_uint64(int(seed)), _ptr(out, C.c_double), n)
    return out


def zig_tables() -> tuple[np.ndarray, np.ndarray]:
    x = np.zeros(257)
    f = np.zeros(257)
    lib().orc_zig_tables(_ptr(x, C.c_double), _ptr(f, C.c_double))
    return x, f


def numpy_seed(rng) -> int:
    """The reference Python wrapper's seed derivation (python/rebop/gillespie.py:139-140)."""
    return int(np.random.default_rng(rng).integers(np.iinfo(np.uint64).max, dtype=np.uint64))


# Reference model factories (the reference's own test/bench networks).
def sir_net(transmission: float = 1e-4, recovery: float = 0.01) -> OracleNet:
    """tests/test_rebop.py:8-12 lowered as pyo3_gillespie.rs:180-196 does: species S, I, R."""
    return (OracleNet(3).add_lma(transmission, [1, 1, 0], [-1, 1, 0])
            .add_lma(recovery, [0, 1, 0], [0, -1, 1]))


def dimer_net() -> OracleNet:
    """src/gillespie.rs:518-525 (gene, mRNA, protein, dimer)."""
    return (OracleNet(4).add_lma(25.0, [1, 0, 0, 0], [0, 1, 0, 0])
            .add_lma(1000.0, [0, 1, 0, 0], [0, 0, 1, 0])
            .add_lma(0.001, [0, 0, 2, 0], [0, 0, -2, 1])
            .add_lma(0.1, [0, 1, 0, 0], [0, -1, 0, 0])
            .add_lma(1.0, [0, 0, 1, 0], [0, 0, -1, 0]))


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(LIB_PATH)
