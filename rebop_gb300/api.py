"""Run-time API of rebop's core engine, on the GPU.

Mirrors ``rebop::gillespie`` (src/gillespie.rs): :class:`Rate`, :class:`Jump`
and the stateful single-trajectory :class:`Gillespie`, plus the batched
entry point the reference does not have: :class:`Network` and
:meth:`Network.run_ensemble`, which run many independent trajectories in one
kernel launch.  Everything calls the C ABI of ``librebop_gb300.so``.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Iterable, Sequence

import numpy as np

from ._lib import RunStats, TuneResult, check, lib, ptr

_u32, _i64, _u64, _f64, _i32 = C.c_uint32, C.c_int64, C.c_uint64, C.c_double, C.c_int32


# --------------------------------------------------------------------- Rate
@dataclass(frozen=True)
class Rate:
    """``rebop::gillespie::Rate`` for the law of mass action (src/gillespie.rs:12-69).

    ``Rate.lma(k, exps)`` holds one exponent per species; ``Rate.lma_sparse(k,
    pairs)`` holds (species index, exponent) pairs multiplied in the given order.
    """

    rate: float
    exponents: tuple = ()
    pairs: tuple | None = None
    expr: object = None  # Rate::Expr: a resolved expression tree (rebop_gb300.expr.Expr)

    @staticmethod
    def lma(rate: float, exponents: Iterable[int]) -> "Rate":
        return Rate(float(rate), tuple(int(e) for e in exponents), None)

    @staticmethod
    def lma_sparse(rate: float, pairs: Iterable[tuple[int, int]]) -> "Rate":
        return Rate(float(rate), (), tuple((int(i), int(e)) for i, e in pairs))

    @staticmethod
    def expression(expr) -> "Rate":
        """``Rate::expr`` (gillespie.rs:33-35): the propensity is the value of a
        resolved expression tree over species counts (src/expr.rs:8-39)."""
        return Rate(0.0, (), None, expr)

    @property
    def is_sparse(self) -> bool:
        return self.pairs is not None

    def dense(self) -> "Rate":
        """Rate::dense (gillespie.rs:37-53): length = 1 + the largest index."""
        if not self.is_sparse:
            return self
        n = max((i + 1 for i, _ in self.pairs), default=0)
        d = [0] * n
        for i, e in self.pairs:
            d[i] += e
        return Rate.lma(self.rate, d)

    def sparse(self) -> "Rate":
        """Rate::sparse (gillespie.rs:55-69): the non-zero exponents in index order."""
        if self.is_sparse:
            return self
        return Rate.lma_sparse(self.rate, [(i, e) for i, e in enumerate(self.exponents) if e > 0])


@dataclass(frozen=True)
class Jump:
    """``rebop::gillespie::Jump`` (src/gillespie.rs:95-153)."""

    differences: tuple = ()
    entries: tuple | None = None

    @staticmethod
    def new(differences: Iterable[int]) -> "Jump":
        return Jump(tuple(int(d) for d in differences), None)

    @staticmethod
    def new_sparse(entries: Iterable[tuple[int, int]]) -> "Jump":
        return Jump((), tuple((int(i), int(d)) for i, d in entries))

    def dense(self) -> "Jump":
        if self.entries is None:
            return self
        n = max((i + 1 for i, _ in self.entries), default=0)
        d = [0] * n
        for i, x in self.entries:
            d[i] += x
        return Jump.new(d)

    def sparse(self) -> "Jump":
        if self.entries is not None:
            return self
        return Jump.new_sparse([(i, d) for i, d in enumerate(self.differences) if d != 0])


def _u32a(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(list(x) if not isinstance(x, np.ndarray) else x, dtype=np.uint32))


def _i64a(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(list(x) if not isinstance(x, np.ndarray) else x, dtype=np.int64))


# ------------------------------------------------------------------ Network
@dataclass
class EnsembleResult:
    """Output of :meth:`Network.run_ensemble`.

    ``counts[i, k, j]`` is saved species k of trajectory j at ``times[i]``.
    """

    times: np.ndarray
    counts: np.ndarray
    events: np.ndarray | None
    final: np.ndarray | None
    stats: dict = field(default_factory=dict)

    @property
    def total_events(self) -> int:
        return int(self.stats.get("events", 0))


class Network:
    """The packed reaction descriptor every kernel reads (C handle ``rb_network``)."""

    def __init__(self, n_species: int = 0, *, _handle=None):
        if _handle is not None:
            self._h = _handle
        else:
            h = C.c_void_p()
            check(lib.rb_network_create(int(n_species), C.byref(h)))
            self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.rb_network_destroy(h)
            self._h = None

    @classmethod
    def from_dsl(cls, text: str) -> "Network":
        """Lower a ``define_system!`` body (src/gillespie_macro.rs:50-58)."""
        h = C.c_void_p()
        check(lib.rb_network_from_dsl(text.encode("utf-8"), C.byref(h)))
        return cls(_handle=h)

    @property
    def nb_species(self) -> int:
        return lib.rb_network_nb_species(self._h)

    @property
    def nb_reactions(self) -> int:
        return lib.rb_network_nb_reactions(self._h)

    @property
    def name(self) -> str:
        buf = C.create_string_buffer(1024)
        check(lib.rb_network_name(self._h, buf, 1024))
        return buf.value.decode()

    @property
    def params(self) -> list[str]:
        out = []
        buf = C.create_string_buffer(1024)
        for i in range(lib.rb_network_nb_params(self._h)):
            check(lib.rb_network_param_name(self._h, i, buf, 1024))
            out.append(buf.value.decode())
        return out

    @property
    def species(self) -> list[str]:
        out = []
        buf = C.create_string_buffer(1024)
        for i in range(self.nb_species):
            check(lib.rb_network_species_name(self._h, i, buf, 1024))
            out.append(buf.value.decode())
        return out

    def set_param(self, name: str, value: float) -> None:
        check(lib.rb_network_set_param(self._h, name.encode("utf-8"), float(value)))

    def reaction_rate(self, r: int) -> float:
        v = C.c_double()
        check(lib.rb_network_reaction_rate(self._h, int(r), C.byref(v)))
        return v.value

    def add_reaction(self, rate: Rate, differences: Sequence[int]) -> "Network":
        """``Gillespie::add_reaction`` (src/gillespie.rs:225-244)."""
        d = _i64a(differences)
        if rate.expr is not None:
            code, consts = rate.expr.to_program()
            c = np.ascontiguousarray(np.asarray(code, dtype=np.int32))
            k = np.ascontiguousarray(np.asarray(consts or [0.0], dtype=np.float64))
            check(lib.rb_network_add_reaction_expr(self._h, ptr(c, _i32), c.size, ptr(k, _f64), len(consts),
                                                   ptr(d, _i64), d.size))
        elif rate.is_sparse:
            idx = _u32a([i for i, _ in rate.pairs])
            ex = _u32a([e for _, e in rate.pairs])
            check(lib.rb_network_add_reaction_lma_sparse(self._h, rate.rate, ptr(idx, _u32), ptr(ex, _u32),
                                                         len(rate.pairs), ptr(d, _i64), d.size))
        else:
            ex = _u32a(rate.exponents)
            check(lib.rb_network_add_reaction_lma(self._h, rate.rate, ptr(ex, _u32), ex.size, ptr(d, _i64),
                                                  d.size))
        return self

    def _save(self, save):
        if save is None:
            return None, -1
        s = np.ascontiguousarray(np.asarray(save, dtype=np.int32))
        return s, s.size

    def run_ensemble(self, x0, seeds, tmax: float, nb_steps: int, *, save=None, rates=None,
                     want_events: bool = True, want_final: bool = False, out: np.ndarray | None = None,
                     events: np.ndarray | None = None) -> EnsembleResult:
        """Run ``len(seeds)`` trajectories from host arrays (``rb_ensemble_run``).

        ``x0`` is one count vector or one per trajectory; ``rates`` is None
        (the network's constants), one rate vector, or one per trajectory.
        ``out`` / ``events`` may be caller-owned (e.g. page-locked) arrays of
        the result shapes, written in place.
        """
        S = self.nb_species
        seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(-1))
        n = seeds.size
        x0 = _i64a(np.asarray(x0, dtype=np.int64))
        x0_per = 1 if x0.ndim == 2 else 0
        if x0_per and x0.shape != (n, S):
            raise ValueError(f"x0 must have shape ({n}, {S})")
        if not x0_per and x0.size != S:
            raise ValueError(f"x0 must have {S} entries")
        r_arr, r_per = None, 0
        if rates is not None:
            r_arr = np.ascontiguousarray(np.asarray(rates, dtype=np.float64))
            r_per = 1 if r_arr.ndim == 2 else 0
            R = self.nb_reactions
            if (r_per and r_arr.shape != (n, R)) or (not r_per and r_arr.size != R):
                raise ValueError("rates must have shape (R,) or (n_traj, R)")
        save_arr, n_save = self._save(save)
        NS = S if n_save < 0 else n_save
        if out is None:
            out = np.empty((nb_steps + 1, NS, n), dtype=np.int64)
        elif out.shape != (nb_steps + 1, NS, n) or out.dtype != np.int64 or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous int64 array of shape {(nb_steps + 1, NS, n)}")
        times = np.empty(nb_steps + 1, dtype=np.float64)
        if events is not None:
            if events.shape != (n,) or events.dtype != np.uint64:
                raise ValueError("events must be a uint64 array with one entry per trajectory")
            ev = events
        else:
            ev = np.empty(n, dtype=np.uint64) if want_events else None
        fin = np.empty((n, S), dtype=np.int64) if want_final else None
        st = RunStats()
        check(lib.rb_ensemble_run(self._h, n, ptr(x0, _i64), x0_per, ptr(r_arr, _f64), r_per,
                                  ptr(seeds, _u64), float(tmax), int(nb_steps), ptr(save_arr, _i32), n_save,
                                  ptr(out, _i64), ptr(times, _f64), ptr(ev, _u64), ptr(fin, _i64),
                                  C.byref(st)))
        stats = {k: getattr(st, k) for k, _ in RunStats._fields_}
        return EnsembleResult(times, out, ev, fin, stats)

    def run_ensemble_device(self, n_traj: int, x0_ptr: int, x0_per_traj: bool, seeds_ptr: int, tmax: float,
                            nb_steps: int, out_ptr: int, *, rates_ptr: int = 0, rates_per_traj: bool = False,
                            save=None, events_ptr: int = 0, final_ptr: int = 0, stream: int = 0) -> None:
        """Enqueue a run on device buffers (``rb_ensemble_run_device``); raw pointers."""
        save_arr, n_save = self._save(save)
        check(lib.rb_ensemble_run_device(self._h, int(n_traj), x0_ptr or None, int(bool(x0_per_traj)),
                                         rates_ptr or None, int(bool(rates_per_traj)), seeds_ptr or None,
                                         float(tmax), int(nb_steps), ptr(save_arr, _i32), n_save,
                                         out_ptr or None, events_ptr or None, final_ptr or None,
                                         stream or None))

    def tune(self, x0, n_traj: int, tmax: float, nb_steps: int, *, rates=None) -> dict:
        """Autotune the kernel and launch shape for ensembles of this network
        (``rb_ensemble_tune``): pilot runs of ``n_traj`` trajectories from
        ``x0`` (one count vector or one per trajectory) with ``rates`` (None,
        one vector, or one per trajectory).  The winner is remembered for
        networks of this shape on this GPU and used by later runs.  Returns
        ``{"best": {...}, "trials": [...]}`` (times in ms)."""
        S = self.nb_species
        x0 = _i64a(np.asarray(x0, dtype=np.int64))
        x0_per = 1 if x0.ndim == 2 else 0
        if x0.size != (n_traj * S if x0_per else S):
            raise ValueError("x0 must have one count per species, or one row per trajectory")
        r_arr, r_per = None, 0
        if rates is not None:
            r_arr = np.ascontiguousarray(np.asarray(rates, dtype=np.float64))
            r_per = 1 if r_arr.ndim == 2 else 0
        best = TuneResult()
        trials = (TuneResult * 64)()
        n = C.c_int32()
        check(lib.rb_ensemble_tune(self._h, int(n_traj), ptr(x0, _i64), x0_per, ptr(r_arr, _f64), r_per,
                                   float(tmax), int(nb_steps), C.byref(best), trials, 64, C.byref(n)))
        return {"best": best.as_dict(), "trials": [trials[k].as_dict() for k in range(min(n.value, 64))]}

    def tuned(self, n_traj: int, *, rates_per_traj: bool = False) -> dict | None:
        """The remembered shape for this network at ``n_traj`` trajectories, or None."""
        out = TuneResult()
        if lib.rb_tune_lookup(self._h, int(n_traj), int(bool(rates_per_traj)), C.byref(out)) != 0:
            return None
        return out.as_dict()

    def last_events(self) -> int:
        v = C.c_uint64()
        check(lib.rb_ensemble_last_events(self._h, C.byref(v)))
        return int(v.value)

    def run_all_events(self, x0, seed: int, tmax: float, *, save=None, cap: int = 4096):
        """Every-event run of one trajectory (``rb_run_all_events``): (times, counts[n, n_save])."""
        x0 = _i64a(x0)
        save_arr, n_save = self._save(save)
        NS = self.nb_species if n_save < 0 else n_save
        while True:
            times = np.empty(cap, dtype=np.float64)
            out = np.empty((cap, NS), dtype=np.int64)
            nrec = C.c_int64()
            check(lib.rb_run_all_events(self._h, ptr(x0, _i64), C.c_uint64(int(seed)), float(tmax),
                                        ptr(save_arr, _i32), n_save, ptr(times, _f64), ptr(out, _i64), cap,
                                        C.byref(nrec)))
            k = int(nrec.value)
            if k <= cap:
                return times[:k], out[:k]
            cap = k


# ----------------------------------------------------------- Gillespie (Rust)
class Gillespie:
    """``rebop::gillespie::Gillespie`` (src/gillespie.rs:157-344): one stateful trajectory.

    ``Gillespie(species, sparse)`` is ``Gillespie::new`` (OS-entropy seed);
    ``Gillespie.new_with_seed(species, sparse, seed)`` pins the stream.  Every
    ``advance_until`` / ``advance_one_reaction`` runs on the GPU.
    """

    def __init__(self, species: Sequence[int], sparse: bool = False, seed: int | None = None):
        sp = _i64a(species)
        h = C.c_void_p()
        if seed is None:
            check(lib.rb_gillespie_new(ptr(sp, _i64), sp.size, int(bool(sparse)), C.byref(h)))
        else:
            check(lib.rb_gillespie_new_with_seed(ptr(sp, _i64), sp.size, int(bool(sparse)), C.c_uint64(int(seed)),
                                                 C.byref(h)))
        self._h = h

    @classmethod
    def new(cls, species: Sequence[int], sparse: bool = False) -> "Gillespie":
        return cls(species, sparse)

    @classmethod
    def new_with_seed(cls, species: Sequence[int], sparse: bool, seed: int) -> "Gillespie":
        return cls(species, sparse, seed)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.rb_gillespie_free(h)
            self._h = None

    def seed(self, seed: int) -> None:
        check(lib.rb_gillespie_seed(self._h, C.c_uint64(int(seed))))

    def nb_species(self) -> int:
        return lib.rb_gillespie_nb_species(self._h)

    def nb_reactions(self) -> int:
        return lib.rb_gillespie_nb_reactions(self._h)

    def add_reaction(self, rate: Rate, differences: Sequence[int]) -> None:
        d = _i64a(differences)
        if rate.expr is not None:
            code, consts = rate.expr.to_program()
            c = np.ascontiguousarray(np.asarray(code, dtype=np.int32))
            k = np.ascontiguousarray(np.asarray(consts or [0.0], dtype=np.float64))
            check(lib.rb_gillespie_add_reaction_expr(self._h, ptr(c, _i32), c.size, ptr(k, _f64), len(consts),
                                                     ptr(d, _i64), d.size))
        elif rate.is_sparse:
            idx = _u32a([i for i, _ in rate.pairs])
            ex = _u32a([e for _, e in rate.pairs])
            check(lib.rb_gillespie_add_reaction_lma_sparse(self._h, rate.rate, ptr(idx, _u32), ptr(ex, _u32),
                                                           len(rate.pairs), ptr(d, _i64), d.size))
        else:
            ex = _u32a(rate.exponents)
            check(lib.rb_gillespie_add_reaction_lma(self._h, rate.rate, ptr(ex, _u32), ex.size, ptr(d, _i64),
                                                    d.size))

    def get_time(self) -> float:
        return lib.rb_gillespie_get_time(self._h)

    def set_time(self, t: float) -> None:
        lib.rb_gillespie_set_time(self._h, float(t))

    def get_species(self, s: int) -> int:
        v = C.c_int64()
        check(lib.rb_gillespie_get_species(self._h, int(s), C.byref(v)))
        return int(v.value)

    def set_species(self, species: Sequence[int]) -> None:
        sp = _i64a(species)
        check(lib.rb_gillespie_set_species(self._h, ptr(sp, _i64), sp.size))

    def advance_one_reaction(self) -> None:
        check(lib.rb_gillespie_advance_one_reaction(self._h))

    def advance_until(self, tmax: float) -> None:
        check(lib.rb_gillespie_advance_until(self._h, float(tmax)))


class Batch:
    """Many ensembles -- different networks, parameters, horizons -- run by one
    CUDA graph (``rb_batch_*``).  ``add`` returns the item's index; after
    ``run``, ``counts(k)`` and ``events(k)`` hold its results, identical to
    ``Network.run_ensemble`` on the same item."""

    def __init__(self):
        h = C.c_void_p()
        check(lib.rb_batch_create(C.byref(h)))
        self._h = h
        self._keep = []   # inputs and outputs the library points to
        self._out = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.rb_batch_destroy(h)
            self._h = None

    def add(self, network: "Network", x0, seeds, tmax: float, nb_steps: int, *, rates=None, save=None,
            want_events: bool = True, copy: bool = True) -> int:
        """Add one ensemble; returns its index.  copy=False: no result arrays of
        its own -- ``counts(k)`` and ``events(k)`` are then views of the batch's
        results (the page-locked staging buffer for items of the persistent
        launch), valid until the next ``run`` or ``add``."""
        S, R = network.nb_species, network.nb_reactions
        seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64).reshape(-1))
        n = seeds.size
        x0 = np.ascontiguousarray(np.asarray(x0, dtype=np.int64))
        x0_per = 1 if x0.ndim == 2 else 0
        if x0.size != (n * S if x0_per else S):
            raise ValueError("x0 must have one count per species, or one row per trajectory")
        r_arr, r_per = None, 0
        if rates is not None:
            r_arr = np.ascontiguousarray(np.asarray(rates, dtype=np.float64))
            r_per = 1 if r_arr.ndim == 2 else 0
            if r_arr.size != (n * R if r_per else R):
                raise ValueError("rates must have one entry per reaction, or one row per trajectory")
        save_arr, n_save = (None, -1) if save is None else (np.ascontiguousarray(np.asarray(save, np.int32)), len(save))
        ns = S if n_save < 0 else n_save
        shape = (int(nb_steps) + 1, ns, n)
        out = np.zeros(shape, dtype=np.int64) if copy else None
        ev = np.zeros(n, dtype=np.uint64) if want_events and copy else None
        check(lib.rb_batch_add(self._h, network._h, n, ptr(x0, _i64), x0_per, ptr(r_arr, _f64), r_per,
                               ptr(seeds, _u64), float(tmax), int(nb_steps), ptr(save_arr, _i32), n_save,
                               ptr(out, _i64), ptr(ev, _u64)))
        self._keep.append((network, seeds, x0, r_arr, save_arr))
        self._out.append((out, ev) if copy else shape)
        return len(self._out) - 1

    def _view(self, k: int):
        o, e = C.POINTER(_i64)(), C.POINTER(_u64)()
        check(lib.rb_batch_item_results(self._h, int(k), C.byref(o), C.byref(e)))
        shape = self._out[k]
        counts = np.ctypeslib.as_array(o, shape=shape) if shape[1] * shape[2] else np.zeros(shape, np.int64)
        events = np.ctypeslib.as_array(e, shape=(shape[2],)) if shape[2] else np.zeros(0, np.uint64)
        return counts, events

    def seeds(self, k: int) -> np.ndarray:
        """Item k's seed array: change it in place between runs for fresh trajectories."""
        return self._keep[k][1]

    def run(self) -> dict:
        st = RunStats()
        check(lib.rb_batch_run(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in RunStats._fields_}

    def counts(self, k: int) -> np.ndarray:
        o = self._out[k]
        return self._view(k)[0] if isinstance(o, tuple) and isinstance(o[0], int) else o[0]

    def events(self, k: int):
        o = self._out[k]
        return self._view(k)[1] if isinstance(o, tuple) and isinstance(o[0], int) else o[1]

    def plan(self) -> tuple[int, int]:
        """(launches of their own, items of the persistent launch)."""
        a, b = C.c_int32(), C.c_int32()
        check(lib.rb_batch_plan(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def times(self) -> dict:
        """Device time of the last run's graph: input copy, kernels, result copy (ms)."""
        a, b, c = C.c_float(), C.c_float(), C.c_float()
        check(lib.rbg_internal_batch_times(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"in_ms": a.value, "kernels_ms": b.value, "out_ms": c.value}

    def mapping(self, k: int) -> int:
        m = C.c_int32()
        check(lib.rb_batch_item_mapping(self._h, int(k), C.byref(m)))
        return m.value


def zig_tables() -> tuple[np.ndarray, np.ndarray]:
    """The Exp1 ziggurat tables the engine uploads (for tests)."""
    x = np.empty(257)
    f = np.empty(257)
    lib.rbg_internal_zig_tables(ptr(x, _f64), ptr(f, _f64))
    return x, f
