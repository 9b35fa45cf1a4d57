"""Python drop-in for ``rebop.Gillespie`` running on the GPU.

Mirrors python/rebop/gillespie.py:22-160 and the PyO3 class it wraps
(src/pyo3_gillespie.rs:10-253): same methods, argument meaning, seed
derivation, warnings and error messages.  ``run`` returns what the reference
returns (an ``xarray.Dataset`` with a ``time`` dimension when xarray is
installed).  :meth:`Gillespie.run_ensemble` is the batched addition: many
trajectories in one GPU launch, trajectory 0 identical to ``run`` with the
same ``rng``.
"""

from __future__ import annotations

import warnings
from collections.abc import Mapping, Sequence

import numpy as np

from . import expr as _expr
from .api import Network, Rate
from .dataset import make_dataset

__all__ = ("Gillespie",)

_INIT_WARNING = "Some species are not involved in any reactions. You should probably instead use parameters."


def _seeds_from_rng(rng, n: int | None) -> np.ndarray | int:
    # python/rebop/gillespie.py:139-140: one u64 below 2**64-1 per run.
    rng_ = np.random.default_rng(rng)
    if n is None:
        return int(rng_.integers(np.iinfo(np.uint64).max, dtype=np.uint64))
    return rng_.integers(np.iinfo(np.uint64).max, size=n, dtype=np.uint64)


class Gillespie:
    """Reaction system composed of species and reactions."""

    def __init__(self) -> None:
        self._species: dict[str, int] = {}
        self._init: dict[str, int] = {}
        self._reactions: list[tuple[float | _expr.PExpr, list[str], list[str], float | str]] = []

    # -- model building (pyo3_gillespie.rs:76-117)
    def add_species(self, species: str) -> None:
        if species not in self._species:
            self._species[species] = len(self._species)

    def nb_species(self) -> int:
        return len(self._species)

    def nb_reactions(self) -> int:
        return len(self._reactions)

    def add_reaction(self, rate: float | str, reactants: Sequence[str], products: Sequence[str],
                     reverse_rate: float | str | None = None) -> None:
        """Add a reaction: a numeric ``rate`` is a mass-action constant, a string an
        arbitrary rate expression over species and ``params`` (gillespie.py:29-90)."""
        if isinstance(rate, str):
            try:
                prate: float | _expr.PExpr = _expr.parse(rate)
            except _expr.ParseError:
                raise ValueError("Rate expression not understood") from None
        else:
            prate = float(rate)
        reactants = [str(r) for r in reactants]
        products = [str(p) for p in products]
        for r in reactants:
            self.add_species(r)
        for p in products:
            self.add_species(p)
        self._reactions.append((prate, reactants, products, rate))
        if reverse_rate is not None:
            self.add_reaction(reverse_rate, products, reactants, None)

    def __str__(self) -> str:
        s = f"{len(self._species)} species and {len(self._reactions)} reactions\n"
        for prate, reactants, products, _ in self._reactions:
            r = f"LMA({_fmt_float(prate)})" if isinstance(prate, float) else str(prate)
            s += " + ".join(reactants) + " --> " + " + ".join(products) + f" @ {r}\n"
        return s

    def set_init(self, init: Mapping[str, int]) -> bool:
        """pyo3_gillespie.rs:119-134: unknown species are added; returns whether to warn."""
        warn = False
        for name in init:
            if name not in self._species:
                warn = True
                self.add_species(name)
        clean = {}
        for name, v in init.items():
            v = int(v)
            if v < 0:
                raise OverflowError("can't convert negative int to unsigned")
            clean[name] = v
        self._init = clean
        return warn

    # -- lowering (pyo3_gillespie.rs:154-196)
    def _lower(self, params: Mapping[str, float], var_names):
        for p in params:
            if p in self._species:
                raise ValueError(f"Species {p} cannot also be a parameter.")
        S = len(self._species)
        x0 = np.zeros(S, dtype=np.int64)
        for name, v in self._init.items():
            if name in self._species:
                x0[self._species[name]] = v
        if var_names is None:
            names = list(self._species)
        else:
            names = [str(v) for v in var_names]
            for v in names:
                if v not in self._species:
                    raise ValueError(f"Unknown species {v!r} in var_names")
        save = [self._species[v] for v in names]
        # Species and reactions are only ever appended, so their counts and
        # the parameters identify the lowered network: repeated runs reuse it
        # (and from the second run on get the kernel compiled for it).
        key = (S, len(self._reactions), tuple(sorted((str(k), float(v)) for k, v in params.items())))
        cached = getattr(self, "_net_cache", None)
        if cached is not None and cached[0] == key:
            return cached[1], x0, names, save
        net = Network(S)
        for prate, reactants, products, _ in self._reactions:
            exps = [0] * S
            for r in reactants:
                exps[self._species[r]] += 1
            diff = [0] * S
            for r in reactants:
                diff[self._species[r]] -= 1
            for p in products:
                diff[self._species[p]] += 1
            if isinstance(prate, float):
                net.add_reaction(Rate.lma(prate, exps), diff)
            else:
                # Rate::Expr: the expression alone is the propensity (gillespie.rs:88)
                net.add_reaction(Rate.expression(prate.to_expr(self._species, params)), diff)
        self._net_cache = (key, net)
        return net, x0, names, save

    # -- runs
    def run(self, init: Mapping[str, int], tmax: float, nb_steps: int, *,
            params: Mapping[str, float] | None = None, rng=None, sparse: bool | None = None,
            var_names: Sequence[str] | None = None):
        """Run the system until ``tmax`` with ``nb_steps`` steps (gillespie.py:96-160).

        ``nb_steps = 0`` returns every reaction, ending with the first one at or
        after ``tmax`` (pyo3_gillespie.rs:209-223).  ``sparse`` is accepted for
        compatibility: the descriptor is always sparse and the representation
        does not change results (tests/test_rebop.py:55-65).
        """
        params = {} if params is None else dict(params)
        seed = _seeds_from_rng(rng, None)
        if self.set_init(init):
            warnings.warn(UserWarning(_INIT_WARNING), stacklevel=2)
        nb_steps = int(nb_steps)
        if nb_steps < 0:
            raise OverflowError("can't convert negative int to unsigned")
        net, x0, names, save = self._lower(params, var_names)
        if nb_steps > 0:
            res = net.run_ensemble(x0, [seed], float(tmax), nb_steps, save=save, want_events=False)
            times = res.times
            values = {n: res.counts[:, k, 0].copy() for k, n in enumerate(names)}
        else:
            times, out = net.run_all_events(x0, seed, float(tmax), save=save)
            values = {n: out[:, k].copy() for k, n in enumerate(names)}
        return make_dataset(times, values)

    def run_ensemble(self, init: Mapping[str, int], tmax: float, nb_steps: int, n_trajectories: int, *,
                     params: Mapping[str, float] | None = None, rng=None, seeds=None,
                     rates=None, sparse: bool | None = None, var_names: Sequence[str] | None = None):
        """Run ``n_trajectories`` independent trajectories in one GPU launch.

        Seeds are drawn like ``run`` draws its one seed, so trajectory 0 equals
        ``run(init, tmax, nb_steps, rng=rng)``; pass ``seeds`` to pin each
        trajectory's stream.  ``rates`` (shape (R,) or (n_trajectories, R), in
        reaction order) overrides the mass-action constants.  Returns a dataset
        with dims (trajectory, time).
        """
        params = {} if params is None else dict(params)
        n = int(n_trajectories)
        if seeds is None:
            seeds = _seeds_from_rng(rng, n)
        seeds = np.asarray(seeds, dtype=np.uint64).reshape(-1)
        if seeds.size != n:
            raise ValueError("need one seed per trajectory")
        if self.set_init(init):
            warnings.warn(UserWarning(_INIT_WARNING), stacklevel=2)
        if int(nb_steps) < 1:
            raise ValueError("run_ensemble needs nb_steps >= 1")
        net, x0, names, save = self._lower(params, var_names)
        res = net.run_ensemble(x0, seeds, float(tmax), int(nb_steps), save=save, rates=rates)
        values = {nm: np.ascontiguousarray(res.counts[:, k, :].T) for k, nm in enumerate(names)}
        ds = make_dataset(res.times, values, trajectories=n)
        return ds


def _fmt_float(x: float) -> str:
    # Rust's Display for f64: integral values print without a decimal point.
    if x == int(x) and abs(x) < 1e16:
        return str(int(x))
    return repr(x)
