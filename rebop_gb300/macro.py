"""``define_system!`` for Python: network text lowered to the packed descriptor.

``define_system(text)`` parses a macro body (src/gillespie_macro.rs:50-58) and
returns a class shaped like the struct the macro generates
(gillespie_macro.rs:59-127): one attribute per species (int, starts at 0) and
per parameter (float, starts at NaN), the clock ``t``, and the methods
``new``, ``with_parameters``, ``seed`` and ``advance_until``.  Every advance
runs on the GPU with the macro's arithmetic; ``run_ensemble`` runs many
copies of the current state in one launch.
"""

from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._lib import check, lib, ptr
from .api import Network


def define_system(text: str) -> type:
    net = Network.from_dsl(text)
    species = net.species
    params = net.params
    name = net.name or "System"

    class System:
        __slots__ = tuple(species) + tuple(params) + ("t", "_rng")
        _network = net
        _species = tuple(species)
        _params = tuple(params)

        def __init__(self, **values):
            for s in species:
                object.__setattr__(self, s, 0)
            for p in params:
                object.__setattr__(self, p, math.nan)
            self.t = 0.0
            st = np.zeros(4, dtype=np.uint64)
            lib.rb_rng_state_from_seed(C.c_uint64(int(np.random.SeedSequence().generate_state(1, np.uint64)[0])),
                                       ptr(st, C.c_uint64))
            self._rng = st
            for k, v in values.items():
                setattr(self, k, v)

        @classmethod
        def new(cls) -> "System":
            """Species at 0, parameters NaN, an entropy-seeded stream (gillespie_macro.rs:71-78)."""
            return cls()

        @classmethod
        def with_parameters(cls, *values: float) -> "System":
            """All parameters in declaration order (gillespie_macro.rs:88-95)."""
            if len(values) != len(params):
                raise TypeError(f"{name}.with_parameters takes {len(params)} values")
            obj = cls()
            for p, v in zip(params, values):
                setattr(obj, p, float(v))
            return obj

        def seed(self, seed: int) -> None:
            """SmallRng::seed_from_u64 (gillespie_macro.rs:81-84)."""
            lib.rb_rng_state_from_seed(C.c_uint64(int(seed)), ptr(self._rng, C.c_uint64))

        def _push_params(self) -> None:
            for p in params:
                net.set_param(p, float(getattr(self, p)))

        def advance_until(self, tmax: float) -> None:
            """Simulate until ``t = tmax`` (gillespie_macro.rs:98-126), on the GPU."""
            self._push_params()
            sp = np.array([int(getattr(self, s)) for s in species], dtype=np.int64)
            t = C.c_double(float(self.t))
            check(lib.rb_trajectory_advance_until(net._h, ptr(sp, C.c_int64), C.byref(t),
                                                  ptr(self._rng, C.c_uint64), float(tmax)))
            for s, v in zip(species, sp.tolist()):
                object.__setattr__(self, s, v)
            self.t = t.value

        def run_ensemble(self, seeds, tmax: float, nb_steps: int, *, rates=None):
            """Many trajectories from the current counts, one per seed (t restarts at 0)."""
            self._push_params()
            x0 = np.array([int(getattr(self, s)) for s in species], dtype=np.int64)
            return net.run_ensemble(x0, seeds, tmax, nb_steps, rates=rates)

        def __repr__(self) -> str:
            body = ", ".join(f"{s}={getattr(self, s)}" for s in species)
            return f"{name}(t={self.t}, {body})"

    System.__name__ = name
    System.__qualname__ = name
    return System
