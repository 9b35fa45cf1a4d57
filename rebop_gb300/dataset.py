"""Result container of the Python drop-in.

The reference returns an ``xarray.Dataset`` with a ``time`` dimension and one
integer variable per species (python/rebop/gillespie.py:153-159).  When
xarray is importable the drop-in returns exactly that; otherwise it returns
this light mapping of numpy arrays with the same access patterns
(``ds.S``, ``ds["S"]``, ``ds.time``, ``"S" in ds``).
"""

from __future__ import annotations

from typing import Iterator, Mapping

import numpy as np

try:  # pragma: no cover - depends on the environment
    import xarray as xr
except ImportError:  # pragma: no cover
    xr = None


class DataArray(np.ndarray):
    """A numpy array that also answers ``.values`` and ``.dims`` like an
    ``xarray.DataArray`` variable of the reference's result."""

    dims: tuple = ()

    @property
    def values(self) -> np.ndarray:
        return np.asarray(self)


def _array(a, dims) -> DataArray:
    v = np.asarray(a).view(DataArray)
    v.dims = dims
    return v


class Dataset(Mapping):
    """Species name -> counts array, plus coordinates (``time``, ``trajectory``)."""

    def __init__(self, data_vars: Mapping[str, np.ndarray], coords: Mapping[str, np.ndarray],
                 dims: tuple[str, ...]):
        self.data_vars = {k: _array(v, dims) for k, v in data_vars.items()}
        self.coords = {k: _array(v, (k,)) for k, v in coords.items()}
        self.dims = dims

    def __getitem__(self, key):
        if isinstance(key, (list, tuple)):
            return Dataset({k: self.data_vars[k] for k in key}, self.coords, self.dims)
        if key in self.data_vars:
            return self.data_vars[key]
        return self.coords[key]

    def __getattr__(self, name):
        d = self.__dict__
        if "data_vars" in d and name in d["data_vars"]:
            return d["data_vars"][name]
        if "coords" in d and name in d["coords"]:
            return d["coords"][name]
        raise AttributeError(name)

    def __iter__(self) -> Iterator[str]:
        return iter(self.data_vars)

    def __len__(self) -> int:
        return len(self.data_vars)

    def __contains__(self, key) -> bool:
        return key in self.data_vars

    @property
    def time(self) -> np.ndarray:
        return self.coords["time"]

    def equals(self, other: "Dataset") -> bool:
        if set(self.data_vars) != set(other.data_vars) or set(self.coords) != set(other.coords):
            return False
        return (all(np.array_equal(self.coords[k], other.coords[k]) for k in self.coords)
                and all(np.array_equal(self.data_vars[k], other.data_vars[k]) for k in self.data_vars))

    def __repr__(self) -> str:
        shape = {d: len(self.coords[d]) for d in self.dims if d in self.coords}
        return f"<rebop_gb300.Dataset dims={shape} vars={list(self.data_vars)}>"


def make_dataset(times: np.ndarray, values: Mapping[str, np.ndarray], trajectories: int | None = None):
    """Build the run() result: an xarray.Dataset when available, else :class:`Dataset`."""
    times = np.asarray(times, dtype=np.float64)
    if trajectories is None:
        dims = ("time",)
        coords = {"time": times}
    else:
        dims = ("trajectory", "time")
        coords = {"trajectory": np.arange(trajectories), "time": times}
    if xr is not None:
        return xr.Dataset(
            data_vars={name: xr.DataArray(v, dims=dims, coords=coords) for name, v in values.items()},
            coords=coords,
        )
    return Dataset(values, coords, dims)
