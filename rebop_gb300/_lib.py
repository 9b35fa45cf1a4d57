"""ctypes binding of ``librebop_gb300.so`` (the C ABI in include/rebop_gb300.h).

The library is the only compute path: if it is missing and cannot be built,
importing this module raises.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import shutil

from . import build as _build

RB_OK = 0
RB_ERR_INVALID = 1
RB_ERR_CUDA = 2
RB_ERR_NOMEM = 3
RB_ERR_PARSE = 4
RB_ERR_UNSUPPORTED = 5
RB_ERR_TIMEOUT = 6


class RunStats(C.Structure):
    _fields_ = [
        ("events", C.c_uint64),
        ("kernel_ms", C.c_double),
        ("total_ms", C.c_double),
        ("h2d_bytes", C.c_uint64),
        ("d2h_bytes", C.c_uint64),
        ("kernel_launches", C.c_int32),
        ("mapping", C.c_int32),
        ("exact_reruns", C.c_uint64),
    ]


class TuneResult(C.Structure):
    _fields_ = [
        ("mapping", C.c_int32),
        ("block", C.c_int32),
        ("phase_steps", C.c_int32),
        ("sched", C.c_int32),
        ("ms", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class EngineError(RuntimeError):
    """A CUDA or resource failure inside the engine."""


def _load() -> C.CDLL:
    if not _build.up_to_date():
        if shutil.which("nvcc") is None and not _build.LIB.exists():
            raise ImportError(
                f"{_build.LIB} is missing and nvcc is not available to build it; "
                "rebop_gb300 has no CPU fallback")
        _build.build()
    return C.CDLL(str(_build.LIB))


lib = _load()

P = C.POINTER
_i32, _i64, _u64, _f64, _u32 = C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_uint32
_vp, _cp, _sz = C.c_void_p, C.c_char_p, C.c_size_t

_SIGS = {
    "rb_version": ([], _cp),
    "rb_last_error": ([_cp, _sz], _sz),
    "rb_network_create": ([_i32, P(_vp)], C.c_int),
    "rb_network_destroy": ([_vp], None),
    "rb_network_nb_species": ([_vp], _i32),
    "rb_network_nb_reactions": ([_vp], _i32),
    "rb_network_add_reaction_lma": ([_vp, _f64, P(_u32), _i32, P(_i64), _i32], C.c_int),
    "rb_network_add_reaction_lma_sparse": ([_vp, _f64, P(_u32), P(_u32), _i32, P(_i64), _i32], C.c_int),
    "rb_network_add_reaction_expr": ([_vp, P(_i32), _i32, P(_f64), _i32, P(_i64), _i32], C.c_int),
    "rb_network_from_dsl": ([_cp, P(_vp)], C.c_int),
    "rb_network_set_param": ([_vp, _cp, _f64], C.c_int),
    "rb_network_nb_params": ([_vp], _i32),
    "rb_network_param_name": ([_vp, _i32, _cp, _sz], C.c_int),
    "rb_network_species_name": ([_vp, _i32, _cp, _sz], C.c_int),
    "rb_network_name": ([_vp, _cp, _sz], C.c_int),
    "rb_network_reaction_rate": ([_vp, _i32, P(_f64)], C.c_int),
    "rb_ensemble_run": ([_vp, _i64, P(_i64), _i32, P(_f64), _i32, P(_u64), _f64, _i64, P(_i32), _i32,
                         P(_i64), P(_f64), P(_u64), P(_i64), P(RunStats)], C.c_int),
    "rb_ensemble_run_device": ([_vp, _i64, _vp, _i32, _vp, _i32, _vp, _f64, _i64, P(_i32), _i32, _vp, _vp,
                                _vp, _vp], C.c_int),
    "rb_ensemble_run_device_noalloc": ([_vp, _i64, _vp, _i32, _vp, _i32, _vp, _f64, _i64, P(_i32), _i32, _vp,
                                        _vp, _vp, _vp], C.c_int),
    "rb_ensemble_last_events": ([_vp, P(_u64)], C.c_int),
    "rb_run_all_events": ([_vp, P(_i64), _u64, _f64, P(_i32), _i32, P(_f64), P(_i64), _i64, P(_i64)],
                          C.c_int),
    "rb_trajectory_advance_until": ([_vp, P(_i64), P(_f64), P(_u64), _f64], C.c_int),
    "rb_rng_state_from_seed": ([_u64, P(_u64)], None),
    "rb_batch_create": ([P(_vp)], C.c_int),
    "rb_batch_destroy": ([_vp], None),
    "rb_batch_add": ([_vp, _vp, _i64, P(_i64), _i32, P(_f64), _i32, P(_u64), _f64, _i64, P(_i32), _i32, P(_i64),
                      P(_u64)], C.c_int),
    "rb_batch_run": ([_vp, P(RunStats)], C.c_int),
    "rb_batch_plan": ([_vp, P(_i32), P(_i32)], C.c_int),
    "rb_batch_item_mapping": ([_vp, _i32, P(_i32)], C.c_int),
    "rb_batch_item_results": ([_vp, _i32, P(P(_i64)), P(P(_u64))], C.c_int),
    "rb_ensemble_tune": ([_vp, _i64, P(_i64), _i32, P(_f64), _i32, _f64, _i64, P(TuneResult), P(TuneResult),
                          _i32, P(_i32)], C.c_int),
    "rb_tune_lookup": ([_vp, _i64, _i32, P(TuneResult)], C.c_int),
    "rb_tune_cache_path": ([_cp, _sz], _sz),
    "rb_tune_clear": ([_i32], None),
    "rbg_internal_tune_key": ([_vp, _i32, _cp, _i64, _i32, _cp, _sz], C.c_int),
    "rbg_internal_tune_candidates": ([_vp, _i32, _sz, _i64, _i64, _f64, _i32, _i32, P(TuneResult), P(TuneResult),
                                      _i32, P(_i32)], C.c_int),
    "rbg_internal_tune_store": ([_cp, P(TuneResult)], C.c_int),
    "rbg_internal_tune_get": ([_cp, P(TuneResult)], C.c_int),
    "rb_gillespie_new": ([P(_i64), _i32, _i32, P(_vp)], C.c_int),
    "rb_gillespie_new_with_seed": ([P(_i64), _i32, _i32, _u64, P(_vp)], C.c_int),
    "rb_gillespie_free": ([_vp], None),
    "rb_gillespie_seed": ([_vp, _u64], C.c_int),
    "rb_gillespie_nb_species": ([_vp], _i32),
    "rb_gillespie_nb_reactions": ([_vp], _i32),
    "rb_gillespie_add_reaction_lma": ([_vp, _f64, P(_u32), _i32, P(_i64), _i32], C.c_int),
    "rb_gillespie_add_reaction_lma_sparse": ([_vp, _f64, P(_u32), P(_u32), _i32, P(_i64), _i32], C.c_int),
    "rb_gillespie_add_reaction_expr": ([_vp, P(_i32), _i32, P(_f64), _i32, P(_i64), _i32], C.c_int),
    "rb_gillespie_get_time": ([_vp], _f64),
    "rb_gillespie_set_time": ([_vp, _f64], None),
    "rb_gillespie_get_species": ([_vp, _i32, P(_i64)], C.c_int),
    "rb_gillespie_set_species": ([_vp, P(_i64), _i32], C.c_int),
    "rb_gillespie_advance_until": ([_vp, _f64], C.c_int),
    "rb_gillespie_advance_one_reaction": ([_vp], C.c_int),
}

for _name, (_args, _res) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.argtypes = _args
    _f.restype = _res

lib.rbg_internal_zig_tables.argtypes = [P(_f64), P(_f64)]
lib.rbg_internal_zig_tables.restype = None
lib.rbg_internal_fp64_fma_rate.argtypes = [_vp]
lib.rbg_internal_fp64_fma_rate.restype = _f64
_f32 = C.c_float
for _name, _args in {
    "rbg_mdn_gemm": [_vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _f32,
                     _vp],
    "rbg_mdn_gemm_tc05": [_vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, C.c_int, C.c_int,
                          _f32, _vp, _vp],
    "rbg_mdn_bias_act": [_vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp],
    "rbg_mdn_silu_backward": [_vp, _vp, _vp, _vp, C.c_int, C.c_int, _vp],
    "rbg_mdn_head_backward": [_vp, _vp, _vp, C.c_int, C.c_int, _vp],
    "rbg_mdn_loss": [_vp, _vp, C.c_int, C.c_int, _vp, _vp, _vp],
    "rbg_mdn_adam": [_vp, _vp, _vp, _vp, _vp, C.c_int, _f32, _f32, _f32, _f32, C.c_int, _vp],
    "rbg_mdn_sample": [_vp, C.c_int, C.c_int, _u64, _vp, C.c_int, _vp, _vp],
    "rbg_mdn_rre": [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, _vp, C.c_int, _vp, _vp],
    "rbg_mdn_count_loss": [_vp, _vp, C.c_int, C.c_int, _vp, _vp, _vp],
    "rbg_mdn_count_sample": [_vp, C.c_int, C.c_int, _u64, _vp, C.c_int, _vp, _vp, _vp],
    "rbg_mdn_infer": [_vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int,
                      _vp, _vp, _vp],
}.items():
    getattr(lib, _name).argtypes = _args
    getattr(lib, _name).restype = C.c_int
lib.rbg_internal_batch_times.argtypes = [_vp, P(C.c_float), P(C.c_float), P(C.c_float)]
lib.rbg_internal_batch_times.restype = C.c_int
lib.rbg_internal_jit_source.argtypes = [_vp, _cp, _sz]
lib.rbg_internal_jit_source.restype = C.c_int
lib.rbg_internal_jit_compile.argtypes = [_vp, P(_u64)]
lib.rbg_internal_jit_compile.restype = C.c_int
lib.rbg_internal_warp_dep_table.argtypes = [_vp, P(C.c_uint16), _sz]
lib.rbg_internal_warp_dep_table.restype = C.c_int


def last_error() -> str:
    buf = C.create_string_buffer(4096)
    lib.rb_last_error(buf, 4096)
    return buf.value.decode("utf-8", "replace")


def check(rc: int) -> None:
    """Raise the Python error matching a C-ABI status."""
    if rc == RB_OK:
        return
    msg = last_error()
    if rc in (RB_ERR_INVALID, RB_ERR_PARSE, RB_ERR_UNSUPPORTED):
        raise ValueError(msg)
    if rc == RB_ERR_NOMEM:
        raise MemoryError(msg)
    raise EngineError(msg)


def ptr(a, ct):
    """ctypes pointer to a numpy array's data (NULL for None)."""
    if a is None:
        return P(ct)()
    return a.ctypes.data_as(P(ct))
