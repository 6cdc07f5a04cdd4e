"""ctypes binding of ``libb3g.so`` (the C ABI in ``include/b3g.h``).

The library is the only compute path: importing this module fails loudly when
the shared object is missing, and every non-OK status raises ``B3GError`` with
the library's own message.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libb3g.so"

B3G_OK = 0
B3G_ERR_INVALID_ARGUMENT = 1
B3G_ERR_OUT_OF_MEMORY = 2
B3G_ERR_CUDA = 3
B3G_ERR_TIMEOUT = 4
B3G_ERR_NUMERIC = 5
B3G_ERR_STATE = 6

PRECISION_F64 = 0
PRECISION_F32 = 1

STATUS_NAMES = {
    0: "OK",
    1: "INVALID_ARGUMENT",
    2: "OUT_OF_MEMORY",
    3: "CUDA",
    4: "TIMEOUT",
    5: "NUMERIC",
    6: "STATE",
}


class B3GError(RuntimeError):
    """A b3g call returned a non-OK status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"b3g {STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Config(ct.Structure):
    _fields_ = [
        ("num_leaves", ct.c_uint32),
        ("num_patterns", ct.c_uint32),
        ("num_states", ct.c_uint32),
        ("num_categories", ct.c_uint32),
        ("precision", ct.c_uint32),
        ("scale_ln", ct.c_uint32),
        ("device", ct.c_int32),
        ("reserved", ct.c_uint32),
    ]


class PruneBuffers(ct.Structure):
    """b3g_prune_buffers: device pointers and sizes for b3g_prune_noalloc."""

    _fields_ = [
        ("tips", ct.c_void_p),
        ("partials", ct.c_void_p),
        ("scales", ct.c_void_p),
        ("ops", ct.c_void_p),
        ("tables", ct.c_void_p),
        ("frequencies", ct.c_void_p),
        ("weights", ct.c_void_p),
        ("site_lnl", ct.c_void_p),
        ("lnl", ct.c_void_p),
        ("n", ct.c_uint32),
        ("ldp", ct.c_uint32),
        ("num_categories", ct.c_uint32),
        ("precision", ct.c_uint32),
        ("scale_ln", ct.c_uint32),
        ("reserved", ct.c_uint32),
    ]


OP_COUNT = 14


class McmcConfig(ct.Structure):
    """b3g_mcmc_config."""

    _fields_ = [
        ("num_chains", ct.c_uint32),
        ("num_categories", ct.c_uint32),
        ("precision", ct.c_uint32),
        ("model", ct.c_uint32),
        ("seed", ct.c_uint64),
        ("heat", ct.c_double),
        ("swap_every", ct.c_uint32),
        ("sample_every", ct.c_uint32),
        ("tune_every", ct.c_uint32),
        ("device", ct.c_int32),
        ("op_weights", ct.c_double * OP_COUNT),
        ("da_pilot_steps", ct.c_uint32),
        ("da_epochs", ct.c_uint32),
        ("da_hidden", ct.c_uint32),
        ("da_reserved", ct.c_uint32),
        ("da_drift_limit", ct.c_double),
        ("clock_categories", ct.c_uint32),
        ("launch", ct.c_uint32),
        ("host_threads", ct.c_uint32),
    ]


class McmcProblem(ct.Structure):
    """b3g_mcmc_problem."""

    _fields_ = [
        ("num_leaves", ct.c_uint32),
        ("num_patterns", ct.c_uint32),
        ("samples", ct.c_void_p),
        ("weights", ct.c_void_p),
        ("parents", ct.c_void_p),
        ("heights", ct.c_void_p),
    ]


NOALLOC_MAX_BLOCKS = 16384
TIP = 0x80000000

_u8p = ct.POINTER(ct.c_uint8)
_u32p = ct.POINTER(ct.c_uint32)
_f64p = ct.POINTER(ct.c_double)
_f32p = ct.POINTER(ct.c_float)
_vp = ct.c_void_p

# name -> (restype, argtypes); every function declared in include/b3g.h
SIGNATURES = {
    "b3g_last_error": (ct.c_char_p, []),
    "b3g_version": (ct.c_char_p, []),
    "b3g_calculator_create": (ct.c_int, [ct.POINTER(Config), _u8p, ct.POINTER(_vp)]),
    "b3g_calculator_destroy": (None, [_vp]),
    "b3g_calculator_num_patterns": (ct.c_uint32, [_vp]),
    "b3g_calculator_propose": (ct.c_int, [_vp, _u32p, _u32p, ct.c_uint32, _f64p, _f64p]),
    "b3g_calculator_likelihoods": (ct.c_int, [_vp, _f64p]),
    "b3g_calculator_accept": (ct.c_int, [_vp]),
    "b3g_calculator_reject": (ct.c_int, [_vp]),
    "b3g_calculator_set_weights": (ct.c_int, [_vp, _u32p]),
    "b3g_calculator_set_eigen": (ct.c_int, [_vp, _f64p, _f64p, _f64p, _f64p, _f64p, ct.c_int]),
    "b3g_calculator_set_reversible": (ct.c_int, [_vp, _f64p, _f64p, ct.c_int]),
    "b3g_calculator_set_category_rates": (ct.c_int, [_vp, _f64p]),
    "b3g_calculator_set_gamma": (ct.c_int, [_vp, ct.c_double]),
    # per-step calls take plain addresses (see addr): cheaper from Python
    "b3g_calculator_propose_lengths": (
        ct.c_int, [_vp, _vp, _vp, ct.c_uint32, _vp, ct.c_double]),
    "b3g_calculator_log_likelihood": (ct.c_int, [_vp, _f64p]),
    "b3g_mcmc_samples": (ct.c_int, [_vp, ct.POINTER(ct.c_uint64), _u32p, _f64p, _f64p,
                                    ct.c_uint64, ct.POINTER(ct.c_uint64)]),
    "b3g_mcmc_set_clock": (ct.c_int, [_vp, ct.c_double, _u32p]),
    "b3g_lognormal_categories": (ct.c_int, [ct.c_double, ct.c_uint32, _f64p]),
    "b3g_deduplicate": (ct.c_int, [_u8p, ct.c_uint32, ct.c_uint32, ct.c_int, ct.c_int32,
                                   _u8p, _u32p, _u32p, _u32p, _f32p]),
    "b3g_hetero_create": (ct.c_int, [ct.POINTER(_vp), ct.c_uint32, ct.POINTER(_vp)]),
    "b3g_hetero_destroy": (None, [_vp]),
    "b3g_hetero_set_classes": (ct.c_int, [_vp, _u32p]),
    "b3g_hetero_log_likelihood": (ct.c_int, [_vp, _f64p]),
    "b3g_hetero_accept": (ct.c_int, [_vp]),
    "b3g_hetero_reject": (ct.c_int, [_vp]),
    "b3g_calculator_autotune": (
        ct.c_int, [_vp, _u32p, _u32p, ct.c_uint32, _f64p, ct.c_double, _u32p]),
    "b3g_calculator_site_log_likelihoods": (ct.c_int, [_vp, _f64p]),
    "b3g_calculator_set_timing": (ct.c_int, [_vp, ct.c_int]),
    "b3g_calculator_last_timing": (ct.c_int, [_vp, _f32p, _f32p]),
    "b3g_calculator_timing_totals": (
        ct.c_int, [_vp, ct.c_int, _f64p, _f64p, ct.POINTER(ct.c_uint64)]),
    "b3g_calculator_last_upload_bytes": (ct.c_int, [_vp, ct.POINTER(ct.c_uint64)]),
    "b3g_calculator_last_launches": (ct.c_int, [_vp, _u32p]),
    "b3g_calculator_span_begin": (ct.c_int, [_vp]),
    "b3g_calculator_span_end": (ct.c_int, [_vp, _f32p]),
    "b3g_prune_noalloc": (ct.c_int, [ct.POINTER(PruneBuffers), _vp]),
    "b3g_surrogate_create": (ct.c_int, [ct.c_uint32, ct.c_uint32, ct.c_uint64, ct.c_int32,
                                        ct.POINTER(_vp)]),
    "b3g_surrogate_destroy": (None, [_vp]),
    "b3g_surrogate_num_params": (ct.c_uint32, [_vp]),
    "b3g_surrogate_get_params": (ct.c_int, [_vp, _f32p]),
    "b3g_surrogate_set_params": (ct.c_int, [_vp, _f32p]),
    "b3g_surrogate_forward": (ct.c_int, [_vp, _f32p, ct.c_uint32, _f32p]),
    "b3g_surrogate_loss_grad": (ct.c_int, [_vp, _f32p, _f32p, _f32p, ct.c_uint32, _f32p,
                                           _f32p]),
    "b3g_surrogate_train": (ct.c_int, [_vp, _f32p, _f32p, _f32p, ct.c_uint32, ct.c_uint32,
                                       ct.c_uint32, ct.c_float, ct.c_uint64, _f32p]),
    "b3g_surrogate_delta": (ct.c_int, [_vp, _f32p, _f32p, _f32p]),
    "b3g_surrogate_deltas": (ct.c_int, [_vp, _f32p, _f32p, ct.c_uint32, _f32p]),
    "b3g_batch_create": (ct.c_int, [ct.POINTER(_vp), ct.c_uint32, ct.POINTER(_vp)]),
    "b3g_batch_destroy": (None, [_vp]),
    "b3g_calculator_stage_lengths": (
        ct.c_int, [_vp, _vp, _vp, ct.c_uint32, _vp, ct.c_double]),
    "b3g_batch_run": (ct.c_int, [_vp]),
    "b3g_batch_log_likelihoods": (ct.c_int, [_vp, _f64p]),
    "b3g_batch_last_ms": (ct.c_int, [_vp, _f32p]),
    "b3g_mcmc_set_tuning": (ct.c_int, [_vp, ct.c_uint32, ct.c_double]),
    "b3g_mcmc_create": (ct.c_int, [ct.POINTER(McmcConfig), ct.c_uint32, ct.c_uint32, _u8p,
                                   _u32p, _u32p, _f64p, ct.POINTER(_vp)]),
    "b3g_mcmc_destroy": (None, [_vp]),
    "b3g_mcmc_create_multi": (ct.c_int, [ct.POINTER(McmcConfig), ct.c_uint32,
                                         ct.POINTER(McmcProblem), ct.POINTER(_vp)]),
    "b3g_mcmc_launch_stats": (ct.c_int, [_vp, ct.POINTER(ct.c_uint32),
                                         ct.POINTER(ct.c_double), ct.POINTER(ct.c_uint64)]),
    "b3g_mcmc_set_parameters": (ct.c_int, [_vp, ct.c_double, _f64p, _f64p, ct.c_double,
                                           ct.c_double]),
    "b3g_mcmc_run": (ct.c_int, [_vp, ct.c_uint64]),
    "b3g_mcmc_trace": (ct.c_int, [_vp, ct.c_uint32, _f64p, ct.c_uint64,
                                  ct.POINTER(ct.c_uint64)]),
    "b3g_mcmc_chain_trace": (ct.c_int, [_vp, ct.c_uint32, ct.c_uint32, _f64p, ct.c_uint64,
                                        ct.POINTER(ct.c_uint64)]),
    "b3g_mcmc_operator_stats": (ct.c_int, [_vp, ct.c_uint32, ct.POINTER(ct.c_uint64), _f64p]),
    "b3g_mcmc_swaps": (ct.c_int, [_vp, ct.POINTER(ct.c_uint64), ct.POINTER(ct.c_uint64)]),
    "b3g_mcmc_dump": (ct.c_int, [_vp, _u8p, ct.c_uint64, ct.POINTER(ct.c_uint64)]),
    "b3g_mcmc_load": (ct.c_int, [_vp, _u8p, ct.c_uint64]),
    "b3g_mcmc_dump_verbatim": (ct.c_int, [_vp, ct.c_uint32, _u32p, ct.c_uint32, _u32p,
                                          ct.c_uint32, _u8p, ct.c_uint64,
                                          ct.POINTER(ct.c_uint64)]),
    "b3g_mcmc_load_verbatim": (ct.c_int, [_vp, ct.c_uint32, _u32p, ct.c_uint32, _u32p,
                                          ct.c_uint32, _u8p, ct.c_uint64]),
    "b3g_mcmc_check": (ct.c_int, [_vp, _f64p]),
    "b3g_mcmc_da_stats": (ct.c_int, [_vp, ct.POINTER(ct.c_uint64), _f64p]),
    "b3g_mcmc_chain_state": (ct.c_int, [_vp, ct.c_uint32, _u32p, _f64p, _f64p, _f64p]),
    "b3g_create": (ct.c_int, [ct.POINTER(Config), _u8p, _u32p, ct.c_uint32, ct.POINTER(_vp)]),
    "b3g_destroy": (None, [_vp]),
    "b3g_set_model": (ct.c_int, [_vp, ct.c_uint32, ct.c_uint32, _f64p, _f64p, _f64p, _f64p,
                                 _f64p, ct.c_uint32]),
    "b3g_set_tree": (ct.c_int, [_vp, ct.c_uint32, _u32p, _f64p, ct.c_double]),
    "b3g_mark_edges": (ct.c_int, [_vp, ct.c_uint32, _u32p, ct.c_uint32]),
    "b3g_mark_all": (ct.c_int, [_vp, ct.c_uint32]),
    "b3g_propose": (ct.c_int, [_vp, ct.c_uint64]),
    "b3g_wait": (ct.c_int, [_vp]),
    "b3g_lnl": (ct.c_int, [_vp, ct.c_uint32, _f64p]),
    "b3g_site_lnl": (ct.c_int, [_vp, ct.c_uint32, _f64p]),
    "b3g_accept": (ct.c_int, [_vp, ct.c_uint32]),
    "b3g_reject": (ct.c_int, [_vp, ct.c_uint32]),
}


def _load() -> ct.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -m aspartik_gb300.build` "
            "(the GPU library is the only compute path; there is no fallback)")
    lib = ct.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(status: int) -> None:
    if status != B3G_OK:
        raise B3GError(status, lib.b3g_last_error().decode())


def as_ptr(arr: np.ndarray, ctype):
    return arr.ctypes.data_as(ct.POINTER(ctype))


def arr_addr(a, dtype) -> tuple:
    """(array, address of its data): `a` itself when it already is a
    C-contiguous array of `dtype` (no copy), else a converted copy.  The
    address comes from a ctypes view of the buffer, a fraction of the cost of
    ``arr.ctypes.data`` on the per-proposal path."""
    if type(a) is not np.ndarray or a.dtype != dtype or not a.flags.c_contiguous:
        a = np.ascontiguousarray(a, dtype=dtype)
    if a.flags.writeable and a.size:
        return a, ct.addressof(ct.c_char.from_buffer(a))
    return a, a.ctypes.data


def addr(arr: np.ndarray) -> int:
    """Address of a contiguous array's data, for void-pointer arguments
    (about half the cost of as_ptr per call)."""
    return arr.ctypes.data


def u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def u8(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint8)
