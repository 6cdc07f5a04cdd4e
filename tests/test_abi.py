"""The C ABI library without a GPU: it loads, exports every symbol that
include/b3g.h declares, the ctypes table covers all of them, and calls fail
with a status and a message instead of crashing."""

import ctypes as ct
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "b3g.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"B3G_API[^;(]*?\b(b3g_\w+)\s*\(", text, flags=re.S)))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "b3g_calculator_create" in names
    assert "b3g_calculator_propose" in names
    assert len(names) >= 18


def test_library_exports_every_declared_symbol():
    from aspartik_gb300 import _native

    lib = ct.CDLL(str(_native.LIB_PATH))
    for name in declared_symbols():
        assert hasattr(lib, name), f"libb3g.so does not export {name}"
    assert set(declared_symbols()) == set(_native.SIGNATURES), \
        "ctypes signature table and header disagree"


def test_only_declared_symbols_are_exported():
    import subprocess

    from aspartik_gb300 import _native

    out = subprocess.run(["nm", "-D", "--defined-only", str(_native.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    ours = sorted({ln.split()[-1] for ln in out.splitlines() if ln.split()[-1].startswith("b3g_")})
    assert ours == declared_symbols()


def test_version_string():
    from aspartik_gb300._native import lib

    assert b"sm_103a" in lib.b3g_version()


def test_create_rejects_bad_config_without_touching_a_gpu():
    from aspartik_gb300 import _native as nat

    handle = ct.c_void_p()
    samples = np.ones(8, dtype=np.uint8)
    cfg = nat.Config(1, 8, 4, 1, 0, 30, 0, 0)  # one leaf: invalid
    st = nat.lib.b3g_calculator_create(ct.byref(cfg), nat.as_ptr(samples, ct.c_uint8),
                                       ct.byref(handle))
    assert st == nat.B3G_ERR_INVALID_ARGUMENT
    assert b"num_leaves" in nat.lib.b3g_last_error()
    cfg = nat.Config(2, 4, 5, 1, 0, 30, 0, 0)  # 5 states: unsupported
    st = nat.lib.b3g_calculator_create(ct.byref(cfg), nat.as_ptr(samples, ct.c_uint8),
                                       ct.byref(handle))
    assert st == nat.B3G_ERR_INVALID_ARGUMENT


def test_null_handles_are_reported():
    from aspartik_gb300 import _native as nat

    assert nat.lib.b3g_calculator_accept(None) == nat.B3G_ERR_INVALID_ARGUMENT
    assert nat.lib.b3g_calculator_num_patterns(None) == 0
    nat.lib.b3g_calculator_destroy(None)  # no-op


def test_no_gpu_reports_cuda_error():
    """On a machine without a GPU, construction fails with a CUDA status."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from aspartik_gb300 import _native as nat

    handle = ct.c_void_p()
    samples = np.ones(8, dtype=np.uint8)
    cfg = nat.Config(2, 4, 4, 1, 0, 30, 0, 0)
    st = nat.lib.b3g_calculator_create(ct.byref(cfg), nat.as_ptr(samples, ct.c_uint8),
                                       ct.byref(handle))
    assert st in (nat.B3G_ERR_CUDA, nat.B3G_ERR_INVALID_ARGUMENT)
    assert nat.lib.b3g_last_error()


def test_array_addresses_for_per_call_arguments():
    """nat.arr_addr: an array already C-contiguous of the asked type comes
    back as itself (no copy) with its data address; anything else is
    converted first; read-only and empty arrays take the ctypes path."""
    from aspartik_gb300 import _native as nat

    a = np.arange(10, dtype=np.uint32)
    same, p = nat.arr_addr(a, np.uint32)
    assert same is a and p == a.ctypes.data
    b = np.arange(20, dtype=np.int64)[::2]
    conv, q = nat.arr_addr(b, np.uint32)
    assert conv is not b and conv.dtype == np.uint32 and conv.flags.c_contiguous
    assert q == conv.ctypes.data and list(conv) == list(range(0, 20, 2))
    m = np.arange(6, dtype=np.float64).reshape(3, 2)
    same2, r = nat.arr_addr(m, np.float64)
    assert same2 is m and r == m.ctypes.data
    ro = np.arange(4, dtype=np.float64)
    ro.flags.writeable = False
    got, s = nat.arr_addr(ro, np.float64)
    assert got is ro and s == ro.ctypes.data
    empty, _ = nat.arr_addr([], np.uint32)
    assert empty.size == 0


def test_mcmc_settings_fill_the_c_config():
    """McmcSettings -> b3g_mcmc_config: operator weights by name, the launch
    mode (independent stepping = 2) and the host thread count land in the
    struct's fields, and an unknown operator name is refused."""
    from aspartik_gb300 import _native as nat
    from aspartik_gb300.mcmc import OPERATORS, McmcSettings, _config

    s = McmcSettings(model="hky", precision="f64", num_categories=1, num_chains=8,
                     weights={"tree_scale": 3, "scale_kappa": 1, "node_slide": 2},
                     launch="independent", host_threads=5, da_pilot_steps=100,
                     clock_categories=4)
    c = _config(s)
    assert c.num_chains == 8 and c.num_categories == 1 and c.model == 0
    assert c.precision == nat.PRECISION_F64
    assert c.launch == 2 and c.host_threads == 5
    assert c.da_pilot_steps == 100 and c.clock_categories == 4 and c.da_reserved == 0
    w = list(c.op_weights)
    assert w[OPERATORS.index("tree_scale")] == 3 and w[OPERATORS.index("node_slide")] == 2
    assert sum(w) == 6
    with pytest.raises(ValueError):
        _config(McmcSettings(weights={"no_such_move": 1}))
