"""Python face of the GB300 pruning calculator.

Mirrors the reference's calculator interface (crates/b3/src/calculator/
mod.rs): ``Calculator`` is the configuration object that Python builds
(``Calculator.CPU()``, ``.CUDAPartials()``, ``.with_scale()``, mod.rs:101-156)
and ``make4`` turns into a live calculator (mod.rs:159-200); the live object
has the trait's methods ``propose / likelihoods / accept / reject /
num_patterns`` (mod.rs:54-76).  All work happens in ``libb3g.so``.
"""

from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _native as nat
from ._native import B3GError, check, lib

PRECISIONS = {"f64": nat.PRECISION_F64, "f32": nat.PRECISION_F32}


class Calculator:
    """Calculator configuration (``CalculatorConfig``, calculator/mod.rs:94-156)."""

    def __init__(self, device: int = 0, precision: str = "f64", scale_ln: int = 30):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        self.device = int(device)
        self.precision = precision
        self.scale_ln = int(scale_ln)

    @classmethod
    def GB300(cls, device: int = 0, precision: str = "f64") -> "Calculator":
        """The sm_103a calculator.  ``precision="f64"`` is the plain form
        (FP64 partials, e^scale_ln rescaling, as ``Calculator.CPU``);
        ``"f32"`` is the chosen form (FP32 partials with exact power-of-two
        rescaling)."""
        return cls(device=device, precision=precision)

    def with_scale(self, scale_ln: int) -> "Calculator":
        """``CalculatorConfig::with_scale`` (calculator/mod.rs:149-155)."""
        self.scale_ln = int(scale_ln)
        return self

    def make4(self, samples: np.ndarray, num_patterns: int,
              num_categories: int = 1) -> "GpuCalculator":
        """``CalculatorConfig::make4`` (calculator/mod.rs:159-200)."""
        return GpuCalculator(samples, num_patterns, device=self.device,
                             precision=self.precision, scale_ln=self.scale_ln,
                             num_categories=num_categories)

    def make20(self, samples: np.ndarray, num_patterns: int,
               num_categories: int = 1) -> "GpuCalculator":
        """20-state (protein) counterpart of ``make4``; the reference has no
        20-state calculator.  ``samples`` are state indices 0..19, any other
        code is unknown; at most 8 categories."""
        return GpuCalculator(samples, num_patterns, device=self.device,
                             precision=self.precision, scale_ln=self.scale_ln,
                             num_categories=num_categories, num_states=20)


class GpuCalculator:
    """A device-resident pruning store for one alignment and one chain."""

    def __init__(self, samples: np.ndarray, num_patterns: int, *, device: int = 0,
                 precision: str = "f64", scale_ln: int = 30, num_categories: int = 1,
                 num_states: int = 4):
        samples = nat.u8(samples).reshape(-1)
        if num_patterns <= 0 or samples.size % num_patterns:
            raise ValueError("samples must hold num_leaves * num_patterns codes")
        self.num_leaves = samples.size // num_patterns
        self._P = int(num_patterns)
        self.num_categories = int(num_categories)
        self.num_states = int(num_states)
        cfg = nat.Config(self.num_leaves, self._P, num_states, self.num_categories,
                         PRECISIONS[precision], int(scale_ln), int(device), 0)
        handle = ct.c_void_p()
        check(lib.b3g_calculator_create(ct.byref(cfg), nat.as_ptr(samples, ct.c_uint8),
                                        ct.byref(handle)))
        self._h = handle

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.b3g_calculator_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- trait Calculator<f64> -------------------------------------------
    def num_patterns(self) -> int:
        return int(lib.b3g_calculator_num_patterns(self._h))

    def propose(self, internals, children, matrices, frequencies) -> None:
        internals = nat.u32(internals)
        children = nat.u32(children).reshape(-1)
        n = internals.size
        matrices = nat.f64(matrices).reshape(-1)
        expected = n * 2 * self.num_categories * self.num_states ** 2
        if matrices.size != expected:
            raise ValueError(f"matrices must hold {expected} values")
        if children.size != 2 * n:
            raise ValueError("children must hold two ids per internal")
        freqs = nat.f64(frequencies)
        check(lib.b3g_calculator_propose(self._h, nat.as_ptr(internals, ct.c_uint32),
                                         nat.as_ptr(children, ct.c_uint32), n,
                                         nat.as_ptr(matrices, ct.c_double),
                                         nat.as_ptr(freqs, ct.c_double)))

    def likelihoods(self) -> np.ndarray:
        out = np.empty((self.num_categories, self._P), dtype=np.float64)
        check(lib.b3g_calculator_likelihoods(self._h, nat.as_ptr(out, ct.c_double)))
        return out[0] if self.num_categories == 1 else out

    def accept(self) -> None:
        check(lib.b3g_calculator_accept(self._h))

    def reject(self) -> None:
        check(lib.b3g_calculator_reject(self._h))

    # -- likelihood level ---------------------------------------------------
    def set_weights(self, weights) -> None:
        w = nat.u32(weights)
        if w.size != self._P:
            raise ValueError("one weight per pattern")
        check(lib.b3g_calculator_set_weights(self._h, nat.as_ptr(w, ct.c_uint32)))

    def set_eigen(self, V, Vinv, lam, Q, pi, shortcuts: bool = True) -> None:
        V, Vinv, lam, Q, pi = (nat.f64(x).reshape(-1) for x in (V, Vinv, lam, Q, pi))
        check(lib.b3g_calculator_set_eigen(
            self._h, nat.as_ptr(V, ct.c_double), nat.as_ptr(Vinv, ct.c_double),
            nat.as_ptr(lam, ct.c_double), nat.as_ptr(Q, ct.c_double),
            nat.as_ptr(pi, ct.c_double), int(bool(shortcuts))))

    def set_reversible(self, rates, pi, shortcuts: bool = True) -> None:
        r, pi = nat.f64(rates), nat.f64(pi)
        s = self.num_states
        if r.size != s * (s - 1) // 2 or pi.size != s:
            raise ValueError("rates need S(S-1)/2 values and pi S values")
        check(lib.b3g_calculator_set_reversible(self._h, nat.as_ptr(r, ct.c_double),
                                                nat.as_ptr(pi, ct.c_double),
                                                int(bool(shortcuts))))

    def set_category_rates(self, rates) -> None:
        r = nat.f64(rates)
        if r.size != self.num_categories:
            raise ValueError("one rate per category")
        check(lib.b3g_calculator_set_category_rates(self._h, nat.as_ptr(r, ct.c_double)))

    def set_gamma(self, alpha: float) -> None:
        check(lib.b3g_calculator_set_gamma(self._h, float(alpha)))

    def propose_lengths(self, internals, children, lengths, clock_rate: float = 1.0) -> None:
        internals, pi = nat.arr_addr(internals, np.uint32)
        children, pc = nat.arr_addr(children, np.uint32)
        lengths, pl = nat.arr_addr(lengths, np.float64)
        n = internals.size
        if children.size != 2 * n or lengths.size != 2 * n:
            raise ValueError("children and lengths need two values per internal")
        check(lib.b3g_calculator_propose_lengths(self._h, pi, pc, n, pl, float(clock_rate)))

    def autotune(self, internals, children, lengths, clock_rate: float = 1.0) -> int:
        """Time the list with each launch configuration of this form and keep
        the fastest (no counterpart in the reference); returns the patterns
        per tile (4 states), 1 / 0 for tensor / CUDA cores (20 states), 0 for
        the FP64 form.  Trial proposals are rejected: call between steps."""
        internals = nat.u32(internals)
        children = nat.u32(children).reshape(-1)
        lengths = nat.f64(lengths).reshape(-1)
        n = internals.size
        if children.size != 2 * n or lengths.size != 2 * n:
            raise ValueError("children and lengths need two values per internal")
        out = ct.c_uint32()
        check(lib.b3g_calculator_autotune(
            self._h, nat.as_ptr(internals, ct.c_uint32), nat.as_ptr(children, ct.c_uint32),
            n, nat.as_ptr(lengths, ct.c_double), float(clock_rate), ct.byref(out)))
        return int(out.value)

    def log_likelihood(self) -> float:
        out = ct.c_double()
        check(lib.b3g_calculator_log_likelihood(self._h, ct.byref(out)))
        return out.value

    def site_log_likelihoods(self) -> np.ndarray:
        out = np.empty(self._P, dtype=np.float64)
        check(lib.b3g_calculator_site_log_likelihoods(self._h, nat.as_ptr(out, ct.c_double)))
        return out

    def set_timing(self, on: bool = True) -> None:
        """CUDA events around every evaluation (for last_timing /
        timing_totals); off by default."""
        check(lib.b3g_calculator_set_timing(self._h, 1 if on else 0))

    def last_timing(self) -> tuple[float, float]:
        """(transition-kernel ms, pruning-kernel ms) of the last proposal."""
        t, p = ct.c_float(), ct.c_float()
        check(lib.b3g_calculator_last_timing(self._h, ct.byref(t), ct.byref(p)))
        return t.value, p.value

    def timing_totals(self, reset: bool = False) -> tuple[float, float, int]:
        """(transition ms, pruning ms, proposals) summed since the last reset."""
        t, p, n = ct.c_double(), ct.c_double(), ct.c_uint64()
        check(lib.b3g_calculator_timing_totals(self._h, int(bool(reset)), ct.byref(t),
                                               ct.byref(p), ct.byref(n)))
        return t.value, p.value, int(n.value)

    def last_upload_bytes(self) -> int:
        """Bytes the last proposal copied host -> device."""
        n = ct.c_uint64()
        check(lib.b3g_calculator_last_upload_bytes(self._h, ct.byref(n)))
        return int(n.value)

    def last_launches(self) -> int:
        """Kernels the last evaluation launched."""
        n = ct.c_uint32()
        check(lib.b3g_calculator_last_launches(self._h, ct.byref(n)))
        return int(n.value)

    def span_begin(self) -> None:
        check(lib.b3g_calculator_span_begin(self._h))

    def span_end(self) -> float:
        ms = ct.c_float()
        check(lib.b3g_calculator_span_end(self._h, ct.byref(ms)))
        return ms.value


def _stage_lengths(self, internals, children, lengths, clock_rate: float = 1.0) -> None:
    """Stage a dirty-path evaluation for this calculator's batch (no launch)."""
    internals = nat.u32(internals)
    children = nat.u32(children).reshape(-1)
    lengths = nat.f64(lengths).reshape(-1)
    n = internals.size
    if children.size != 2 * n or lengths.size != 2 * n:
        raise ValueError("children and lengths need two values per internal")
    check(lib.b3g_calculator_stage_lengths(
        self._h, nat.addr(internals), nat.addr(children), n, nat.addr(lengths),
        float(clock_rate)))


GpuCalculator.stage_lengths = _stage_lengths


class Batch:
    """Many FP32 calculators evaluated by one graph-replayed launch."""

    def __init__(self, members: list):
        self.members = list(members)
        arr = (ct.c_void_p * len(self.members))(*[m._h.value for m in self.members])
        h = ct.c_void_p()
        check(lib.b3g_batch_create(arr, len(self.members), ct.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.b3g_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self) -> None:
        check(lib.b3g_batch_run(self._h))

    def log_likelihoods(self) -> np.ndarray:
        out = np.empty(len(self.members))
        check(lib.b3g_batch_log_likelihoods(self._h, nat.as_ptr(out, ct.c_double)))
        return out

    def last_ms(self) -> float:
        ms = ct.c_float()
        check(lib.b3g_batch_last_ms(self._h, ct.byref(ms)))
        return ms.value


def deduplicate(msa: np.ndarray, dna: bool = True, device: int = 0):
    """Site-pattern compression on the GPU (``deduplicate``,
    likelihood/mod.rs:74-132): returns (leaves [L][P], weights [P],
    site_to_pattern [N], device milliseconds)."""
    msa = np.ascontiguousarray(msa, dtype=np.uint8)
    L, N = msa.shape
    leaves = np.empty(L * N, dtype=np.uint8)
    weights = np.empty(N, dtype=np.uint32)
    s2p = np.empty(N, dtype=np.uint32)
    P = ct.c_uint32()
    ms = ct.c_float()
    check(lib.b3g_deduplicate(nat.as_ptr(msa, ct.c_uint8), L, N, int(bool(dna)), int(device),
                              nat.as_ptr(leaves, ct.c_uint8), nat.as_ptr(weights, ct.c_uint32),
                              nat.as_ptr(s2p, ct.c_uint32), ct.byref(P), ct.byref(ms)))
    p = P.value
    return leaves[: L * p].reshape(L, p).copy(), weights[:p].copy(), s2p, ms.value


class Hetero:
    """Per-pattern class mixture over calculators (``HeteroLikelihood``,
    likelihood/hetero.rs:97-168): class k is member k (its own model and
    clock), pattern p counts under class c(p).  Members must be evaluated and
    accepted before the mixture is built; per step propose the changed
    members and/or ``set_classes``, then ``log_likelihood`` and exactly one of
    ``accept`` / ``reject``."""

    def __init__(self, members: list):
        self.members = list(members)
        arr = (ct.c_void_p * len(self.members))(*[m._h.value for m in self.members])
        h = ct.c_void_p()
        check(lib.b3g_hetero_create(arr, len(self.members), ct.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.b3g_hetero_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_classes(self, classes) -> None:
        c = nat.u32(classes)
        if c.size != self.members[0].num_patterns():
            raise ValueError("one class per pattern")
        check(lib.b3g_hetero_set_classes(self._h, nat.as_ptr(c, ct.c_uint32)))

    def log_likelihood(self) -> float:
        out = ct.c_double()
        check(lib.b3g_hetero_log_likelihood(self._h, ct.byref(out)))
        return out.value

    def accept(self) -> None:
        check(lib.b3g_hetero_accept(self._h))

    def reject(self) -> None:
        check(lib.b3g_hetero_reject(self._h))


__all__ = ["Calculator", "GpuCalculator", "Batch", "Hetero", "deduplicate", "B3GError"]
