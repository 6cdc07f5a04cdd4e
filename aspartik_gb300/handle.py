"""Tree-level handle: ``b3g_create`` / ``b3g_set_tree`` / ``b3g_mark_edges``
/ ``b3g_propose`` / ``b3g_lnl`` / ``b3g_accept`` ... (``include/b3g.h``).

The library mirrors each chain's tree and builds the dirty list itself, as
b3's ``DatedTree::partials_lists`` does (crates/b3/src/parameters/
tree.rs:357-461); the caller only loads the tree state and marks the edges
its move changed, as b3's MCMC does before asking the likelihood
(likelihood/dna.rs:68-124, likelihood/gamma.rs:97-169).
"""

from __future__ import annotations

import ctypes as ct

import numpy as np

from . import _native as nat
from ._native import check, lib

TOMBSTONE = 0xFFFFFFFF


class Handle:
    """``num_chains`` chains (1..64) over one deduplicated alignment
    ``samples`` [L][P] (4-bit codes, as ``b3g_calculator_create``) with
    pattern ``weights``; one calculator and CUDA stream per chain."""

    def __init__(self, samples: np.ndarray, weights, num_chains: int = 1, *, device: int = 0,
                 precision: str = "f64", num_categories: int = 1, scale_ln: int = 30,
                 num_states: int = 4):
        samples = nat.u8(samples)
        if samples.ndim != 2:
            raise ValueError("samples must be [num_leaves][num_patterns]")
        L, P = samples.shape
        self.num_leaves, self.num_patterns = L, P
        self.num_categories, self.num_states = num_categories, num_states
        self.num_chains = num_chains
        cfg = nat.Config(L, P, num_states, num_categories,
                         nat.PRECISION_F32 if precision == "f32" else nat.PRECISION_F64,
                         scale_ln, device, 0)
        w = nat.u32(weights)
        if w.size != P:
            raise ValueError("one weight per pattern")
        self._h = ct.c_void_p()
        check(lib.b3g_create(ct.byref(cfg), nat.as_ptr(samples, ct.c_uint8),
                             nat.as_ptr(w, ct.c_uint32), num_chains, ct.byref(self._h)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib.b3g_destroy(self._h)
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

    def set_model(self, chain: int, V, Vinv, lam, pi, cat_rates) -> None:
        S, C = self.num_states, self.num_categories
        V, Vinv, lam, pi, cr = (nat.f64(a).reshape(-1) for a in (V, Vinv, lam, pi, cat_rates))
        if V.size != S * S or Vinv.size != S * S or lam.size != S or pi.size != S \
                or cr.size != C:
            raise ValueError("model arrays of the wrong size")
        check(lib.b3g_set_model(self._h, chain, S, nat.as_ptr(V, ct.c_double),
                                nat.as_ptr(Vinv, ct.c_double), nat.as_ptr(lam, ct.c_double),
                                nat.as_ptr(pi, ct.c_double), nat.as_ptr(cr, ct.c_double), C))

    def set_tree(self, chain: int, parents, heights, clock_rate: float = 1.0) -> None:
        """parents[2L-1] with the root's entry 0xFFFFFFFF, heights[2L-1]."""
        n = 2 * self.num_leaves - 1
        parents = nat.u32(parents)
        heights = nat.f64(heights)
        if parents.size != n or heights.size != n:
            raise ValueError("parents and heights need 2L-1 entries")
        check(lib.b3g_set_tree(self._h, chain, nat.as_ptr(parents, ct.c_uint32),
                               nat.as_ptr(heights, ct.c_double), float(clock_rate)))

    def mark_edges(self, chain: int, edges) -> None:
        e = nat.u32(edges).reshape(-1)
        check(lib.b3g_mark_edges(self._h, chain, nat.as_ptr(e, ct.c_uint32), e.size))

    def mark_all(self, chain: int) -> None:
        check(lib.b3g_mark_all(self._h, chain))

    def propose(self, chains=None) -> None:
        """Evaluate the given chains (all by default), asynchronously."""
        if chains is None:
            mask = (1 << self.num_chains) - 1
        else:
            mask = 0
            for c in chains:
                mask |= 1 << int(c)
        check(lib.b3g_propose(self._h, ct.c_uint64(mask)))

    def wait(self) -> None:
        check(lib.b3g_wait(self._h))

    def lnl(self, chain: int) -> float:
        out = ct.c_double()
        check(lib.b3g_lnl(self._h, chain, ct.byref(out)))
        return out.value

    def site_lnl(self, chain: int) -> np.ndarray:
        out = np.empty(self.num_patterns, dtype=np.float64)
        check(lib.b3g_site_lnl(self._h, chain, nat.as_ptr(out, ct.c_double)))
        return out

    def accept(self, chain: int) -> None:
        check(lib.b3g_accept(self._h, chain))

    def reject(self, chain: int) -> None:
        check(lib.b3g_reject(self._h, chain))
