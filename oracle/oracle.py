"""CPU oracle of the b3 pruning likelihood.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module, and only as the checker or the timed baseline.

It wraps ``libb3oracle.so`` (b3oracle.c, the C restatement of
crates/b3/src/calculator/cpu4.rs, substitution.rs and gamma.rs) and restates
in Python the host-side orchestration around it:

* ``DatedTree``       parameters/tree.rs:32-1017 (dirty tracking, moves,
                      accept/reject)
* ``Transitions``     transitions.rs:6-73 with sk_slice_buf.rs:8-47
* ``DnaLikelihood``   likelihood/dna.rs:17-124
* ``GammaLikelihood`` likelihood/gamma.rs:20-225
* substitution models JC, K80, HKY, GTR (substitution.rs:102-604)

Parity status: pinned against values produced by the reference itself.
The reference's Rust CPU pruner cannot be built here (no Rust toolchain,
an un-vendored git dependency), but the kernels of its two FP64 CUDA
calculators (crates/b3/src/calculator/cuda_partials/kernels.cu and
cuda_propagations/kernels.cu) are compiled from the reference tree into
oracle/_ref (oracle/build.py::build_ref) and run on a GB300
(oracle/ref_cuda.py): their per-pattern log-likelihoods, stored with their
inputs in tests/golden/ref_cuda_partials.npz, are reproduced by this
restatement to 1e-12 relative (tests/test_ref_golden.py; the live kernels
in tests/test_reference_cuda_gpu.py).  Also pinned against closed forms,
scipy's expm, scipy's gammaincinv and brute-force enumeration
(oracle/brute.py); the Gamma quantile of the reference's un-vendored
computare-distributions stays unpinned (scipy stands in for it).
"""

from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
TOMBSTONE = 0xFFFFFFFF

_u8p = ct.POINTER(ct.c_uint8)
_u32p = ct.POINTER(ct.c_uint32)
_f64p = ct.POINTER(ct.c_double)


def _load():
    from . import build as _build

    path = _build.build()
    lib = ct.CDLL(str(path))
    sig = {
        "orc_cpu4_new": (ct.c_void_p, [ct.c_size_t, _u8p, ct.c_size_t, ct.c_uint32, ct.c_size_t]),
        "orc_cpu4_free": (None, [ct.c_void_p]),
        "orc_cpu4_propose": (None, [ct.c_void_p, _u32p, _u32p, ct.c_size_t, _f64p, _f64p]),
        "orc_cpu4_likelihoods": (_f64p, [ct.c_void_p]),
        "orc_cpu4_accept": (None, [ct.c_void_p]),
        "orc_cpu4_reject": (None, [ct.c_void_p]),
        "orc_cpu4_num_patterns": (ct.c_size_t, [ct.c_void_p]),
        "orc_cpu4_num_threads": (ct.c_size_t, [ct.c_void_p]),
        "orc_deduplicate": (ct.c_size_t, [_u8p, ct.c_size_t, ct.c_size_t, _u8p, _u32p, _u32p]),
        "orc_weighted_sum": (ct.c_double, [_f64p, _u32p, ct.c_size_t]),
        "orc_log_sum_exp": (ct.c_double, [_f64p, ct.c_size_t]),
        "orc_jc_transition": (None, [ct.c_double, _f64p]),
        "orc_k80_transition": (None, [ct.c_double, ct.c_double, _f64p]),
        "orc_hky_eigen": (None, [ct.c_double, _f64p, _f64p, _f64p, _f64p, _f64p]),
        "orc_gtr_q": (None, [_f64p, _f64p, _f64p]),
        "orc_reversible_q": (None, [ct.c_int, _f64p, _f64p, _f64p]),
        "orc_reversible_eigen": (ct.c_int, [ct.c_int, _f64p, _f64p, _f64p, _f64p, _f64p]),
        "orc_eigen_transition": (None, [ct.c_int, _f64p, _f64p, _f64p, _f64p, _f64p,
                                        ct.c_double, ct.c_int, _f64p]),
        "orc_gamma_p": (ct.c_double, [ct.c_double, ct.c_double]),
        "orc_gamma_p_inv": (ct.c_double, [ct.c_double, ct.c_double]),
        "orc_gamma_categories": (None, [ct.c_double, ct.c_int, _f64p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(ct.POINTER(t))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ---------------------------------------------------------------------------
# pruner


class Cpu4Calculator:
    """``Cpu4Calculator`` (calculator/cpu4.rs:12-166) through b3oracle.c."""

    def __init__(self, samples: np.ndarray, num_patterns: int, scale_ln: int = 30,
                 num_threads: int = 0):
        s = np.ascontiguousarray(samples, dtype=np.uint8).reshape(-1)
        self._s = s
        self._h = lib.orc_cpu4_new(num_patterns, _p(s, ct.c_uint8), s.size, scale_ln,
                                   num_threads)
        if not self._h:
            raise ValueError("bad calculator shape")
        self._P = num_patterns

    def __del__(self):
        if getattr(self, "_h", None):
            lib.orc_cpu4_free(self._h)
            self._h = None

    def num_patterns(self) -> int:
        return self._P

    def num_threads(self) -> int:
        return int(lib.orc_cpu4_num_threads(self._h))

    def propose(self, internals, children, matrices, frequencies) -> None:
        internals = np.ascontiguousarray(internals, dtype=np.uint32)
        children = np.ascontiguousarray(children, dtype=np.uint32).reshape(-1)
        m = _f64(matrices).reshape(-1)
        f = _f64(frequencies)
        assert m.size == internals.size * 32
        lib.orc_cpu4_propose(self._h, _p(internals, ct.c_uint32), _p(children, ct.c_uint32),
                             internals.size, _p(m, ct.c_double), _p(f, ct.c_double))

    def likelihoods(self) -> np.ndarray:
        ptr = lib.orc_cpu4_likelihoods(self._h)
        return np.ctypeslib.as_array(ptr, shape=(self._P,)).copy()

    def accept(self) -> None:
        lib.orc_cpu4_accept(self._h)

    def reject(self) -> None:
        lib.orc_cpu4_reject(self._h)


def weighted_sum(values, weights) -> float:
    v, w = _f64(values), np.ascontiguousarray(weights, dtype=np.uint32)
    return lib.orc_weighted_sum(_p(v, ct.c_double), _p(w, ct.c_uint32), v.size)


def log_sum_exp(values) -> float:
    v = _f64(values)
    return lib.orc_log_sum_exp(_p(v, ct.c_double), v.size)


def deduplicate(msa: np.ndarray):
    msa = np.ascontiguousarray(msa, dtype=np.uint8)
    L, N = msa.shape
    leaves = np.zeros(L * N, dtype=np.uint8)
    weights = np.zeros(N, dtype=np.uint32)
    s2p = np.zeros(N, dtype=np.uint32)
    P = lib.orc_deduplicate(_p(msa, ct.c_uint8), L, N, _p(leaves, ct.c_uint8),
                            _p(weights, ct.c_uint32), _p(s2p, ct.c_uint32))
    return leaves[: L * P].reshape(L, P), weights[:P].copy(), s2p


def gamma_categories(alpha: float, k: int) -> np.ndarray:
    out = np.zeros(k)
    lib.orc_gamma_categories(alpha, k, _p(out, ct.c_double))
    return out


def gamma_p_inv(a: float, p: float) -> float:
    return lib.orc_gamma_p_inv(a, p)


# ---------------------------------------------------------------------------
# substitution models (substitution.rs)


class EigenModel:
    """An eigensystem-backed model with the HKY/GTR write_transition
    shortcuts (substitution.rs:403-420, 571-588)."""

    shortcuts = True

    def __init__(self, V, Vinv, lam, Q, pi):
        self.V, self.Vinv, self.lam, self.Q, self.pi = map(_f64, (V, Vinv, lam, Q, pi))
        self.n = self.pi.size

    def transition(self, d: float) -> np.ndarray:
        out = np.zeros(self.n * self.n)
        lib.orc_eigen_transition(self.n, _p(self.V, ct.c_double), _p(self.Vinv, ct.c_double),
                                 _p(self.lam, ct.c_double), _p(self.Q, ct.c_double),
                                 _p(self.pi, ct.c_double), float(d), int(self.shortcuts),
                                 _p(out, ct.c_double))
        return out.reshape(self.n, self.n)

    def frequencies(self) -> np.ndarray:
        return self.pi.copy()


def hky(kappa: float, pi) -> EigenModel:
    pi = _f64(pi)
    V, Vi, lam, Q = (np.zeros(16), np.zeros(16), np.zeros(4), np.zeros(16))
    lib.orc_hky_eigen(kappa, _p(pi, ct.c_double), _p(V, ct.c_double), _p(Vi, ct.c_double),
                      _p(lam, ct.c_double), _p(Q, ct.c_double))
    return EigenModel(V, Vi, lam, Q, pi)


def gtr(rates, pi) -> EigenModel:
    """GTR with the reference's Q (substitution.rs:502-541) decomposed by the
    oracle's Jacobi solver."""
    rates, pi = _f64(rates), _f64(pi)
    Q = np.zeros(16)
    lib.orc_gtr_q(_p(rates, ct.c_double), _p(pi, ct.c_double), _p(Q, ct.c_double))
    return _decompose(Q, pi)


def reversible(rates, pi) -> EigenModel:
    rates, pi = _f64(rates), _f64(pi)
    n = pi.size
    Q = np.zeros(n * n)
    lib.orc_reversible_q(n, _p(rates, ct.c_double), _p(pi, ct.c_double), _p(Q, ct.c_double))
    return _decompose(Q, pi)


def _decompose(Q, pi) -> EigenModel:
    n = pi.size
    V, Vi, lam = np.zeros(n * n), np.zeros(n * n), np.zeros(n)
    lib.orc_reversible_eigen(n, _p(Q, ct.c_double), _p(pi, ct.c_double), _p(V, ct.c_double),
                             _p(Vi, ct.c_double), _p(lam, ct.c_double))
    return EigenModel(V, Vi, lam, Q, pi)


class JC:
    """Jukes-Cantor closed form (substitution.rs:126-156)."""

    def transition(self, d):
        out = np.zeros(16)
        lib.orc_jc_transition(float(d), _p(out, ct.c_double))
        return out.reshape(4, 4)

    def frequencies(self):
        return np.full(4, 0.25)


class K80:
    """Kimura 1980 closed form (substitution.rs:196-243)."""

    def __init__(self, kappa: float):
        self.kappa = float(kappa)

    def transition(self, d):
        out = np.zeros(16)
        lib.orc_k80_transition(self.kappa, float(d), _p(out, ct.c_double))
        return out.reshape(4, 4)

    def frequencies(self):
        return np.full(4, 0.25)


# ---------------------------------------------------------------------------
# DatedTree (parameters/tree.rs)


class DatedTree:
    """Host tree with the reference's dirty tracking and epoch buffers."""

    def __init__(self, parents, heights):
        parents = np.asarray(parents, dtype=np.int64)
        self.num_nodes = parents.size
        self.num_leaves = (self.num_nodes + 1) // 2
        self.num_internals = self.num_leaves - 1
        self.parents = [int(p) for p in parents]
        self.heights = [float(h) for h in heights]
        # load_parents (tree.rs:906-930): children in node order
        self.children = [TOMBSTONE] * (2 * self.num_internals)
        self.root_ = None
        for node, par in enumerate(self.parents):
            if par == TOMBSTONE:
                self.root_ = node
                continue
            off = (par - self.num_leaves) * 2
            if self.children[off] == TOMBSTONE:
                self.children[off] = node
            else:
                self.children[off + 1] = node
        self.updated_edges = [False] * self.num_nodes
        self.updated_partials = [False] * self.num_nodes
        self._backup()

    # -- epoch buffers (sk/src/epoch.rs) ------------------------------------
    def _backup(self):
        self._bk = (list(self.parents), list(self.heights), list(self.children), self.root_)

    def accept(self):  # tree.rs:980-986
        self._backup()
        self._clear_updated()

    def reject(self):  # tree.rs:988-994
        self.parents, self.heights, self.children, self.root_ = (
            list(self._bk[0]), list(self._bk[1]), list(self._bk[2]), self._bk[3])
        self._clear_updated()

    def _clear_updated(self):
        self.updated_edges = [False] * self.num_nodes
        self.updated_partials = [False] * self.num_nodes

    # -- structure -----------------------------------------------------------
    def root(self) -> int:
        return self.root_

    def is_leaf(self, v) -> bool:
        return v < self.num_leaves

    def children_of(self, v):
        off = (v - self.num_leaves) * 2
        return self.children[off], self.children[off + 1]

    def parent_of(self, v):
        p = self.parents[v]
        return None if p == TOMBSTONE else p

    def edge_length(self, edge) -> float:  # tree.rs:732-736
        return self.heights[self.parents[edge]] - self.heights[edge]

    def edges(self):  # tree.rs:833-836
        r = self.root_
        return [e for e in range(self.num_nodes) if e != r]

    # -- dirty tracking --------------------------------------------------------
    def mark_edge_updated(self, edge):  # tree.rs:357-374
        self.updated_edges[edge] = True
        curr = edge
        while True:
            nxt = self.parent_of(curr)
            if nxt is None:
                break
            curr = nxt
            if self.updated_partials[curr]:
                break
            self.updated_partials[curr] = True

    def mark_all_edges_updated(self):  # tree.rs:382-386
        self.updated_edges = [True] * self.num_nodes
        self.updated_partials = [True] * self.num_nodes

    def is_changed(self) -> bool:  # tree.rs:976-978
        return any(self.updated_edges)

    def edges_to_update(self):  # tree.rs:388-396
        return [e for e in self.edges() if self.updated_edges[e]]

    def _updated_internals(self):  # tree.rs:398-421
        out = [self.root_]
        queue = [self.root_]
        while queue:
            node = queue.pop(0)
            left, right = self.children_of(node)
            for ch in (left, right):
                if self.updated_partials[ch] and not self.is_leaf(ch):
                    out.append(ch)
                    queue.append(ch)
        out.reverse()
        return out

    def partials_lists(self):  # tree.rs:423-461
        internals = self._updated_internals()
        children = []
        for v in internals:
            l, r = self.children_of(v)
            children.append((l, r) if l < r else (r, l))
        return (np.array(internals, dtype=np.uint32),
                np.array(children, dtype=np.uint32).reshape(-1, 2))

    # -- moves ---------------------------------------------------------------
    def set_height(self, node, h):  # tree.rs:516-527
        self.heights[node] = float(h)
        if self.parent_of(node) is not None:
            self.mark_edge_updated(node)
        if not self.is_leaf(node):
            l, r = self.children_of(node)
            self.mark_edge_updated(l)
            self.mark_edge_updated(r)

    def replace_child(self, parent, old, new):  # tree.rs:471-495
        self.parents[new] = parent
        off = (parent - self.num_leaves) * 2
        if self.children[off] == old:
            self.children[off] = new
        elif self.children[off + 1] == old:
            self.children[off + 1] = new
        else:
            raise ValueError(f"{old} is not a child of {parent}")
        self.mark_edge_updated(new)

    def scale(self, s):  # tree.rs:335-348
        for v in range(self.num_leaves, self.num_nodes):
            self.set_height(v, self.heights[v] * s)

    def validate(self):  # tree.rs:584-651 (the structural part)
        for v in range(self.num_leaves, self.num_nodes):
            l, r = self.children_of(v)
            assert self.heights[v] > self.heights[l] and self.heights[v] > self.heights[r]
            assert self.parents[l] == v and self.parents[r] == v
        assert [i for i, p in enumerate(self.parents) if p == TOMBSTONE] == [self.root_]


# ---------------------------------------------------------------------------
# Transitions (transitions.rs with sk_slice_buf.rs)


class Transitions:
    def __init__(self, size: int, num_nodes: int):
        self.size = size
        self.slots = np.zeros((num_nodes, 2, size, size))
        self.edits = np.zeros(num_nodes, dtype=np.uint8)  # EditBuf
        self.freqs = np.zeros(size)

    def _offset(self, e):
        return int(self.edits[e] & 1)

    def update(self, tree: DatedTree, model, rate_of_edge):  # transitions.rs:26-48
        for edge in tree.edges_to_update():
            length = tree.edge_length(edge) * rate_of_edge(edge)
            m = self.edits[edge]
            if not (m & 2):
                self.edits[edge] = ((m & 1) ^ 1) | 2
            self.slots[edge, self._offset(edge)] = model.transition(length)
        self.freqs = model.frequencies()

    def accept(self):
        self.edits &= 1

    def reject(self):
        self.edits = (self.edits ^ (self.edits >> 1)) & 1

    def write_matrices(self, edges) -> np.ndarray:  # transitions.rs:62-72
        return np.stack([self.slots[e, self._offset(e)] for e in edges])


# ---------------------------------------------------------------------------
# likelihoods (likelihood/dna.rs, likelihood/gamma.rs)


class DnaLikelihood:
    """``DnaLikelihood`` (likelihood/dna.rs:17-124) with a strict clock."""

    def __init__(self, leaves, weights, tree: DatedTree, model, clock_rate=1.0,
                 scale_ln=30, num_threads=0):
        leaves = np.ascontiguousarray(leaves, dtype=np.uint8)
        self.weights = np.ascontiguousarray(weights, dtype=np.uint32)
        self.calc = Cpu4Calculator(leaves, self.weights.size, scale_ln, num_threads)
        self.tree = tree
        self.model = model
        self.clock_rate = float(clock_rate)
        self.transitions = Transitions(4, tree.num_nodes)
        self.cache = float("nan")
        self.last = float("nan")
        self.launched = False
        tree.mark_all_edges_updated()
        self.likelihood()
        self.accept()

    def set_model(self, model):
        """A substitution-model or clock change marks every edge
        (dna.rs:73-78)."""
        self.model = model
        self.tree.mark_all_edges_updated()

    def likelihood(self) -> float:  # dna.rs:68-100
        tree = self.tree
        if not tree.is_changed():
            self.last = self.cache
            return self.cache
        self.transitions.update(tree, self.model, lambda e: self.clock_rate)
        self.launched = True
        internals, children = tree.partials_lists()
        mats = self.transitions.write_matrices(children.reshape(-1))
        self.calc.propose(internals, children, mats, self.transitions.freqs)
        self.last = weighted_sum(self.calc.likelihoods(), self.weights)
        return self.last

    def accept(self):  # dna.rs:102-113
        self.cache = self.last
        if self.launched:
            self.calc.accept()
            self.transitions.accept()
        self.launched = False

    def reject(self):  # dna.rs:115-124
        if self.launched:
            self.calc.reject()
            self.transitions.reject()
        self.launched = False


class GammaLikelihood:
    """``GammaLikelihood`` (likelihood/gamma.rs:20-203)."""

    def __init__(self, leaves, weights, tree: DatedTree, model, num_categories: int,
                 alpha: float, clock_rate=1.0, scale_ln=30, num_threads=0):
        leaves = np.ascontiguousarray(leaves, dtype=np.uint8)
        self.weights = np.ascontiguousarray(weights, dtype=np.uint32)
        self.K = int(num_categories)
        self.calcs = [Cpu4Calculator(leaves, self.weights.size, scale_ln, num_threads)
                      for _ in range(self.K)]
        self.transitions = [Transitions(4, tree.num_nodes) for _ in range(self.K)]
        self.tree = tree
        self.model = model
        self.clock_rate = float(clock_rate)
        self.alpha = float(alpha)
        self.categories = gamma_categories(self.alpha, self.K)
        self.cache = float("nan")
        self.last = float("nan")
        self.launched = False
        tree.mark_all_edges_updated()
        self.likelihood()
        self.accept()

    def set_model(self, model):
        self.model = model
        self.tree.mark_all_edges_updated()

    def set_alpha(self, alpha):  # gamma.rs:120-124
        self.alpha = float(alpha)
        self.categories = gamma_categories(self.alpha, self.K)
        self.tree.mark_all_edges_updated()

    def likelihood(self) -> float:  # gamma.rs:97-169
        tree = self.tree
        if not tree.is_changed():
            self.last = self.cache
            return self.cache
        for tr, cat in zip(self.transitions, self.categories):
            tr.update(tree, self.model, lambda e, cat=cat: self.clock_rate * cat)
        self.launched = True
        internals, children = tree.partials_lists()
        for calc, tr in zip(self.calcs, self.transitions):
            calc.propose(internals, children, tr.write_matrices(children.reshape(-1)), tr.freqs)
        lik = 0.0
        div = np.log(1.0 / self.K)
        per = [c.likelihoods() for c in self.calcs]
        for i in range(self.weights.size):
            s = log_sum_exp([per[c][i] for c in range(self.K)]) + div
            lik += s * float(self.weights[i])
        self.last = lik
        return lik

    def accept(self):
        self.cache = self.last
        if self.launched:
            for c in self.calcs:
                c.accept()
            for t in self.transitions:
                t.accept()
        self.launched = False

    def reject(self):
        if self.launched:
            for c in self.calcs:
                c.reject()
            for t in self.transitions:
                t.reject()
        self.launched = False
