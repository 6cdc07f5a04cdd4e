"""Runs the reference's own FP64 CUDA calculators.  TEST INFRASTRUCTURE ONLY.

``oracle/_ref/ref_partials.cubin`` and ``oracle/_ref/ref_propagations.cubin``
are crates/b3/src/calculator/cuda_partials/kernels.cu and
cuda_propagations/kernels.cu compiled from the reference tree
(``oracle/build.py::build_ref``).  This module loads them through the CUDA
driver API (ctypes over libcuda, no other dependency) and drives full
evaluations the way the reference's calculators do:

* ``RefCudaPartials``: ``CudaPartialsCalculator`` (cuda_partials/
  mod.rs:63-166): tip codes mapped to 0..4 (mod.rs:188-196), zeroed
  partials, scales and scale sums, the children-first list, the gathered
  transition matrices (rows of P, transitions.rs:55-72), the root
  frequencies, one thread per pattern in 32-thread blocks.
* ``RefCudaPropagations``: ``CudaPropagationsCalculator`` (cuda_propagations/
  mod.rs:75-260), the reference's default GPU calculator: raw tip codes,
  per-edge projections, the node list of ``propagation_lists`` (tree.rs:
  436-454: every updated leaf, then the updated internals children-first,
  the root last), leaf projections by their own kernel when there are more
  than 10, the propagation kernel in 64-thread blocks (four threads per
  pattern), then the root kernel.

The result is the per-pattern log-likelihood with the scaling removed, as
``likelihoods()`` returns it.  Only fresh full evaluations are driven: the
accept/reject path is restated by the oracle, and a repeated proposal
within one epoch would double-count the reference's scale sums
(cpu4.rs:403-433), which is not what is being pinned.
"""

from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

REF = Path(__file__).resolve().parent / "_ref"
CUBIN = REF / "ref_partials.cubin"
CUBIN_PROPAGATIONS = REF / "ref_propagations.cubin"

_cu = None


def _lib():
    global _cu
    if _cu is None:
        cu = ct.CDLL("libcuda.so.1")
        vp, u64, sz, i, u = ct.c_void_p, ct.c_uint64, ct.c_size_t, ct.c_int, ct.c_uint
        sig = {
            "cuInit": [u],
            "cuDeviceGet": [ct.POINTER(i), i],
            "cuDevicePrimaryCtxRetain": [ct.POINTER(vp), i],
            "cuDevicePrimaryCtxRelease_v2": [i],
            "cuCtxSetCurrent": [vp],
            "cuCtxSynchronize": [],
            "cuModuleLoad": [ct.POINTER(vp), ct.c_char_p],
            "cuModuleUnload": [vp],
            "cuModuleGetFunction": [ct.POINTER(vp), vp, ct.c_char_p],
            "cuModuleGetGlobal_v2": [ct.POINTER(u64), ct.POINTER(sz), vp, ct.c_char_p],
            "cuMemAlloc_v2": [ct.POINTER(u64), sz],
            "cuMemFree_v2": [u64],
            "cuMemsetD8_v2": [u64, ct.c_ubyte, sz],
            "cuMemcpyHtoD_v2": [u64, vp, sz],
            "cuMemcpyDtoH_v2": [vp, u64, sz],
            "cuLaunchKernel": [vp, u, u, u, u, u, u, u, vp, ct.POINTER(vp), ct.POINTER(vp)],
            "cuGetErrorString": [i, ct.POINTER(ct.c_char_p)],
            "cuEventCreate": [ct.POINTER(vp), u],
            "cuEventRecord": [vp, vp],
            "cuEventSynchronize": [vp],
            "cuEventElapsedTime": [ct.POINTER(ct.c_float), vp, vp],
            "cuEventDestroy_v2": [vp],
        }
        for name, args in sig.items():
            f = getattr(cu, name)
            f.argtypes = args
            f.restype = i
        _cu = cu
    return _cu


def _check(res: int, what: str) -> None:
    if res != 0:
        msg = ct.c_char_p()
        _lib().cuGetErrorString(res, ct.byref(msg))
        raise RuntimeError(f"{what}: CUDA driver error {res} "
                           f"({msg.value.decode() if msg.value else '?'})")


def available() -> bool:
    return CUBIN.exists()


def propagations_available() -> bool:
    return CUBIN_PROPAGATIONS.exists()


def dna_codes_to_ref(leaves: np.ndarray) -> np.ndarray:
    """4-bit IUPAC codes -> 0..3 for single bases, 4 otherwise
    (cuda_partials/mod.rs:188-196)."""
    out = np.full(leaves.shape, 4, dtype=np.uint8)
    for bit, state in ((1, 0), (2, 1), (4, 2), (8, 3)):
        out[leaves == bit] = state
    return out


class _RefModule:
    """The primary context of `device`, one loaded reference module and the
    named entry points; device buffers by name."""

    def __init__(self, cubin: Path, functions, device: int = 0):
        if not cubin.exists():
            raise FileNotFoundError(f"{cubin} is missing (built from the reference tree)")
        cu = _lib()
        _check(cu.cuInit(0), "cuInit")
        dev = ct.c_int()
        _check(cu.cuDeviceGet(ct.byref(dev), device), "cuDeviceGet")
        self.dev = dev.value
        self.ctx = ct.c_void_p()
        _check(cu.cuDevicePrimaryCtxRetain(ct.byref(self.ctx), dev), "primary context")
        _check(cu.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")
        self.mod = ct.c_void_p()
        _check(cu.cuModuleLoad(ct.byref(self.mod), str(cubin).encode()), "cuModuleLoad")
        self.fns = {}
        for name in functions:
            f = ct.c_void_p()
            _check(cu.cuModuleGetFunction(ct.byref(f), self.mod, name.encode()),
                   f"function {name}")
            self.fns[name] = f
        self.bufs = {}
        self._keep = []

    def close(self) -> None:
        cu = _lib()
        self.free()
        if getattr(self, "mod", None):
            cu.cuModuleUnload(self.mod)
            self.mod = None
        if getattr(self, "ctx", None):
            cu.cuDevicePrimaryCtxRelease_v2(self.dev)
            self.ctx = None

    def free(self) -> None:
        cu = _lib()
        for ptr in getattr(self, "bufs", {}).values():
            cu.cuMemFree_v2(ptr)
        self.bufs = {}

    def _current(self) -> None:
        _check(_lib().cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")

    def _alloc(self, name: str, nbytes: int, host: np.ndarray | None = None) -> None:
        cu = _lib()
        ptr = ct.c_uint64()
        _check(cu.cuMemAlloc_v2(ct.byref(ptr), max(int(nbytes), 1)), f"alloc {name}")
        self.bufs[name] = ptr
        if host is None:
            _check(cu.cuMemsetD8_v2(ptr, 0, max(int(nbytes), 1)), f"zero {name}")
        else:
            self._upload(name, host)

    def _upload(self, name: str, host: np.ndarray) -> None:
        host = np.ascontiguousarray(host)
        _check(_lib().cuMemcpyHtoD_v2(self.bufs[name], host.ctypes.data_as(ct.c_void_p),
                                      host.nbytes), f"upload {name}")

    def _zero(self, name: str, nbytes: int) -> None:
        _check(_lib().cuMemsetD8_v2(self.bufs[name], 0, int(nbytes)), f"zero {name}")

    def _download(self, name: str, out: np.ndarray) -> np.ndarray:
        self.synchronize()
        _check(_lib().cuMemcpyDtoH_v2(out.ctypes.data_as(ct.c_void_p), self.bufs[name],
                                      out.nbytes), f"download {name}")
        return out

    def _set_const(self, name: str, value) -> None:
        cu = _lib()
        ptr, size = ct.c_uint64(), ct.c_size_t()
        _check(cu.cuModuleGetGlobal_v2(ct.byref(ptr), ct.byref(size), self.mod, name.encode()),
               f"global {name}")
        buf = np.array([value], dtype=np.uint32 if isinstance(value, int) else np.float64)
        assert buf.nbytes == size.value
        _check(cu.cuMemcpyHtoD_v2(ptr, buf.ctypes.data_as(ct.c_void_p), size.value),
               f"set {name}")

    def _set_sizes(self, L: int, P: int, scale_ln: int) -> None:
        self._set_const("ref_num_patterns", int(P))
        self._set_const("ref_num_leaves", int(L))
        self._set_const("ref_scale_ln", int(scale_ln))
        self._set_const("ref_scale_threshold", float(np.exp(-float(scale_ln))))
        self._set_const("ref_scale_mult", float(np.exp(float(scale_ln))))

    def _params(self, args) -> ct.Array:
        """Kernel parameter array: each argument is a ctypes scalar (a device
        pointer as c_uint64) or a numpy array passed by value."""
        ptrs = []
        for a in args:
            if isinstance(a, np.ndarray):
                ptrs.append(ct.c_void_p(a.ctypes.data))
            else:
                ptrs.append(ct.c_void_p(ct.addressof(a)))
        self._keep.append(args)
        return (ct.c_void_p * len(ptrs))(*ptrs)

    def _launch(self, fn: str, grid, block, params) -> None:
        gx, gy, gz = (tuple(grid) + (1, 1))[:3]
        bx, by, bz = (tuple(block) + (1, 1))[:3]
        _check(_lib().cuLaunchKernel(self.fns[fn], gx, gy, gz, bx, by, bz, 0, None, params,
                                     None), f"launch {fn}")

    def synchronize(self) -> None:
        _check(_lib().cuCtxSynchronize(), "synchronize")

    def time(self, launch, reps: int) -> float:
        """Device milliseconds per call of `launch` (which queues the same
        kernels with the same arguments), over `reps` calls between two
        events."""
        cu = _lib()
        e0, e1 = ct.c_void_p(), ct.c_void_p()
        _check(cu.cuEventCreate(ct.byref(e0), 0), "event")
        _check(cu.cuEventCreate(ct.byref(e1), 0), "event")
        try:
            _check(cu.cuEventRecord(e0, None), "record")
            for _ in range(reps):
                launch()
            _check(cu.cuEventRecord(e1, None), "record")
            _check(cu.cuEventSynchronize(e1), "event sync")
            ms = ct.c_float()
            _check(cu.cuEventElapsedTime(ct.byref(ms), e0, e1), "elapsed")
            return ms.value / reps
        finally:
            cu.cuEventDestroy_v2(e0)
            cu.cuEventDestroy_v2(e1)


class RefCudaPartials(_RefModule):
    """The reference's partials calculator (one launch per evaluation)."""

    def __init__(self, device: int = 0):
        super().__init__(CUBIN, ["propose"], device)

    def setup(self, ref_leaves: np.ndarray, scale_ln: int = 30) -> None:
        """Device buffers as CudaPartialsCalculator::new allocates them
        (cuda_partials/mod.rs:171-270), for tip codes ref_leaves [L][P]."""
        self._current()
        self.free()
        leaves = np.ascontiguousarray(ref_leaves, dtype=np.uint8)
        L, P = leaves.shape
        I = L - 1
        self.L, self.P, self.scale_ln = L, P, int(scale_ln)
        self._alloc("leaves", leaves.nbytes, leaves)
        self._alloc("partials", I * 2 * P * 32)
        self._alloc("scales", I * 2 * P)
        self._alloc("scale_sums", P * 4)
        self._alloc("selectors", I)
        self._alloc("internals", I * 4)
        self._alloc("children", I * 8)
        self._alloc("transitions", I * 2 * 16 * 8)
        self._alloc("likelihoods", P * 8)

    def propose(self, internals, children, matrices, frequencies) -> None:
        """One evaluation from zeroed scale state (asynchronous):
        internals [n], children [n][2], matrices [n][2][4][4], frequencies [4]."""
        self._current()
        L, P, I = self.L, self.P, self.L - 1
        internals = np.ascontiguousarray(internals, dtype=np.uint32)
        children = np.ascontiguousarray(children, dtype=np.uint32).reshape(-1)
        n = internals.size
        mats = np.ascontiguousarray(matrices, dtype=np.float64).reshape(n * 2, 16)
        if children.size != 2 * n or not (1 <= n <= I):
            raise ValueError("bad lists")
        if internals.min() < L or internals.max() >= 2 * L - 1 or children.max() >= 2 * L - 1:
            raise ValueError("node ids out of range")
        self._set_sizes(L, P, self.scale_ln)
        self._zero("scales", I * 2 * P)
        self._zero("scale_sums", P * 4)
        self._upload("internals", internals)
        self._upload("children", children)
        self._upload("transitions", mats)
        b = self.bufs
        freqs = np.ascontiguousarray(frequencies, dtype=np.float64)
        params = self._params([b["leaves"], b["partials"], b["scales"], b["scale_sums"],
                               b["selectors"], ct.c_uint32(n), b["internals"], b["children"],
                               b["transitions"], b["likelihoods"], freqs])
        grid = ((P + 31) // 32,)
        self._last = lambda: self._launch("propose", grid, (32,), params)
        self._last()

    def time_last(self, reps: int) -> float:
        return self.time(self._last, reps)

    def result(self) -> np.ndarray:
        return self._download("likelihoods", np.empty(self.P, dtype=np.float64))

    def likelihoods(self, ref_leaves: np.ndarray, internals, children, matrices,
                    frequencies, scale_ln: int = 30) -> np.ndarray:
        """Per-pattern lnL of one full evaluation on fresh buffers."""
        self.setup(ref_leaves, scale_ln)
        try:
            self.propose(internals, children, matrices, frequencies)
            return self.result()
        finally:
            self.free()


class RefCudaPropagations(_RefModule):
    """The reference's propagations calculator, its default GPU calculator
    (leaf kernel, propagation kernel, root kernel per evaluation)."""

    LEAF_BLOCK = 256
    PROP_BLOCK = 64

    def __init__(self, device: int = 0):
        super().__init__(CUBIN_PROPAGATIONS, ["update_leaves", "propose", "update_likelihoods"],
                         device)

    def setup(self, leaves_codes: np.ndarray, scale_ln: int = 30) -> None:
        """Device buffers as CudaPropagationsCalculator::new allocates them
        (cuda_propagations/mod.rs:270-340); raw 4-bit tip codes [L][P]."""
        self._current()
        self.free()
        leaves = np.ascontiguousarray(leaves_codes, dtype=np.uint8)
        L, P = leaves.shape
        N, I = 2 * L - 1, L - 1
        self.L, self.P, self.scale_ln = L, P, int(scale_ln)
        self._alloc("leaves", leaves.nbytes, leaves)
        self._alloc("projections", N * P * 2 * 4 * 8)
        self._alloc("scales", N * P * 2)
        self._alloc("scale_sums", P * 4)
        self._alloc("selectors", N)
        self._alloc("nodes", N * 4)
        self._alloc("children", I * 8)
        self._alloc("transitions", (N - 1) * 16 * 8)
        self._alloc("likelihoods", P * 8)

    def propose(self, nodes, num_leaves_listed: int, children, matrices, frequencies) -> None:
        """One evaluation from zeroed scale state (asynchronous).  nodes [m]:
        the listed leaves (num_leaves_listed of them), then the listed
        internals children-first, the root last; children [m -
        num_leaves_listed][2] of those internals; matrices [m - 1][4][4], P of
        the edge above each listed node but the root; frequencies [4]."""
        self._current()
        L, P = self.L, self.P
        N, I = 2 * L - 1, L - 1
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32)
        children = np.ascontiguousarray(children, dtype=np.uint32).reshape(-1, 2)
        m = nodes.size
        k = int(num_leaves_listed)
        mats = np.ascontiguousarray(matrices, dtype=np.float64).reshape(-1, 16)
        if not (2 <= m <= N) or not (0 <= k < m) or children.shape[0] != m - k \
                or children.shape[0] > I or mats.shape[0] != m - 1:
            raise ValueError("bad lists")
        if nodes.max() >= N or children.max() >= N or (k and nodes[:k].max() >= L) \
                or nodes[k:].min() < L:
            raise ValueError("node ids out of range")
        self._set_sizes(L, P, self.scale_ln)
        self._zero("scales", N * P * 2)
        self._zero("scale_sums", P * 4)
        self._upload("nodes", nodes)
        self._upload("children", children)
        self._upload("transitions", mats)
        b = self.bufs
        leaves_end = k
        launches = []
        if leaves_end > 10:  # cuda_propagations/mod.rs:106-110
            pl = self._params([b["leaves"], b["projections"], b["selectors"], b["nodes"],
                               b["transitions"]])
            grid = ((P * 4 + self.LEAF_BLOCK - 1) // self.LEAF_BLOCK, leaves_end)
            block = (self.LEAF_BLOCK // 4, 4)
            launches.append(lambda: self._launch("update_leaves", grid, block, pl))
            leaves_end = 0
        pp = self._params([b["leaves"], b["projections"], b["scales"], b["scale_sums"],
                           b["selectors"], ct.c_uint32(m - 1), b["nodes"], b["children"],
                           b["transitions"], ct.c_uint32(leaves_end), ct.c_uint32(k)])
        pgrid = ((P * 4 + self.PROP_BLOCK - 1) // self.PROP_BLOCK,)
        launches.append(lambda: self._launch("propose", pgrid, (self.PROP_BLOCK,), pp))
        root = int(nodes[-1])
        left, right = (int(x) for x in children[-1])
        freqs = np.ascontiguousarray(frequencies, dtype=np.float64)
        pr = self._params([b["projections"], b["likelihoods"], b["scales"], b["scale_sums"],
                           b["selectors"], ct.c_uint32(root), ct.c_uint32(left),
                           ct.c_uint32(right), freqs])
        rgrid = ((P + 31) // 32,)
        launches.append(lambda: self._launch("update_likelihoods", rgrid, (32,), pr))

        def run():
            for f in launches:
                f()

        self._last = run
        run()

    def time_last(self, reps: int) -> float:
        return self.time(self._last, reps)

    def result(self) -> np.ndarray:
        return self._download("likelihoods", np.empty(self.P, dtype=np.float64))


def propagation_inputs(tree, model, rate, L):
    """The lists of the reference's propagations calculator for a full
    evaluation (tree.rs:436-454): every leaf, then the internals
    children-first with the root last; the children of those internals; P
    of the edge above every node but the root."""
    from oracle import oracle as O

    t = O.DatedTree(tree.parents, tree.heights)
    t.mark_all_edges_updated()
    internals, children = t.partials_lists()
    nodes = np.concatenate([np.arange(L, dtype=np.uint32), np.asarray(internals, np.uint32)])
    mats = np.array([model.transition(t.edge_length(int(v)) * rate) for v in nodes[:-1]])
    return nodes, L, np.asarray(children, np.uint32), mats
