"""Runs the reference's own FP64 CUDA pruning kernel.  TEST INFRASTRUCTURE ONLY.

``oracle/_ref/ref_partials.cubin`` is crates/b3/src/calculator/cuda_partials/
kernels.cu compiled from the reference tree (``oracle/build.py::build_ref``).
This module loads it through the CUDA driver API (ctypes over libcuda, no
other dependency) and drives one evaluation the way
``CudaPartialsCalculator`` does (cuda_partials/mod.rs:63-100,134-166): tip
codes mapped to 0..4 (mod.rs:188-196), zeroed partials, scales and scale
sums, the children-first list, the gathered transition matrices (rows of
P, ``transitions.rs:55-72``), the root frequencies, one thread per pattern
in 32-thread blocks.  The result is the per-pattern log-likelihood with the
scaling removed, as ``likelihoods()`` returns it.

Only fresh full evaluations are driven: the reference's accept/reject path
is restated by the oracle, and a repeated proposal within one epoch would
double-count its scale sums (cpu4.rs:403-433), which is not what is being
pinned here.
"""

from __future__ import annotations

import ctypes as ct
from pathlib import Path

import numpy as np

CUBIN = Path(__file__).resolve().parent / "_ref" / "ref_partials.cubin"
BLOCK = 32

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


def dna_codes_to_ref(leaves: np.ndarray) -> np.ndarray:
    """4-bit IUPAC codes -> 0..3 for single bases, 4 otherwise
    (cuda_partials/mod.rs:188-196)."""
    out = np.full(leaves.shape, 4, dtype=np.uint8)
    for bit, state in ((1, 0), (2, 1), (4, 2), (8, 3)):
        out[leaves == bit] = state
    return out


class RefCudaPartials:
    """One device and context (the primary context of `device`), the loaded
    reference module and its `propose` entry point."""

    def __init__(self, device: int = 0):
        if not available():
            raise FileNotFoundError(f"{CUBIN} is missing (built from the reference tree)")
        cu = _lib()
        _check(cu.cuInit(0), "cuInit")
        dev = ct.c_int()
        _check(cu.cuDeviceGet(ct.byref(dev), device), "cuDeviceGet")
        self.ctx = ct.c_void_p()
        _check(cu.cuDevicePrimaryCtxRetain(ct.byref(self.ctx), dev), "primary context")
        self.dev = dev.value
        _check(cu.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")
        self.mod = ct.c_void_p()
        _check(cu.cuModuleLoad(ct.byref(self.mod), str(CUBIN).encode()), "cuModuleLoad")
        self.fn = ct.c_void_p()
        _check(cu.cuModuleGetFunction(ct.byref(self.fn), self.mod, b"propose"),
               "cuModuleGetFunction")

    def close(self) -> None:
        cu = _lib()
        self.free()
        if getattr(self, "mod", None):
            cu.cuModuleUnload(self.mod)
            self.mod = None
        if getattr(self, "ctx", None):
            cu.cuDevicePrimaryCtxRelease_v2(self.dev)
            self.ctx = None

    def _set_const(self, name: str, value) -> None:
        cu = _lib()
        ptr, size = ct.c_uint64(), ct.c_size_t()
        _check(cu.cuModuleGetGlobal_v2(ct.byref(ptr), ct.byref(size), self.mod, name.encode()),
               f"global {name}")
        buf = np.array([value], dtype=np.uint32 if isinstance(value, int) else np.float64)
        assert buf.nbytes == size.value
        _check(cu.cuMemcpyHtoD_v2(ptr, buf.ctypes.data_as(ct.c_void_p), size.value),
               f"set {name}")

    def setup(self, ref_leaves: np.ndarray, scale_ln: int = 30) -> None:
        """Device buffers of one calculator (as CudaPartialsCalculator::new,
        cuda_partials/mod.rs:171-270) for tip codes ref_leaves [L][P]."""
        cu = _lib()
        _check(cu.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")
        self.free()
        leaves = np.ascontiguousarray(ref_leaves, dtype=np.uint8)
        L, P = leaves.shape
        I = L - 1
        self.L, self.P, self.scale_ln = L, P, int(scale_ln)
        self.bufs = {}

        def alloc(name, nbytes, host=None):
            ptr = ct.c_uint64()
            _check(cu.cuMemAlloc_v2(ct.byref(ptr), max(int(nbytes), 1)), f"alloc {name}")
            self.bufs[name] = ptr
            if host is None:
                _check(cu.cuMemsetD8_v2(ptr, 0, max(int(nbytes), 1)), f"zero {name}")
            else:
                _check(cu.cuMemcpyHtoD_v2(ptr, host.ctypes.data_as(ct.c_void_p), host.nbytes),
                       f"upload {name}")

        alloc("leaves", leaves.nbytes, leaves)
        alloc("partials", I * 2 * P * 32)
        alloc("scales", I * 2 * P)
        alloc("scale_sums", P * 4)
        alloc("selectors", I)
        alloc("internals", I * 4)
        alloc("children", I * 8)
        alloc("transitions", I * 2 * 16 * 8)
        alloc("likelihoods", P * 8)

    def free(self) -> None:
        cu = _lib()
        for ptr in getattr(self, "bufs", {}).values():
            cu.cuMemFree_v2(ptr)
        self.bufs = {}

    def propose(self, internals, children, matrices, frequencies) -> None:
        """One launch over the list (asynchronous), from zeroed scale state:
        internals [n], children [n][2], matrices [n][2][4][4], frequencies [4]."""
        cu = _lib()
        _check(cu.cuCtxSetCurrent(self.ctx), "cuCtxSetCurrent")
        L, P, I = self.L, self.P, self.L - 1
        internals = np.ascontiguousarray(internals, dtype=np.uint32)
        children = np.ascontiguousarray(children, dtype=np.uint32).reshape(-1)
        n = internals.size
        mats = np.ascontiguousarray(matrices, dtype=np.float64).reshape(n * 2, 16)
        if children.size != 2 * n or not (1 <= n <= I):
            raise ValueError("bad lists")
        if internals.min() < L or internals.max() >= 2 * L - 1 or children.max() >= 2 * L - 1:
            raise ValueError("node ids out of range")
        self._set_const("ref_num_patterns", int(P))
        self._set_const("ref_num_leaves", int(L))
        self._set_const("ref_scale_ln", self.scale_ln)
        self._set_const("ref_scale_threshold", float(np.exp(-float(self.scale_ln))))
        self._set_const("ref_scale_mult", float(np.exp(float(self.scale_ln))))
        b = self.bufs
        _check(cu.cuMemsetD8_v2(b["scales"], 0, I * 2 * P), "zero scales")
        _check(cu.cuMemsetD8_v2(b["scale_sums"], 0, P * 4), "zero scale sums")
        for name, arr in (("internals", internals), ("children", children),
                          ("transitions", mats)):
            _check(cu.cuMemcpyHtoD_v2(b[name], arr.ctypes.data_as(ct.c_void_p), arr.nbytes),
                   f"upload {name}")
        self._freqs = np.ascontiguousarray(frequencies, dtype=np.float64)
        self._n = ct.c_uint32(n)
        args = [b["leaves"], b["partials"], b["scales"], b["scale_sums"], b["selectors"],
                self._n, b["internals"], b["children"], b["transitions"], b["likelihoods"]]
        ptrs = [ct.c_void_p(ct.addressof(a)) for a in args]
        ptrs.append(ct.c_void_p(self._freqs.ctypes.data))
        self._params = (ct.c_void_p * len(ptrs))(*ptrs)
        grid = (P + BLOCK - 1) // BLOCK
        _check(cu.cuLaunchKernel(self.fn, grid, 1, 1, BLOCK, 1, 1, 0, None, self._params, None),
               "launch")

    def time_launch(self, reps: int) -> float:
        """Device milliseconds per launch of the last proposal's kernel,
        relaunched `reps` times with the same arguments between two events
        (every launch does the same work)."""
        cu = _lib()
        e0, e1 = ct.c_void_p(), ct.c_void_p()
        _check(cu.cuEventCreate(ct.byref(e0), 0), "event")
        _check(cu.cuEventCreate(ct.byref(e1), 0), "event")
        try:
            grid = (self.P + BLOCK - 1) // BLOCK
            _check(cu.cuEventRecord(e0, None), "record")
            for _ in range(reps):
                _check(cu.cuLaunchKernel(self.fn, grid, 1, 1, BLOCK, 1, 1, 0, None,
                                         self._params, None), "launch")
            _check(cu.cuEventRecord(e1, None), "record")
            _check(cu.cuEventSynchronize(e1), "event sync")
            ms = ct.c_float()
            _check(cu.cuEventElapsedTime(ct.byref(ms), e0, e1), "elapsed")
            return ms.value / reps
        finally:
            cu.cuEventDestroy_v2(e0)
            cu.cuEventDestroy_v2(e1)

    def synchronize(self) -> None:
        _check(_lib().cuCtxSynchronize(), "synchronize")

    def result(self) -> np.ndarray:
        """Per-pattern lnL of the last proposal (waits for it)."""
        self.synchronize()
        out = np.empty(self.P, dtype=np.float64)
        _check(_lib().cuMemcpyDtoH_v2(out.ctypes.data_as(ct.c_void_p), self.bufs["likelihoods"],
                                      out.nbytes), "download")
        return out

    def likelihoods(self, ref_leaves: np.ndarray, internals, children, matrices,
                    frequencies, scale_ln: int = 30) -> np.ndarray:
        """Per-pattern lnL of one full evaluation on fresh buffers."""
        self.setup(ref_leaves, scale_ln)
        try:
            self.propose(internals, children, matrices, frequencies)
            return self.result()
        finally:
            self.free()
