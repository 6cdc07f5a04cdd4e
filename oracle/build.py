"""Build recipe of the CPU oracle ``oracle/libb3oracle.so``.

TEST INFRASTRUCTURE ONLY: the oracle is the checker of the GPU path and the
timed CPU baseline; nothing in the product links or loads it.

The reference's Rust workspace cannot be compiled here (no Rust toolchain,
and its git dependency ``computare`` is not vendored), so the restatement
stands in for its CPU pruner.  Its FP64 CUDA pruning kernel, however, is a
self-contained CUDA source: ``build_ref()`` compiles it (through the wrapper
``ref_cuda_partials.cu``) into ``oracle/_ref/ref_partials.cubin`` when the
reference tree is present, and the tests run it beside the oracle.
"""

from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "b3oracle.c"
HDR = HERE / "b3oracle.h"
LIB = HERE / "libb3oracle.so"


def build(verbose: bool = False) -> Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler found to build the oracle")
    if LIB.exists() and LIB.stat().st_mtime >= max(SRC.stat().st_mtime, HDR.stat().st_mtime):
        return LIB
    cmd = [cc, "-O3", "-std=c11", "-fPIC", "-shared", "-pthread", "-Wall",
           str(SRC), "-o", str(LIB), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


# the reference tree, read only at build time in the development container;
# the GPU machine receives the built cubin
REF_PARTIALS = Path("/root/reference/crates/b3/src/calculator/cuda_partials")
REF_WRAPPER = HERE / "ref_cuda_partials.cu"
REF_CUBIN = HERE / "_ref" / "ref_partials.cubin"


def build_ref(verbose: bool = False) -> Path | None:
    """Compile the reference's cuda_partials kernel for sm_103a into
    ``oracle/_ref/`` (None when the reference sources are absent: the
    prebuilt cubin, if any, is used as it is)."""
    srcs = [REF_PARTIALS / "kernels.cu", REF_PARTIALS / "typedefs.h"]
    if not all(p.exists() for p in srcs):
        return REF_CUBIN if REF_CUBIN.exists() else None
    deps = srcs + [REF_WRAPPER]
    if REF_CUBIN.exists() and REF_CUBIN.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return REF_CUBIN
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    REF_CUBIN.parent.mkdir(exist_ok=True)
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
           f"-I{REF_PARTIALS}", str(REF_WRAPPER), "-o", str(REF_CUBIN)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference kernel build failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {REF_CUBIN}")
    return REF_CUBIN


if __name__ == "__main__":
    build(verbose=True)
    build_ref(verbose=True)
