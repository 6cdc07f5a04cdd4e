"""Build recipe of the CPU oracle ``oracle/libb3oracle.so``.

TEST INFRASTRUCTURE ONLY: the oracle is the checker of the GPU path and the
timed CPU baseline; nothing in the product links or loads it.

The reference's Rust workspace cannot be compiled here (no Rust toolchain,
and its git dependency ``computare`` is not vendored), so the restatement
stands in for its CPU pruner.  Its FP64 CUDA pruning kernel, however, is a
self-contained CUDA source, and so are the kernels of its default GPU
calculator (cuda_propagations): ``build_ref()`` compiles both (through the
wrappers ``ref_cuda_partials.cu`` and ``ref_cuda_propagations.cu``) into
``oracle/_ref/`` when the reference tree is present, and the tests run them
beside the oracle.
"""

from __future__ import annotations

import os
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


# The reference tree is read only at build time: the argument of
# build_ref, else the B3G_REFERENCE_ROOT environment variable, else the
# development container's checkout.  The GPU machine receives the built
# cubins.
DEFAULT_REFERENCE_ROOT = "/root/reference"
# (calculator directory under crates/b3/src/calculator, wrapper, output)
REF_BUILDS = [
    ("cuda_partials", HERE / "ref_cuda_partials.cu", HERE / "_ref" / "ref_partials.cubin"),
    ("cuda_propagations", HERE / "ref_cuda_propagations.cu",
     HERE / "_ref" / "ref_propagations.cubin"),
]
REF_CUBIN = REF_BUILDS[0][2]


def reference_root(root: str | os.PathLike | None = None) -> Path:
    return Path(root or os.environ.get("B3G_REFERENCE_ROOT") or DEFAULT_REFERENCE_ROOT)


def build_ref(verbose: bool = False, root: str | os.PathLike | None = None) -> list[Path]:
    """Compile the reference's CUDA calculator kernels for sm_103a into
    ``oracle/_ref/`` from the reference tree at ``root`` (see
    ``reference_root``); where the reference sources are absent the
    prebuilt cubins, if any, are used as they are.  Returns the cubins
    present."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    calc = reference_root(root) / "crates" / "b3" / "src" / "calculator"
    out = []
    for name, wrapper, cubin in REF_BUILDS:
        src_dir = calc / name
        srcs = [src_dir / "kernels.cu", src_dir / "typedefs.h"]
        if not all(p.exists() for p in srcs):
            if cubin.exists():
                out.append(cubin)
            continue
        deps = srcs + [wrapper]
        if not (cubin.exists() and
                cubin.stat().st_mtime >= max(p.stat().st_mtime for p in deps)):
            cubin.parent.mkdir(exist_ok=True)
            cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                   f"-I{src_dir}", str(wrapper), "-o", str(cubin)]
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"reference kernel build failed:\n{res.stdout}\n"
                                   f"{res.stderr}")
            if verbose:
                print(f"built {cubin}")
        out.append(cubin)
    return out


if __name__ == "__main__":
    build(verbose=True)
    build_ref(verbose=True)
