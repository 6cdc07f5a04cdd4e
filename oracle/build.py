"""Build recipe of the CPU oracle ``oracle/libb3oracle.so``.

TEST INFRASTRUCTURE ONLY: the oracle is the checker of the GPU path and the
timed CPU baseline; nothing in the product links or loads it.

The reference itself (a Rust workspace) cannot be compiled here: there is no
Rust toolchain and its git dependency ``computare`` is not vendored, so no
``oracle/_ref`` build exists and this restatement stands in for it.
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


if __name__ == "__main__":
    build(verbose=True)
