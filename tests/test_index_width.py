"""The element-index width decision of the pruning walks
(aspartik_gb300/csrc/index_width.hpp), compiled on its own with the host C++
compiler: 32-bit indices only when every slot * C * ldp + column stays below
2^31, and always 64-bit indices for the allocation-free entry point, whose
slot ids index caller buffers of unknown size."""

import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include "index_width.hpp"
#include <cstdio>
using namespace b3g;
#define CHECK(x) do { if (!(x)) { std::printf("failed: %s\n", #x); return 1; } } while (0)
int main() {
    // the 256-taxon workload: 510 slots x 4 categories x 17,792 patterns
    CHECK(narrow_index(510, 4, 17792));
    // exactly at the limit and one slot past it
    CHECK(narrow_index(1ull << 21, 1, 1024) == false);
    CHECK(narrow_index((1ull << 21) - 1, 1, 1024));
    CHECK(narrow_index((1ull << 31) / (16 * 524288), 16, 524288) == false);
    // products that overflow 64 bits are not narrow
    CHECK(narrow_index(~0ull - 1, 16, 524288) == false);
    CHECK(narrow_index(kUnknownSlots, 1, 128) == false);
    // the allocation-free entry point: 64-bit for every shape it accepts
    for (unsigned C = 1; C <= 16; ++C)
        for (unsigned long long ldp = 128; ldp <= (1ull << 21); ldp *= 2)
            CHECK(noalloc_narrow_index(C, ldp) == false);
    std::printf("ok\n");
    return 0;
}
"""


def test_index_width_decision():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        with open(src, "w") as f:
            f.write(PROGRAM)
        inc = os.path.join(ROOT, "aspartik_gb300", "csrc")
        subprocess.run([cxx, "-std=c++17", "-O1", f"-I{inc}", src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr
        assert out.stdout.strip() == "ok"
