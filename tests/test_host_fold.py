"""The host-side fold of the FP32 walks' block sums
(aspartik_gb300/csrc/host_fold.hpp), compiled on its own with the host C++
compiler, against a restatement of the device fold's order (block_fold in
runs4.cuh): 32 lanes, lane l adding sums l, l + 32, ... in order, then
__shfl_down_sync levels 16, 8, 4, 2, 1 where every lane reads its partner's
value from before the level and a lane whose partner is out of range keeps
its own.  The totals must agree bit for bit for every count, including
counts below and not a multiple of 32, and with infinities and NaNs."""

import math
import os
import shutil
import struct
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include "host_fold.hpp"
#include <cstdio>
#include <cstring>
#include <vector>
int main() {
    unsigned n;
    while (std::scanf("%u", &n) == 1) {
        std::vector<double> v(n);
        for (unsigned k = 0; k < n; ++k) {
            unsigned long long b;
            std::scanf("%llx", &b);
            std::memcpy(&v[k], &b, 8);
        }
        const double t = b3g::fold_block_sums(v.data(), n);
        unsigned long long b;
        std::memcpy(&b, &t, 8);
        std::printf("%016llx\n", b);
    }
    return 0;
}
"""


def device_order(sums):
    """The warp's fold, simulated lane by lane in Python floats (IEEE
    doubles, the same rounding as the device's FP64 adds)."""
    lane = [0.0] * 32
    for l in range(32):
        s = 0.0
        for k in range(l, len(sums), 32):
            s = s + sums[k]
        lane[l] = s
    off = 16
    while off:
        prev = lane[:]
        lane = [prev[l] + (prev[l + off] if l + off < 32 else prev[l]) for l in range(32)]
        off //= 2
    return lane[0]


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def test_host_fold_matches_the_device_order():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    rng = np.random.default_rng(5)
    cases = [list(-rng.gamma(2.0, 5e3, size=n)) for n in (1, 5, 31, 32, 33, 139, 278, 1112)]
    cases.append([-1e300, -1e300, 1e-300] + list(rng.normal(size=40)))
    cases.append([-math.inf] + list(-rng.gamma(2.0, 5e3, size=60)))
    cases.append([math.nan] + list(-rng.gamma(2.0, 5e3, size=10)))
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "t.cpp"), os.path.join(d, "t")
        with open(src, "w") as f:
            f.write(PROGRAM)
        inc = os.path.join(ROOT, "aspartik_gb300", "csrc")
        subprocess.run([cxx, "-std=c++17", "-O2", f"-I{inc}", src, "-o", exe], check=True)
        text = "".join(f"{len(c)} " + " ".join(f"{bits(x):x}" for x in c) + "\n" for c in cases)
        out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True)
    got = [int(line, 16) for line in out.stdout.split()]
    assert len(got) == len(cases)
    for c, g in zip(cases, got):
        want = device_order(c)
        if math.isnan(want):
            assert math.isnan(struct.unpack("<d", struct.pack("<Q", g))[0])
        else:
            assert g == bits(want), len(c)
