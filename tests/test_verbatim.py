"""The verbatim byte layout of state files (aspartik_gb300/csrc/verbatim.hpp),
compiled on its own with the host C++ compiler, against the Python
restatement of the reference's writer and reader rules (tests/verbatim_ref.py):
the same sequence of values gives the same bytes (padding after odd-length
slices, before a u128, none before an empty slice), the reader reads the
restatement's bytes back, and a short stream is an error."""

import os
import shutil
import subprocess
import tempfile

import pytest

from tests.verbatim_ref import STATE_TAG, STATE_VERSION, Reader, Writer

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include "verbatim.hpp"
#include <cstdio>
#include <vector>
using namespace b3g;
int main(int argc, char **argv) {
    if (argc > 1) { // read the hex stream on stdin back
        std::vector<uint8_t> in;
        unsigned x;
        while (std::scanf("%2x", &x) == 1) in.push_back((uint8_t)x);
        verbatim::Reader r(in.data(), in.size());
        const uint8_t tag[4] = {0x62, 0x33, 0xb3, 0x44};
        if (!r.tag(tag, 4)) { std::printf("tag\n"); return 1; }
        const unsigned version = r.u32();
        const unsigned long long step = r.u64();
        const double posterior = r.f64();
        std::printf("%u %llu %.17g", version, step, posterior);
        for (uint32_t v : r.slice_u32()) std::printf(" %u", v);
        for (double v : r.slice_f64()) std::printf(" %.17g", v);
        std::printf(" %u", (unsigned)r.slice_u32().size());
        std::printf(" %lld", (long long)r.i64());
        uint64_t lo, hi;
        r.u128(lo, hi);
        std::printf(" %llu %llu", (unsigned long long)lo, (unsigned long long)hi);
        std::printf(" left %zu\n", r.left());
        try {
            r.u32();
        } catch (const std::runtime_error &) {
            std::printf("short\n");
        }
        return 0;
    }
    verbatim::Writer w;
    const uint8_t tag[4] = {0x62, 0x33, 0xb3, 0x44};
    w.tag(tag, 4);
    w.u32(19);
    w.u64(123456789012ull);
    w.f64(-2105517.25);
    const uint32_t parents[3] = {2, 2, 0xFFFFFFFFu};
    w.slice_u32(parents, 3);
    const double heights[3] = {0.0, 0.0, 0.75};
    w.slice_f64(heights, 3);
    w.slice_u32(nullptr, 0);
    w.i64(-7);
    w.u128(0x0123456789abcdefull, 0xfedcba9876543210ull);
    for (uint8_t b : w.bytes()) std::printf("%02x", b);
    std::printf("\n");
    return 0;
}
"""


def expected() -> bytes:
    w = Writer()
    w.tag(STATE_TAG)
    w.prim("u32", STATE_VERSION)
    w.prim("u64", 123456789012)
    w.prim("f64", -2105517.25)
    w.slice("u32", [2, 2, 0xFFFFFFFF])
    w.slice("f64", [0.0, 0.0, 0.75])
    w.slice("u32", [])
    w.prim("i64", -7)
    w.u128(0xFEDCBA9876543210 << 64 | 0x0123456789ABCDEF)
    return bytes(w.out)


@pytest.fixture(scope="module")
def program():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    d = tempfile.mkdtemp()
    src, exe = os.path.join(d, "t.cpp"), os.path.join(d, "t")
    with open(src, "w") as f:
        f.write(PROGRAM)
    inc = os.path.join(ROOT, "aspartik_gb300", "csrc")
    subprocess.run([cxx, "-std=c++17", "-O1", f"-I{inc}", src, "-o", exe], check=True)
    yield exe
    shutil.rmtree(d)


def test_writer_matches_the_reference_layout(program):
    out = subprocess.run([program], capture_output=True, text=True, check=True)
    got = bytes.fromhex(out.stdout.strip())
    want = expected()
    assert got == want
    # the layout's fixed points: version at byte 4 (the reference's own
    # version test rewrites that byte), the odd u32 slice padded before the
    # f64 slice's elements, the u128 on a multiple of 16
    assert got[:4] == STATE_TAG and got[4] == STATE_VERSION
    assert len(got) % 16 == 0


def test_reader_reads_the_reference_layout(program):
    out = subprocess.run([program, "read"], input=expected().hex(), capture_output=True,
                         text=True, check=True)
    lines = out.stdout.split("\n")
    assert lines[0] == ("19 123456789012 -2105517.25 2 2 4294967295 0 0 0.75 0 -7 "
                        f"{0x0123456789ABCDEF} {0xFEDCBA9876543210} left 0")
    assert lines[1] == "short"


def test_python_restatement_round_trips():
    r = Reader(expected())
    assert r.tag(4) == STATE_TAG
    assert r.prim("u32") == STATE_VERSION
    assert r.prim("u64") == 123456789012
    assert r.prim("f64") == -2105517.25
    assert r.slice("u32") == [2, 2, 0xFFFFFFFF]
    assert r.slice("f64") == [0.0, 0.0, 0.75]
    assert r.slice("u32") == []
    assert r.prim("i64") == -7
    assert r.u128() == 0xFEDCBA9876543210 << 64 | 0x0123456789ABCDEF
    assert r.left() == 0
