"""The host thread pool of the MCMC driver (aspartik_gb300/csrc/host_pool.hpp),
compiled on its own with the host C++ compiler: every worker index runs once
per call, calls are repeatable many times (spinning and sleeping workers
alike), the exception of the lowest index is rethrown, a failing worker
start ends the pool, and the ctypes mirror of b3g_mcmc_config has the C
header's layout."""

import ctypes as ct
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

POOL_PROGRAM = r"""
#include "host_pool.hpp"
#include <chrono>
#include <cstdio>
#include <stdexcept>
#include <string>
using namespace b3g;
#define CHECK(x) do { if (!(x)) { std::printf("failed: %s\n", #x); return 1; } } while (0)
int main() {
    for (unsigned T : {1u, 2u, 3u, 8u}) {
        std::atomic<int> inits{0};
        HostPool pool(T, [&] { ++inits; });
        CHECK(pool.size() == T);
        CHECK(inits.load() == (int)T - 1);
        std::vector<int> hits(T, 0);
        for (int call = 0; call < 20000; ++call)
            pool.run([&](uint32_t w) { ++hits[w]; });
        for (unsigned w = 0; w < T; ++w)
            CHECK(hits[w] == 20000);
        // workers that went to sleep wake for the next call
        std::this_thread::sleep_for(std::chrono::milliseconds(50));
        pool.run([&](uint32_t w) { ++hits[w]; });
        for (unsigned w = 0; w < T; ++w)
            CHECK(hits[w] == 20001);
        // the lowest index's exception, and the pool stays usable
        if (T > 2) {
            std::string what;
            try {
                pool.run([&](uint32_t w) {
                    if (w >= 1)
                        throw std::runtime_error("worker " + std::to_string(w));
                });
            } catch (const std::exception &e) {
                what = e.what();
            }
            CHECK(what == "worker 1");
            int sum = 0;
            std::atomic<int> s{0};
            pool.run([&](uint32_t w) { s += (int)w; });
            for (unsigned w = 0; w < T; ++w)
                sum += (int)w;
            CHECK(s.load() == sum);
        }
    }
    // a worker whose start fails: the constructor throws and joins
    bool threw = false;
    try {
        HostPool bad(4, [] { throw std::runtime_error("no device"); });
    } catch (const std::exception &) {
        threw = true;
    }
    CHECK(threw);
    std::printf("ok\n");
    return 0;
}
"""

LAYOUT_PROGRAM = r"""
#include "b3g.h"
#include <stddef.h>
#include <stdio.h>
int main(void) {
    printf("%zu %zu %zu %zu %zu\n", sizeof(b3g_mcmc_config),
           offsetof(b3g_mcmc_config, da_drift_limit),
           offsetof(b3g_mcmc_config, clock_categories),
           offsetof(b3g_mcmc_config, launch),
           offsetof(b3g_mcmc_config, host_threads));
    return 0;
}
"""


def _run(compiler: str, program: str, suffix: str, flags: list[str]) -> str:
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t" + suffix)
        exe = os.path.join(d, "t")
        with open(src, "w") as f:
            f.write(program)
        subprocess.run([compiler, *flags, src, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert out.returncode == 0, out.stdout + out.stderr
        return out.stdout.strip()


def test_host_pool():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    inc = os.path.join(ROOT, "aspartik_gb300", "csrc")
    assert _run(cxx, POOL_PROGRAM, ".cpp", ["-std=c++17", "-O1", "-pthread", f"-I{inc}"]) == "ok"


def test_mcmc_config_layout_matches_header():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    from aspartik_gb300._native import McmcConfig

    out = _run(cc, LAYOUT_PROGRAM, ".c", ["-std=c11", f"-I{os.path.join(ROOT, 'include')}"])
    size, drift, clock, launch, threads = map(int, out.split())
    assert ct.sizeof(McmcConfig) == size
    assert McmcConfig.da_drift_limit.offset == drift
    assert McmcConfig.clock_categories.offset == clock
    assert McmcConfig.launch.offset == launch
    assert McmcConfig.host_threads.offset == threads
