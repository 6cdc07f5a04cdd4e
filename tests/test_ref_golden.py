"""The CPU oracle pinned to the reference itself: per-pattern log-likelihoods
that the reference's own FP64 CUDA calculators (crates/b3/src/calculator/
cuda_partials/kernels.cu and cuda_propagations/kernels.cu, compiled from
the reference tree) wrote on a GB300, stored with their inputs in tests/golden/ref_cuda_partials.npz
by tests/golden/make_ref_cuda_golden.py.  The oracle's restatement of
cpu4.rs must give the same values from the same inputs (FP64, 1e-12
relative: the two differ only in the compiler's contraction of the dot
products)."""

import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_cuda_partials.npz")


def names():
    g = np.load(GOLDEN)
    return sorted({k.split("/")[0] for k in g.files})


@pytest.mark.parametrize("name", names())
def test_oracle_reproduces_reference_kernel(name):
    g = np.load(GOLDEN)
    leaves = g[f"{name}/leaves"]
    P = leaves.shape[1]
    calc = O.Cpu4Calculator(leaves, P, int(g[f"{name}/scale_ln"]), 1)
    calc.propose(g[f"{name}/internals"], g[f"{name}/children"], g[f"{name}/matrices"],
                 g[f"{name}/frequencies"])
    got = np.array(calc.likelihoods())
    want = g[f"{name}/site_lnl"]
    assert np.isfinite(want).all()
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=0.0)
    # the reference's default GPU calculator (propagations), same inputs
    if f"{name}/site_lnl_propagations" in g.files:
        np.testing.assert_allclose(got, g[f"{name}/site_lnl_propagations"], rtol=1e-12,
                                   atol=0.0)


def test_fixture_inputs_regenerate_here():
    """The seeded inputs of the fixtures come out the same on this machine,
    so the fixtures and the GPU test of the live kernel describe the same
    cases."""
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_ref_cuda_golden import CASES, inputs

    g = np.load(GOLDEN)
    for case in CASES:
        leaves, internals, children, mats, pi, _, _ = inputs(case)
        name = case[0]
        assert np.array_equal(leaves, g[f"{name}/leaves"]), name
        assert np.array_equal(internals, g[f"{name}/internals"]), name
        np.testing.assert_allclose(mats, g[f"{name}/matrices"], rtol=1e-14, atol=1e-16)
