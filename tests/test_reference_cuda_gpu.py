"""The reference's own FP64 CUDA calculators (crates/b3/src/calculator/
cuda_partials/kernels.cu and cuda_propagations/kernels.cu, compiled from the
reference tree into oracle/_ref/) run beside the CPU oracle and this
library's FP64 calculator on the same inputs: per-pattern log-likelihoods
of full evaluations with the calculator-level interface (given transition
matrices, cpu4.rs:39-76 / cuda_partials/mod.rs:63-100), over tip codes with
gaps and ambiguity, deep trees and scale constants that force rescaling.
This pins the oracle to values the reference itself computes."""

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import dna_case
from tests.test_gpu_parity import full, lists_and_lengths, make_gpu

pytestmark = pytest.mark.gpu

CASES = [  # taxa, sites, model, seed, root height, gaps, ambiguous, rate, scale_ln
    (16, 1000, "hky", 1, 0.5, 0.0, 0.0, 1.0, 30),
    (40, 2000, "gtr", 2, 1.0, 0.03, 0.02, 0.3, 30),
    (40, 2000, "gtr", 2, 1.0, 0.03, 0.02, 2.5, 3),
    (128, 600, "gtr", 3, 3.0, 0.01, 0.0, 1.7, 30),
    (200, 400, "hky", 4, 2.0, 0.05, 0.05, 1.0, 3),
]


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_cuda

    if not ref_cuda.available():
        pytest.skip("the reference kernel is built only where the reference tree is present")
    r = ref_cuda.RefCudaPartials(0)
    yield r
    r.close()


@pytest.mark.parametrize("case", CASES)
def test_reference_kernel_matches_oracle_and_library(ref, case):
    from oracle.ref_cuda import dna_codes_to_ref

    L, N, model_name, seed, rh, gaps, amb, rate, scale_ln = case
    c = dna_case(L, N, seed=seed, model=model_name, root_height=rh, gaps=gaps,
                 ambiguous=amb)
    model = O.gtr(c.rates, c.pi) if model_name == "gtr" else O.hky(2.0, c.pi)
    tree = full(c.tree.parents, c.tree.heights)
    internals, children, lengths = lists_and_lengths(tree)
    mats = np.array([[model.transition(d * rate) for d in pair] for pair in lengths])
    P = c.leaves.shape[1]

    want_ref = ref.likelihoods(dna_codes_to_ref(c.leaves), internals, children, mats,
                               model.pi, scale_ln)
    cpu = O.Cpu4Calculator(c.leaves, P, scale_ln, 1)
    cpu.propose(internals, children, mats, model.pi)
    oracle = np.array(cpu.likelihoods())
    g = make_gpu(c.leaves, c.weights, 1, "f64", scale_ln)
    g.propose(internals, children, mats, model.pi)
    mine = g.likelihoods()
    g.close()

    assert np.isfinite(want_ref).all()
    np.testing.assert_allclose(oracle, want_ref, rtol=1e-12, atol=0.0)
    # the reference's default GPU calculator (propagations) on the same inputs
    from oracle import ref_cuda

    if ref_cuda.propagations_available():
        prop = ref_cuda.RefCudaPropagations(0)
        try:
            prop.setup(c.leaves, scale_ln)
            nodes, k, pch, pmats = ref_cuda.propagation_inputs(c.tree, model, rate, L)
            prop.propose(nodes, k, pch, pmats, model.pi)
            got_prop = prop.result()
        finally:
            prop.close()
        np.testing.assert_allclose(oracle, got_prop, rtol=1e-12, atol=0.0)
    np.testing.assert_allclose(mine, want_ref, rtol=1e-12, atol=0.0)
    # and the weighted sums
    w = c.weights.astype(np.float64)
    assert float(mine @ w) == pytest.approx(float(want_ref @ w), rel=1e-12)
