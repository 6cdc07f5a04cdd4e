"""Generates tests/golden/ref_cuda_partials.npz: outputs of the reference's
own FP64 CUDA calculators (crates/b3/src/calculator/cuda_partials/
kernels.cu and cuda_propagations/kernels.cu, built into oracle/_ref/ by
oracle/build.py::build_ref) on seeded inputs, stored with those inputs so
that the CPU tests can pin the oracle to them without a GPU.

Needs a GPU and the built cubin.  Run on a GPU machine:
    python tests/golden/make_ref_cuda_golden.py [output path]
"""

from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from oracle import ref_cuda  # noqa: E402
from tests.cases import dna_case  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_cuda_partials.npz")

# name, taxa, sites, model, seed, root height, gaps, ambiguous, rate, scale_ln
CASES = [
    ("hky16", 16, 1000, "hky", 1, 0.5, 0.0, 0.0, 1.0, 30),
    ("gtr40_slow", 40, 2000, "gtr", 2, 1.0, 0.03, 0.02, 0.3, 30),
    ("gtr40_fast_scale3", 40, 2000, "gtr", 2, 1.0, 0.03, 0.02, 2.5, 3),
    ("gtr128_deep", 128, 600, "gtr", 3, 3.0, 0.01, 0.0, 1.7, 30),
    ("hky200_scale3", 200, 400, "hky", 4, 2.0, 0.05, 0.05, 1.0, 3),
]


def inputs(case):
    _, L, N, model_name, seed, rh, gaps, amb, rate, scale_ln = case
    c = dna_case(L, N, seed=seed, model=model_name, root_height=rh, gaps=gaps, ambiguous=amb)
    model = O.gtr(c.rates, c.pi) if model_name == "gtr" else O.hky(2.0, c.pi)
    t = O.DatedTree(c.tree.parents, c.tree.heights)
    t.mark_all_edges_updated()
    internals, children = t.partials_lists()
    lengths = np.array([[t.edge_length(int(a)), t.edge_length(int(b))] for a, b in children])
    mats = np.array([[model.transition(d * rate) for d in pair] for pair in lengths])
    prop = ref_cuda.propagation_inputs(c.tree, model, rate, L)
    return c.leaves, np.asarray(internals), np.asarray(children), mats, model.pi, scale_ln, prop


def main(out: str = OUT) -> None:
    ref = ref_cuda.RefCudaPartials(0)
    prop = ref_cuda.RefCudaPropagations(0)
    arrays = {}
    try:
        for case in CASES:
            name = case[0]
            leaves, internals, children, mats, pi, scale_ln, pin = inputs(case)
            lnl = ref.likelihoods(ref_cuda.dna_codes_to_ref(leaves), internals, children, mats,
                                  pi, scale_ln)
            nodes, k, pch, pmats = pin
            prop.setup(leaves, scale_ln)
            prop.propose(nodes, k, pch, pmats, pi)
            lnl_prop = prop.result()
            prop.free()
            arrays.update({f"{name}/leaves": leaves, f"{name}/internals": internals,
                           f"{name}/children": children, f"{name}/matrices": mats,
                           f"{name}/frequencies": pi, f"{name}/scale_ln": np.int64(scale_ln),
                           f"{name}/site_lnl": lnl, f"{name}/site_lnl_propagations": lnl_prop})
    finally:
        ref.close()
        prop.close()
    np.savez_compressed(out, **arrays)
    print(f"wrote {out}")


if __name__ == "__main__":
    main(*sys.argv[1:])
