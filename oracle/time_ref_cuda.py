"""Times the reference's own FP64 CUDA calculators (cuda_partials and
cuda_propagations kernels, built into oracle/_ref by
oracle/build.py::build_ref) on the bench's default workload, on the same
GPU as this library.  A measurement of the baseline, not part of the
product.

One evaluation of the reference's GammaLikelihood with a CUDA calculator is
one calculator evaluation per Gamma category over the whole tree (each
category a separate calculator, likelihood/gamma.rs:97-169), plus the
host-side log-sum-exp; the script reports the device time of the launches
(inputs resident, as for this library's `value`), per category and per
evaluation, and the same algorithmic bytes per evaluation as bench.py with
the reference's FP64 element and one-byte scale flags.

Run on a GPU machine: python oracle/time_ref_cuda.py [workload]
"""

from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from aspartik_gb300 import schedule  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import ref_cuda  # noqa: E402


def main(workload: str = bench.DEFAULT_WORKLOAD, reps: int = 20) -> dict:
    wl = bench.make_workload(workload)
    spec = wl["spec"]
    C = spec["categories"]
    model = O.gtr(wl["rates"], wl["pi"])
    cats = O.gamma_categories(spec["alpha"], C) if spec["alpha"] else np.ones(1)
    internals, children, lengths = wl["top"].full()
    P = int(wl["leaves"].shape[1])
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_ref_cuda_golden import propagation_inputs

    L = int(wl["leaves"].shape[0])
    part = ref_cuda.RefCudaPartials(0)
    per_cat, per_cat_prop = [], []
    try:
        part.setup(ref_cuda.dna_codes_to_ref(wl["leaves"]), 30)
        for r in cats:
            mats = np.array([[model.transition(d * r) for d in pair] for pair in lengths])
            part.propose(internals, children, mats, wl["pi"])
            part.result()
            part.time_last(3)  # warm-up
            per_cat.append(part.time_last(reps))
    finally:
        part.close()
    prop = ref_cuda.RefCudaPropagations(0)
    try:
        prop.setup(wl["leaves"], 30)
        for r in cats:
            nodes, k, pch, pmats = propagation_inputs(wl["tree"], model, r, L)
            prop.propose(nodes, k, pch, pmats, wl["pi"])
            prop.result()
            prop.time_last(3)
            per_cat_prop.append(prop.time_last(reps))
    finally:
        prop.close()
    ms, ms_prop = float(sum(per_cat)), float(sum(per_cat_prop))
    B64 = schedule.algorithmic_bytes(wl["top"], internals, P, C, 4, w=8, e_b=1, w_p=8)
    out = {"workload": workload, "patterns": P, "categories": C,
           "partials": {"kernel_ms_per_category": [round(x, 4) for x in per_cat],
                        "ms_per_evaluation": round(ms, 4),
                        "GB_s": round(B64 / (ms * 1e-3) / 1e9, 2)},
           "propagations": {"kernel_ms_per_category": [round(x, 4) for x in per_cat_prop],
                            "ms_per_evaluation": round(ms_prop, 4),
                            "GB_s": round(B64 / (ms_prop * 1e-3) / 1e9, 2)},
           "note": "reference CUDA calculators, FP64: partials (one launch per category, one "
                   "thread per pattern) and propagations, the default (leaf, propagation and "
                   "root kernels per category, four threads per pattern); device time, "
                   "inputs resident; GB/s by the FP64 byte formula"}
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main(*sys.argv[1:])
