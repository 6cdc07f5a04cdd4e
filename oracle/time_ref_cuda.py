"""Times the reference's own FP64 CUDA pruning kernel (cuda_partials/
kernels.cu, built into oracle/_ref by oracle/build.py::build_ref) on the
bench's default workload, on the same GPU as this library.  A measurement
of the baseline, not part of the product.

One evaluation of the reference's GammaLikelihood with its CUDA calculator
is one kernel launch per Gamma category over the whole-tree list (each
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
    ref = ref_cuda.RefCudaPartials(0)
    per_cat = []
    try:
        ref.setup(ref_cuda.dna_codes_to_ref(wl["leaves"]), 30)
        for r in cats:
            mats = np.array([[model.transition(d * r) for d in pair] for pair in lengths])
            ref.propose(internals, children, mats, wl["pi"])
            ref.result()
            ref.time_launch(3)  # warm-up
            per_cat.append(ref.time_launch(reps))
    finally:
        ref.close()
    ms = float(sum(per_cat))
    B64 = schedule.algorithmic_bytes(wl["top"], internals, P, C, 4, w=8, e_b=1, w_p=8)
    out = {"workload": workload, "patterns": P, "categories": C,
           "kernel_ms_per_category": [round(x, 4) for x in per_cat],
           "ms_per_evaluation": round(ms, 4),
           "GB_s": round(B64 / (ms * 1e-3) / 1e9, 2),
           "note": "reference cuda_partials kernel, FP64, one thread per pattern, 32-thread "
                   "blocks, one launch per category; device time, inputs resident"}
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    main(*sys.argv[1:])
