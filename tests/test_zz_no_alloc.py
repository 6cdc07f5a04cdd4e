"""b3g_prune_noalloc, the allocation-free entry point, against the
calculator's own path.

Some callers cannot let this library allocate device memory: a program whose
device buffers all come from its own allocator or pool (the way the
reference's CUDA calculators own their buffers), or an MCMC step that is being
recorded into a CUDA graph or must never stall the device on cudaMalloc or
cudaFree.  For them the library offers b3g_prune_noalloc: the caller owns every
input and output buffer, and the call's only working memory is a fixed array
compiled into the library.

Here the caller-owned buffers are allocated by torch before the calls (not by
the entry point), filled with the layouts documented in include/b3g.h, and two
calls run back to back on two different problems.  Each result is checked
against b3g_calculator_propose + b3g_calculator_log_likelihood on the same
inputs, within the parity tolerances of the other GPU tests (1e-10 relative for
the FP64 form, 1e-6 for FP32).  The file sorts last so that a run stopping at
the first failure has already run every other test.
"""

import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-10, "f32": 1e-6}


def problem(num_leaves, num_sites, seed, K, alpha):
    from oracle import oracle as O
    from tests.cases import dna_case

    c = dna_case(num_leaves, num_sites, seed=seed, model="gtr", root_height=1.0,
                 alpha=alpha, num_categories=K)
    tree = O.DatedTree(c.tree.parents, c.tree.heights)
    tree.mark_all_edges_updated()
    internals, children = tree.partials_lists()
    model = O.gtr(c.rates, c.pi)
    rates = O.gamma_categories(alpha, K) if K > 1 else np.ones(1)
    lengths = np.array([[tree.edge_length(int(a)), tree.edge_length(int(b))]
                        for a, b in children])
    mats = np.zeros((len(internals), 2, K, 4, 4))
    for i in range(len(internals)):
        for s in range(2):
            for k in range(K):
                mats[i, s, k] = model.transition(lengths[i, s] * rates[k])
    return c, internals, children, mats


def existing_entry(c, internals, children, mats, precision, K):
    from aspartik_gb300.calculator import Calculator

    calc = Calculator.GB300(0, precision).make4(c.leaves, c.leaves.shape[1], num_categories=K)
    calc.set_weights(c.weights)
    calc.propose(internals, children, mats, c.pi)
    lnl = calc.log_likelihood()
    calc.close()
    return lnl


def caller_buffers(torch, c, internals, children, mats, precision, K):
    """Device buffers owned by the caller, in the layouts of include/b3g.h."""
    from aspartik_gb300 import _native as nat

    L, P = c.leaves.shape
    ldp = (P + 127) // 128 * 128
    I = L - 1
    remap = np.full(256, 4, dtype=np.uint8)
    remap[[1, 2, 4, 8]] = [0, 1, 2, 3]
    tips = np.full((L, ldp), 4, dtype=np.uint8)
    tips[:, :P] = remap[c.leaves]
    n = len(internals)
    ops = np.zeros((n, 4), dtype=np.uint32)
    for i, v in enumerate(internals):
        ops[i, 0] = (int(v) - L) * 2
        for s in range(2):
            ch = int(children[i, s])
            ops[i, 1 + s] = (nat.TIP | ch) if ch < L else (ch - L) * 2
        ops[i, 3] = 1
    tables = np.ones((n, 2, K, 5, 4))
    tables[:, :, :, :4, :] = np.swapaxes(mats, -1, -2)
    weights = np.zeros(ldp, dtype=np.uint32)
    weights[:P] = c.weights
    real = torch.float64 if precision == "f64" else torch.float32
    dev = torch.device("cuda", 0)
    bufs = {
        "tips": torch.from_numpy(tips).to(dev),
        "partials": torch.zeros((2 * I, K, ldp, 4), dtype=real, device=dev),
        "scales": torch.zeros((2 * I, K, ldp), dtype=torch.int32, device=dev),
        "ops": torch.from_numpy(ops.view(np.int32)).to(dev),
        "tables": torch.from_numpy(tables).to(dev, real),
        "frequencies": torch.from_numpy(np.ascontiguousarray(c.pi)).to(dev),
        "weights": torch.from_numpy(weights.view(np.int32)).to(dev),
        "site_lnl": torch.zeros(ldp, dtype=torch.float64, device=dev),
        "lnl": torch.zeros(1, dtype=torch.float64, device=dev),
    }
    desc = nat.PruneBuffers(
        *(bufs[k].data_ptr() for k in ("tips", "partials", "scales", "ops", "tables",
                                       "frequencies", "weights", "site_lnl", "lnl")),
        n, ldp, K, nat.PRECISION_F64 if precision == "f64" else nat.PRECISION_F32, 30, 0)
    return bufs, desc


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_noalloc_matches_calculator_on_two_calls_in_a_row(precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from aspartik_gb300 import _native as nat

    specs = [(24, 400, 5, 4, 0.5), (40, 700, 6, 1, None)]
    problems = [problem(*s) for s in specs]
    expected = [existing_entry(c, i, ch, m, precision, s[3])
                for (c, i, ch, m), s in zip(problems, specs)]

    torch.cuda.init()
    prepared = [caller_buffers(torch, c, i, ch, m, precision, s[3])
                for (c, i, ch, m), s in zip(problems, specs)]
    stream = torch.cuda.current_stream(0).cuda_stream
    torch.cuda.synchronize()
    for _, desc in prepared:  # two calls in a row, no synchronisation between
        nat.check(nat.lib.b3g_prune_noalloc(ct.byref(desc), ct.c_void_p(stream)))
    torch.cuda.synchronize()
    for (bufs, _), want in zip(prepared, expected):
        got = float(bufs["lnl"].cpu()[0])
        assert got == pytest.approx(want, rel=TOL[precision])


def test_noalloc_rejects_problems_over_its_maximum():
    from aspartik_gb300 import _native as nat

    fake = 256  # never dereferenced: the size check comes first
    too_many = (nat.NOALLOC_MAX_BLOCKS + 1) * 128
    desc = nat.PruneBuffers(*([fake] * 9), 1, too_many, 1, nat.PRECISION_F64, 30, 0)
    st = nat.lib.b3g_prune_noalloc(ct.byref(desc), None)
    assert st == nat.B3G_ERR_INVALID_ARGUMENT
    assert b"maximum" in nat.lib.b3g_last_error()
