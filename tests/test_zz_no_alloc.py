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
the entry point), filled with the layouts documented in include/b3g.h, and the
calls run back to back on different problems (one, two, three, four and eight
categories; the list's `run` fields give the lengths of the runs of mutually
independent entries, so the kernel's batched loads of two and four entries are
used).  Each result is checked against b3g_calculator_propose +
b3g_calculator_log_likelihood on the same inputs, within the parity tolerances
of the other GPU tests (1e-10 relative for the FP64 form, 1e-6 for FP32).  A
last case puts the slots so high in a large caller buffer that their element
indices exceed 2^32 and checks that every value lands in its own slot.  The
file sorts last so that a run stopping at the first failure has already run
every other test.
"""

import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-10, "f32": 1e-6}

# (taxa, sites, seed, categories, Gamma shape)
SPECS = [(24, 400, 5, 4, 0.5), (40, 700, 6, 1, None), (30, 300, 7, 2, 0.7),
         (20, 500, 8, 3, 1.0), (28, 350, 9, 8, 0.4)]


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


def run_lengths(internals, children):
    """`run` of every entry: the entries left, itself included, in its run of
    mutually independent entries (an entry opens a new run when one of its
    children is the output of an entry of the current run)."""
    n = len(internals)
    start, pos, run_of = 0, {}, []
    for i in range(n):
        if any(pos.get(int(ch), -1) >= start for ch in children[i]):
            start = i
        pos[int(internals[i])] = i
        run_of.append(start)
    runs = np.ones(n, dtype=np.uint32)
    for i in range(n - 2, -1, -1):
        if run_of[i + 1] == run_of[i]:
            runs[i] = runs[i + 1] + 1
    return runs


def caller_buffers(torch, c, internals, children, mats, precision, K, slot_base=0,
                   partials=None, scales=None):
    """Device buffers owned by the caller, in the layouts of include/b3g.h.
    Output slot of internal v: slot_base + (v - L) * 2."""
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
        ops[i, 0] = slot_base + (int(v) - L) * 2
        for s in range(2):
            ch = int(children[i, s])
            ops[i, 1 + s] = (nat.TIP | ch) if ch < L else slot_base + (ch - L) * 2
    ops[:, 3] = run_lengths(internals, children)
    tables = np.ones((n, 2, K, 5, 4))
    tables[:, :, :, :4, :] = np.swapaxes(mats, -1, -2)
    weights = np.zeros(ldp, dtype=np.uint32)
    weights[:P] = c.weights
    real = torch.float64 if precision == "f64" else torch.float32
    dev = torch.device("cuda", 0)
    bufs = {
        "tips": torch.from_numpy(tips).to(dev),
        "partials": partials if partials is not None else
        torch.zeros((2 * I, K, ldp, 4), dtype=real, device=dev),
        "scales": scales if scales is not None else
        torch.zeros((2 * I, K, ldp), dtype=torch.int32, device=dev),
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
def test_noalloc_matches_calculator_on_calls_in_a_row(precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from aspartik_gb300 import _native as nat

    problems = [problem(*s) for s in SPECS]
    expected = [existing_entry(c, i, ch, m, precision, s[3])
                for (c, i, ch, m), s in zip(problems, SPECS)]
    # the lists hold runs of two and more independent entries
    assert max(int(run_lengths(i, ch).max()) for _, i, ch, _ in problems) >= 4

    torch.cuda.init()
    prepared = [caller_buffers(torch, c, i, ch, m, precision, s[3])
                for (c, i, ch, m), s in zip(problems, SPECS)]
    stream = torch.cuda.current_stream(0).cuda_stream
    torch.cuda.synchronize()
    for _, desc in prepared:  # calls in a row, no synchronisation between
        nat.check(nat.lib.b3g_prune_noalloc(ct.byref(desc), ct.c_void_p(stream)))
    torch.cuda.synchronize()
    for (bufs, _), want, s in zip(prepared, expected, SPECS):
        got = float(bufs["lnl"].cpu()[0])
        assert got == pytest.approx(want, rel=TOL[precision]), s


def test_noalloc_slot_ids_past_32_bit_element_indices():
    """Slots at 2^25 and above with one category and 128 padded patterns:
    slot * C * ldp reaches 2^32 partial vectors, so a 32-bit element index
    would wrap around to the low slots.  Every output must land in its own
    high slot (equal to the same list walked in low slots) and the low slots
    must stay untouched.  Needs ~80 GiB of free device memory."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from aspartik_gb300 import _native as nat

    free, _ = torch.cuda.mem_get_info(0)
    c, internals, children, mats = problem(16, 100, 11, 1, None)
    L, P = c.leaves.shape
    ldp = 128
    assert P <= ldp
    base = 1 << 25  # base * C * ldp = 2^32 partial vectors
    slots = base + 2 * (L - 1)
    need = slots * ldp * (16 + 4)
    if free < need + (8 << 30):
        pytest.skip(f"needs {need / 2**30:.0f} GiB free, {free / 2**30:.0f} GiB available")
    want = existing_entry(c, internals, children, mats, "f32", 1)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(0).cuda_stream

    low_bufs, low_desc = caller_buffers(torch, c, internals, children, mats, "f32", 1)
    nat.check(nat.lib.b3g_prune_noalloc(ct.byref(low_desc), ct.c_void_p(stream)))

    # caller-owned large buffers: only the low slots (where wrapped indices
    # would land) and the high slots the list writes are initialised
    partials = torch.empty((slots, 1, ldp, 4), dtype=torch.float32, device=dev)
    scales = torch.empty((slots, 1, ldp), dtype=torch.int32, device=dev)
    partials[:2 * (L - 1)].zero_()
    scales[:2 * (L - 1)].zero_()
    partials[base:].fill_(-1.0)
    scales[base:].fill_(-1)
    high_bufs, high_desc = caller_buffers(torch, c, internals, children, mats, "f32", 1,
                                          slot_base=base, partials=partials, scales=scales)
    nat.check(nat.lib.b3g_prune_noalloc(ct.byref(high_desc), ct.c_void_p(stream)))
    torch.cuda.synchronize()
    try:
        assert float(high_bufs["lnl"].cpu()[0]) == pytest.approx(want, rel=TOL["f32"])
        assert float(low_bufs["lnl"].cpu()[0]) == pytest.approx(want, rel=TOL["f32"])
        written = [(int(v) - L) * 2 for v in internals]
        hi = partials[base:].cpu().numpy()
        lo_ref = low_bufs["partials"].cpu().numpy()
        np.testing.assert_array_equal(hi[written], lo_ref[written])
        np.testing.assert_array_equal(scales[base:].cpu().numpy()[written],
                                      low_bufs["scales"].cpu().numpy()[written])
        # nothing wrapped around into the low slots
        assert not partials[:2 * (L - 1)].any().item()
        assert not scales[:2 * (L - 1)].any().item()
    finally:
        del partials, scales, high_bufs
        torch.cuda.empty_cache()


def test_noalloc_rejects_problems_over_its_maximum():
    from aspartik_gb300 import _native as nat

    fake = 256  # never dereferenced: the size check comes first
    too_many = (nat.NOALLOC_MAX_BLOCKS + 1) * 128
    desc = nat.PruneBuffers(*([fake] * 9), 1, too_many, 1, nat.PRECISION_F64, 30, 0)
    st = nat.lib.b3g_prune_noalloc(ct.byref(desc), None)
    assert st == nat.B3G_ERR_INVALID_ARGUMENT
    assert b"maximum" in nat.lib.b3g_last_error()
