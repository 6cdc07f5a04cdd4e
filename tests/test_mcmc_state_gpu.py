"""Checkpoints of the native MCMC driver (b3g_mcmc_dump / b3g_mcmc_load,
the counterpart of Mcmc::dump, mcmc.rs:251-268): a driver that loads a
checkpoint continues exactly as the dumped one does (same traces, trees,
operator statistics, swaps and a byte-identical second checkpoint), with
several heated chains, in both forms and with a relaxed clock; corrupted,
truncated or foreign checkpoints are refused and leave the driver usable."""

import numpy as np
import pytest

from aspartik_gb300._native import B3G_ERR_INVALID_ARGUMENT, B3G_ERR_STATE, B3GError
from tests.cases import dna_case

pytestmark = pytest.mark.gpu

FIELDS = ("lnl", "prior", "posterior", "root_height", "kappa_or_rate0", "alpha",
          "tree_length", "clock_sd")


def fresh(c, clock=0, **kw):
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    s = McmcSettings(model="gtr", num_categories=4, sample_every=5, tune_every=100, seed=11,
                     clock_categories=clock, **kw)
    m = Mcmc(c.leaves, c.weights, c.tree.parents, c.tree.heights, s)
    if clock:
        m.set_clock(0.3)
    m.set_parameters(rates=np.ones(6), frequencies=c.pi, alpha=0.5, birth_rate=2.0)
    return m


@pytest.mark.parametrize("precision,clock,chains", [("f32", 0, 3), ("f64", 0, 1),
                                                     ("f32", 4, 1)])
def test_checkpoint_continues_bit_for_bit(precision, clock, chains):
    c = dna_case(20, 600, seed=33, model="gtr", alpha=0.5, num_categories=4)
    kw = dict(precision=precision, num_chains=chains, heat=0.2 if chains > 1 else 0.0,
              swap_every=5 if chains > 1 else 0)
    a = fresh(c, clock, **kw)
    a.run(700)
    state = a.dump()
    done = {k: a.trace(k).size for k in FIELDS}
    a.run(700)
    b = fresh(c, clock, **kw)
    b.load(state)
    b.run(700)
    for k in FIELDS:
        np.testing.assert_array_equal(a.trace(k)[done[k]:], b.trace(k), err_msg=k)
    for ch in range(chains):
        pa, ha, la, ba = a.chain_state(ch)
        pb, hb, lb, bb = b.chain_state(ch)
        assert np.array_equal(pa, pb) and np.array_equal(ha, hb)
        assert la == lb and ba == bb
    assert a.operator_stats() == b.operator_stats()
    assert a.swaps() == b.swaps()
    assert b.check() < 1e-12
    assert a.dump() == b.dump()
    a.close()
    b.close()


def test_bad_checkpoints_are_refused():
    c = dna_case(12, 300, seed=34, model="gtr", alpha=0.5, num_categories=4)
    a = fresh(c, precision="f32")
    a.run(50)
    state = a.dump()
    b = fresh(c, precision="f32")
    corrupt = bytearray(state)
    corrupt[40] ^= 0x5A
    for bad in (bytes(corrupt), state[:-9], state[:20], b"not a checkpoint at all"):
        with pytest.raises(B3GError) as e:
            b.load(bad)
        assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    other = fresh(c, precision="f32", num_chains=2, heat=0.1, swap_every=5)
    with pytest.raises(B3GError) as e:
        other.load(state)
    assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    # still usable, and a good checkpoint still loads
    b.run(20)
    b.load(state)
    b.run(20)
    assert b.check() < 1e-12
    da = fresh(c, precision="f32", da_pilot_steps=50)
    with pytest.raises(B3GError) as e:
        da.dump()
    assert e.value.status == B3G_ERR_STATE
    for m in (a, b, other, da):
        m.close()


# A reference configuration's order: GTR + Gamma with a Yule tree
# (parameters as python/aspartik/b3/config lists them for such a run) and
# its scheduler's operators with their tuning flags.
GTR_PARAMS = ["birth_rate", "rates", "frequencies", "alpha", "tree"]
CLOCK_PARAMS = ["birth_rate", "rates", "frequencies", "alpha", "clock_sd",
                "clock_categories", "tree"]
OPS = [("tree_scale", True), ("subtree_slide", True), ("narrow_exchange", False),
       ("wide_exchange", False), ("node_slide", False), ("root_slide", True),
       ("up_down", True), ("scale_alpha", True), ("scale_birth_rate", True),
       ("delta_rates", True), ("delta_frequencies", True)]


def parse_state(state: bytes, params, ops, nodes):
    from tests.verbatim_ref import STATE_TAG, STATE_VERSION, Reader

    r = Reader(state)
    assert r.tag(4) == STATE_TAG
    assert r.prim("u32") == STATE_VERSION
    out = {"step": r.prim("u64"), "posterior": r.prim("f64")}
    sizes = {"rates": 6, "frequencies": 4, "clock_categories": nodes}
    for p in params:
        if p == "tree":
            out["parents"] = r.slice("u32")
            out["heights"] = r.slice("f64")
        elif p == "clock_categories":
            out[p] = [r.prim("u32") for _ in range(nodes)]
        elif p in sizes:
            out[p] = [r.prim("f64") for _ in range(sizes[p])]
        else:
            out[p] = r.prim("f64")
    out["ops"] = []
    for _, tuned in ops:
        a, rj = r.prim("u32"), r.prim("u32")
        out["ops"].append((a, rj, r.prim("f64") if tuned else None))
    out["rng"] = (r.u128(), r.u128())
    assert r.left() == 0
    return out


@pytest.mark.parametrize("clock", [0, 4])
def test_reference_layout_state_round_trip(clock):
    """A chain's state in the reference's state-file layout: the bytes parse
    under the restated reference reader with the chain's tree, parameters,
    step, posterior and operator tunings; a fresh driver that loads them
    holds the same tree and parameters, re-evaluates the same likelihood,
    and keeps stepping with its incremental likelihood exact."""
    from aspartik_gb300.mcmc import OPERATORS

    c = dna_case(18, 500, seed=35, model="gtr", alpha=0.5, num_categories=4)
    params = CLOCK_PARAMS if clock else GTR_PARAMS
    ops = OPS + ([("relaxed_category", False), ("scale_clock_sd", True)] if clock else [])
    a = fresh(c, clock, precision="f32")
    a.run(600)  # a multiple of sample_every: the last sample is the state
    state = a.dump_verbatim(params, ops)
    nodes = c.tree.parents.size
    st = parse_state(state, params, ops, nodes)
    par, hei, lnl, _ = a.chain_state(0)
    smp = a.samples()
    assert st["step"] == 600
    assert st["parents"] == list(par) and st["heights"] == list(hei)
    assert st["posterior"] == pytest.approx(a.trace("posterior")[-1], rel=0, abs=0)
    assert st["rates"] == list(smp["rates"][-1])
    assert st["frequencies"] == list(smp["frequencies"][-1])
    assert st["alpha"] == smp["alpha"][-1] and st["birth_rate"] == smp["birth_rate"][-1]
    if clock:
        assert st["clock_sd"] == smp["clock_sd"][-1]
        assert max(v for i, v in enumerate(st["clock_categories"])
                   if par[i] != 0xFFFFFFFF) < clock
    stats = a.operator_stats()
    for (name, tuned), (acc, rej, tuning) in zip(ops, st["ops"]):
        assert acc + rej <= stats[name]["accepts"] + stats[name]["rejects"]
        if tuned:
            assert tuning == stats[name]["tuning"]

    b = fresh(c, clock, precision="f32")
    b.load_verbatim(state, params, ops)
    pb, hb, lb, _ = b.chain_state(0)
    assert np.array_equal(pb, par) and np.array_equal(hb, hei)
    assert lb == pytest.approx(lnl, rel=1e-12)  # a whole-tree evaluation
    again = b.dump_verbatim(params, ops)
    # all but the posterior (re-evaluated) and the RNG words (reseeded)
    assert again[:16] == state[:16] and again[24:-32] == state[24:-32]
    for name, tuned in ops:
        if tuned:
            assert b.operator_stats()[name]["tuning"] == stats[name]["tuning"]
    b.run(300)
    assert b.check() < 1e-12
    assert b.dump_verbatim(params, ops)[8:16] == (900).to_bytes(8, "little")
    assert OPERATORS  # the names used above are the driver's
    a.close()
    b.close()


def test_reference_layout_states_that_do_not_fit_are_refused():
    """Version 7 in byte 4 (the reference's own version test), a foreign
    tag, a parameter list longer or shorter than the writer's, a tree of
    another size and a short state are refused, and the driver is unchanged."""
    c = dna_case(14, 300, seed=36, model="gtr", alpha=0.5, num_categories=4)
    a = fresh(c, precision="f32")
    a.run(100)
    state = a.dump_verbatim(GTR_PARAMS, OPS)
    b = fresh(c, precision="f32")
    before = b.chain_state(0)
    v7 = state[:4] + b"\x07" + state[5:]
    with pytest.raises(B3GError, match="protocol version v7 is incompatible"):
        b.load_verbatim(v7, GTR_PARAMS, OPS)
    for bad, params in ((b"XXXX" + state[4:], GTR_PARAMS), (state, GTR_PARAMS[:-1]),
                        (state, GTR_PARAMS + ["birth_rate"]), (state[:-40], GTR_PARAMS),
                        (state + b"\0" * 8, GTR_PARAMS)):
        with pytest.raises(B3GError) as e:
            b.load_verbatim(bad, params, OPS)
        assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    small = dna_case(10, 300, seed=37, model="gtr", alpha=0.5, num_categories=4)
    s = fresh(small, precision="f32")
    with pytest.raises(B3GError) as e:
        s.load_verbatim(state, GTR_PARAMS, OPS)
    assert e.value.status == B3G_ERR_INVALID_ARGUMENT
    after = b.chain_state(0)
    assert np.array_equal(before[0], after[0]) and before[2] == after[2]
    with pytest.raises(B3GError):
        a.dump_verbatim(["kappa"], [])  # kappa belongs to HKY chains
    for m in (a, b, s):
        m.close()
