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
