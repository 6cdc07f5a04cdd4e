"""The native MCMC driver over several alignments (b3g_mcmc_create_multi):
chains of different taxa and site counts step together, each problem's
chains form its own temperature ladder and swap only among themselves, every
chain's incremental likelihood equals a fresh full evaluation, and the
batched launch mode (one graph replay per step for every chain) keeps the
same invariants."""

import numpy as np
import pytest

from tests.cases import dna_case

pytestmark = pytest.mark.gpu

HEAT = 0.1


def problems():
    out = []
    for L, N, seed in ((14, 300, 31), (27, 500, 32)):
        c = dna_case(L, N, seed=seed, model="gtr", alpha=0.5, num_categories=4,
                     root_height=0.8)
        out.append((c.leaves, c.weights, c.tree.parents, c.tree.heights))
    return out


@pytest.mark.parametrize("precision,launch", [("f64", "streams"), ("f32", "streams"),
                                              ("f32", "batch")])
def test_chains_over_several_alignments(precision, launch):
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    probs = problems()
    group = 3
    s = McmcSettings(model="gtr", precision=precision, num_categories=4,
                     num_chains=group * len(probs), heat=HEAT, swap_every=5, seed=9,
                     sample_every=10, launch=launch)
    m = Mcmc.multi(probs, s)
    m.set_parameters(rates=np.ones(6), frequencies=np.full(4, 0.25), alpha=0.5,
                     birth_rate=1.0)
    for _ in range(4):
        m.run(500)
        assert m.check() < 1e-12
    stats = m.launch_stats()
    assert stats["batched"] == (launch == "batch")
    if launch == "batch":
        assert stats["launches"] > 0 and stats["device_ms"] > 0.0
    tried, accepted = m.swaps()
    assert tried == len(probs) * (2000 // 5)  # one attempt per problem each time
    assert accepted > 0
    ladder = sorted(1.0 / (1.0 + HEAT * k) for k in range(group))
    for g, (leaves, _, parents, _) in enumerate(probs):
        betas = []
        for i in range(g * group, (g + 1) * group):
            par, hei, lnl, beta = m.chain_state(i)
            assert par.size == parents.size == 2 * leaves.shape[0] - 1
            assert np.isfinite(lnl) and lnl < 0.0
            betas.append(beta)
        np.testing.assert_allclose(sorted(betas), ladder, rtol=0, atol=1e-15)
    # every chain's trace, the cold chain's samples from problem 0
    for i in range(s.num_chains):
        assert m.trace("lnl", chain=i).size == 200
    assert m.samples()["parents"].shape[1] == probs[0][2].size
    m.close()


def test_problems_must_divide_the_chains():
    from aspartik_gb300._native import B3GError
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    s = McmcSettings(model="gtr", precision="f32", num_categories=4, num_chains=5)
    with pytest.raises(B3GError):
        Mcmc.multi(problems(), s)
