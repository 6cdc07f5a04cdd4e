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


@pytest.mark.parametrize("launch,da", [("streams", 0), ("streams", 300), ("batch", 0)])
def test_host_threads_leave_the_results_unchanged(launch, da):
    """The same run on the calling thread alone and on three or eight host
    threads (chain i on thread i % threads): every chain's trace, the cold
    chain's samples, the operator, swap and delayed-acceptance statistics
    are identical."""
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    c = dna_case(20, 400, seed=41, model="gtr", alpha=0.5, num_categories=4,
                 root_height=0.7)
    runs = []
    for threads in (1, 3, 8):
        s = McmcSettings(model="gtr", precision="f32", num_categories=4, num_chains=8,
                         heat=0.05, swap_every=7, seed=13, sample_every=5, tune_every=200,
                         launch=launch, host_threads=threads, da_pilot_steps=da,
                         da_epochs=5, da_hidden=64)
        m = Mcmc(c.leaves, c.weights, c.tree.parents, c.tree.heights, s)
        m.set_parameters(rates=np.ones(6), frequencies=np.full(4, 0.25), alpha=0.5,
                         birth_rate=1.0)
        m.run(1500)
        assert m.check() < 1e-12
        runs.append(dict(traces=[m.trace("lnl", chain=i) for i in range(8)],
                         heights=m.samples()["heights"], ops=m.operator_stats(),
                         swaps=m.swaps(), da=m.da_stats()))
        m.close()
    base = runs[0]
    if da:
        assert base["da"]["pilot_pairs"] > 0
    for other in runs[1:]:
        for a, b in zip(base["traces"], other["traces"]):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(base["heights"], other["heights"])
        assert base["ops"] == other["ops"]
        assert base["swaps"] == other["swaps"]
        assert base["da"] == other["da"]


@pytest.mark.parametrize("da", [0, 300])
def test_independent_stepping_is_deterministic(da):
    """Uncoupled chains advancing on their own between synchronisation
    points (operator tuning, the pilot's end): the same traces, samples and
    operator and delayed-acceptance statistics on 1, 3 and 8 host threads
    and whether the steps come in one call or in several; the incremental
    likelihood stays exact."""
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    c = dna_case(20, 400, seed=43, model="gtr", alpha=0.5, num_categories=4,
                 root_height=0.7)
    runs = []
    for threads, split in ((1, (1500,)), (3, (1500,)), (8, (700, 45, 755))):
        s = McmcSettings(model="gtr", precision="f32", num_categories=4, num_chains=8,
                         heat=0.0, swap_every=0, seed=17, sample_every=5, tune_every=200,
                         launch="independent", host_threads=threads, da_pilot_steps=da,
                         da_epochs=5, da_hidden=64)
        m = Mcmc(c.leaves, c.weights, c.tree.parents, c.tree.heights, s)
        m.set_parameters(rates=np.ones(6), frequencies=np.full(4, 0.25), alpha=0.5,
                         birth_rate=1.0)
        for k in split:
            m.run(k)
        assert m.check() < 1e-12
        runs.append(dict(traces=[m.trace("lnl", chain=i) for i in range(8)],
                         heights=m.samples()["heights"], ops=m.operator_stats(),
                         da=m.da_stats()))
        m.close()
    base = runs[0]
    assert base["traces"][0].size == 300
    if da:
        assert base["da"]["pilot_pairs"] > 0 and base["da"]["exact_evaluations"] > 0
    for other in runs[1:]:
        for a, b in zip(base["traces"], other["traces"]):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(base["heights"], other["heights"])
        assert base["ops"] == other["ops"]
        assert base["da"] == other["da"]


def test_independent_stepping_with_swaps_is_deterministic():
    """MC3 chains advancing on their own between swap attempts: the same
    traces (each chain's and the cold chain's), swaps and temperatures on 1
    and 4 host threads and over several calls as the lockstep driver's
    (without delayed acceptance the statistics merge changes nothing), and
    the ladder stays a permutation of the temperatures."""
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    probs = problems()
    runs = []
    for launch, threads, split in (("independent", 1, (800,)), ("independent", 4, (333, 467)),
                                   ("streams", 2, (800,))):
        s = McmcSettings(model="gtr", precision="f32", num_categories=4, num_chains=6,
                         heat=HEAT, swap_every=7, seed=19, sample_every=5, tune_every=100,
                         launch=launch, host_threads=threads)
        m = Mcmc.multi(probs, s)
        m.set_parameters(rates=np.ones(6), frequencies=np.full(4, 0.25), alpha=0.5,
                         birth_rate=1.0)
        for k in split:
            m.run(k)
        assert m.check() < 1e-12
        betas = [m.chain_state(i)[3] for i in range(6)]
        runs.append(dict(traces=[m.trace("lnl", chain=i) for i in range(6)],
                         cold=m.trace("lnl"), swaps=m.swaps(), betas=betas,
                         ops=m.operator_stats()))
        m.close()
    a = runs[0]
    assert a["swaps"][0] == 2 * (800 // 7) and a["swaps"][1] > 0
    for b in runs[1:]:
        assert a["swaps"] == b["swaps"] and a["betas"] == b["betas"] and a["ops"] == b["ops"]
        np.testing.assert_array_equal(a["cold"], b["cold"])
        for x, y in zip(a["traces"], b["traces"]):
            np.testing.assert_array_equal(x, y)
    ladder = sorted(1.0 / (1.0 + HEAT * k) for k in range(3))
    for g in range(2):
        np.testing.assert_allclose(sorted(a["betas"][3 * g:3 * g + 3]), ladder, rtol=0,
                                   atol=1e-15)
