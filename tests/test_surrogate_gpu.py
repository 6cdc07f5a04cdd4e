"""The surrogate's CUDA forward, backward and training kernels against the
numpy oracle, and delayed-acceptance MCMC: the target distribution is kept
and the trained network saves exact likelihood evaluations."""

import numpy as np
import pytest

from oracle import mlp as M
from tests.cases import dna_case

pytestmark = pytest.mark.gpu

INPUTS, HIDDEN = 14, 64


def net(seed=1, hidden=HIDDEN):
    from aspartik_gb300.surrogate import Surrogate

    return Surrogate(INPUTS, hidden, seed=seed)


def test_forward_matches_oracle(rng):
    s = net()
    p = s.get_params().astype(np.float64)
    x = rng.normal(size=(37, INPUTS)).astype(np.float32)
    np.testing.assert_allclose(s.forward(x), M.forward(p, x, INPUTS, HIDDEN), rtol=2e-4,
                               atol=2e-5)


def test_gradient_matches_oracle(rng):
    s = net(seed=2)
    p = s.get_params().astype(np.float64)
    xn = rng.normal(size=(50, INPUTS)).astype(np.float32)
    xo = rng.normal(size=(50, INPUTS)).astype(np.float32)
    d = rng.normal(size=50).astype(np.float32)
    loss, g = s.loss_grad(xn, xo, d)
    ref_loss, ref_g = M.loss_grad(p, xn, xo, d, INPUTS, HIDDEN)
    assert loss == pytest.approx(ref_loss, rel=1e-4)
    scale = np.abs(ref_g).max()
    np.testing.assert_allclose(g, ref_g, rtol=2e-3, atol=2e-5 * scale)


@pytest.mark.parametrize("hidden", [256, 96, 32])
def test_fused_pair_kernel_matches_forward(rng, hidden):
    """The single-pair kernel (a cluster of eight CTAs, each computing a
    slice of every layer: 32, 12 or 4 units) against the batched forward
    pass and the numpy oracle; the 14-input first layer takes the kernel's
    scalar path (rows not float4-aligned)."""
    s = net(seed=3, hidden=hidden)
    p = s.get_params().astype(np.float64)
    for _ in range(4):
        xn = rng.normal(size=INPUTS).astype(np.float32)
        xo = rng.normal(size=INPUTS).astype(np.float32)
        f = s.forward(np.stack([xn, xo]))
        ref = M.forward(p, np.stack([xn, xo]), INPUTS, hidden)
        d = s.delta(xn, xo)
        assert d == pytest.approx(f[0] - f[1], rel=1e-4, abs=1e-5)
        assert d == pytest.approx(ref[0] - ref[1], rel=1e-4, abs=1e-5)


@pytest.mark.parametrize("count", [1, 5, 256])
def test_batched_pairs_match_single_pairs(rng, count):
    """One launch over `count` pairs (a cluster per pair) gives, pair by
    pair, the single-pair launch's bits; more than 256 pairs are refused."""
    from aspartik_gb300._native import B3GError

    s = net(seed=5, hidden=256)
    xn = rng.normal(size=(count, INPUTS)).astype(np.float32)
    xo = rng.normal(size=(count, INPUTS)).astype(np.float32)
    d = s.deltas(xn, xo)
    assert d.shape == (count,)
    for k in range(0, count, max(1, count // 9)):
        assert d[k] == s.delta(xn[k], xo[k])
    with pytest.raises(B3GError):
        s.deltas(np.zeros((257, INPUTS), np.float32), np.zeros((257, INPUTS), np.float32))


def test_training_learns_a_difference_function(rng):
    """delta = g(x_new) - g(x_old) for a smooth g: the trained network's
    differences explain most of the variance."""
    g = lambda x: np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] - 0.3 * x[:, 3] ** 2  # noqa: E731
    n = 20000
    xo = rng.normal(size=(n, INPUTS)).astype(np.float32)
    xn = (xo + 0.3 * rng.normal(size=(n, INPUTS))).astype(np.float32)
    d = (g(xn) - g(xo)).astype(np.float32)
    s = net(seed=4, hidden=128)
    before, _ = s.loss_grad(xn[:2000], xo[:2000], d[:2000])
    s.train(xn, xo, d, epochs=15, batch=256, lr=2e-3)
    after, _ = s.loss_grad(xn[:2000], xo[:2000], d[:2000])
    assert after < 0.1 * np.var(d[:2000])
    assert after < 0.2 * before


def make(case, **kw):
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    return Mcmc(case.leaves, case.weights, case.tree.parents, case.tree.heights,
                McmcSettings(**kw))


def test_delayed_acceptance_keeps_the_posterior_and_saves_evaluations():
    """Same data and moves with and without delayed acceptance: posterior
    means agree within Monte Carlo error, and the screened chain runs fewer
    exact likelihood evaluations per step than the plain one."""
    c = dna_case(24, 800, seed=24, root_height=0.6)
    # tree scale and kappa moves re-evaluate the whole tree: screened
    weights = dict(subtree_slide=20, narrow_exchange=20, tree_scale=10, scale_kappa=10)
    steps, pilot = 40_000, 8_000
    runs = {}
    for name, da in (("plain", 0), ("da", pilot)):
        m = make(c, model="hky", precision="f32", num_categories=1, seed=21 if da else 22,
                 sample_every=5, weights=weights, da_pilot_steps=da, da_epochs=25,
                 da_hidden=128)
        m.set_parameters(kappa=2.0, frequencies=c.pi)
        m.run(steps)
        runs[name] = (m.trace("root_height")[pilot // 5:], m.trace("tree_length")[pilot // 5:],
                      m.da_stats())
        assert m.check() < 1e-12
    from aspartik_gb300.ess import ess

    for k in (0, 1):
        a, b = runs["plain"][k], runs["da"][k]
        se = np.sqrt(a.var() / ess(a, 0.0) + b.var() / ess(b, 0.0))
        assert abs(a.mean() - b.mean()) < 5 * se
    st = runs["da"][2]
    assert st["pilot_pairs"] > 1000 and st["fallback"] == 0
    assert st["stage1_rejects"] > 0
    assert st["exact_evaluations"] < runs["plain"][2]["exact_evaluations"]
