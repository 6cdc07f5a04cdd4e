"""Pattern-sharded likelihood (aspartik_gb300/shard.py): the slices cover the
patterns exactly; two gloo ranks on CPU, each holding half the patterns,
give the whole alignment's log-likelihood after one scalar all-reduce; on
the GPU the shards' sums equal the unsharded calculator."""

import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

from aspartik_gb300.shard import shard_bounds, shard_patterns

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("P,world", [(1, 1), (7, 2), (17764, 8), (100, 3), (5, 5)])
def test_bounds_cover_the_patterns(P, world):
    got = [shard_bounds(P, r, world) for r in range(world)]
    assert got[0][0] == 0 and got[-1][1] == P
    for (a, b), (c, _) in zip(got, got[1:]):
        assert b == c
    sizes = [b - a for a, b in got]
    assert min(sizes) >= 1 and max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(P, world, world)


class OracleCalc:
    """A calculator over one pattern slice on the CPU oracle (restated cpu4
    per Gamma category, log-sum-exp, weighted sum)."""

    def __init__(self, leaves, weights, rates, pi, alpha, K):
        from oracle import oracle as O

        self.O = O
        self.leaves, self.w = leaves, weights.astype(np.float64)
        self.model = O.gtr(rates, pi)
        self.cats = O.gamma_categories(alpha, K)
        self.calcs = [O.Cpu4Calculator(leaves, leaves.shape[1], 30, 1) for _ in self.cats]

    def propose_lengths(self, internals, children, lengths, clock_rate=1.0):
        per = []
        for calc, r in zip(self.calcs, self.cats):
            mats = np.array([[self.model.transition(d * clock_rate * r) for d in pair]
                             for pair in lengths])
            calc.propose(internals, children, mats, self.model.pi)
            per.append(np.array(calc.likelihoods()))
        per = np.array(per)
        mx = per.max(axis=0)
        site = mx + np.log(np.exp(per - mx).sum(axis=0)) + np.log(1.0 / len(self.cats))
        self.value = float(site @ self.w)

    def log_likelihood(self):
        return self.value

    def accept(self):
        for c in self.calcs:
            c.accept()

    def reject(self):
        for c in self.calcs:
            c.reject()


def lists(parents, heights):
    from oracle import oracle as O

    t = O.DatedTree(parents, heights)
    t.mark_all_edges_updated()
    internals, children = t.partials_lists()
    lengths = np.array([[t.edge_length(int(a)), t.edge_length(int(b))] for a, b in children])
    return internals, children, lengths


def _rank(rank, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    from aspartik_gb300.shard import ShardedLikelihood
    from tests.cases import dna_case

    dist.init_process_group("gloo", rank=rank, world_size=2)
    c = dna_case(20, 900, seed=55, model="gtr", alpha=0.5, num_categories=4)
    sh = ShardedLikelihood(lambda l, w: OracleCalc(l, w, c.rates, c.pi, 0.5, 4),
                           c.leaves, c.weights, rank, 2)
    sh.propose_lengths(*lists(c.tree.parents, c.tree.heights))
    total = sh.log_likelihood()
    sh.accept()
    # a second evaluation with every height scaled
    sh.propose_lengths(*lists(c.tree.parents, c.tree.heights * 1.3))
    total2 = sh.log_likelihood()
    q.put((rank, sh.bounds, total, total2))
    dist.destroy_process_group()


def test_two_gloo_ranks_sum_to_the_whole_alignment():
    from tests.cases import dna_case

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    c = dna_case(20, 900, seed=55, model="gtr", alpha=0.5, num_categories=4)
    whole = OracleCalc(c.leaves, c.weights, c.rates, c.pi, 0.5, 4)
    whole.propose_lengths(*lists(c.tree.parents, c.tree.heights))
    want = whole.log_likelihood()
    whole.accept()
    whole.propose_lengths(*lists(c.tree.parents, c.tree.heights * 1.3))
    want2 = whole.log_likelihood()
    assert res[0][1][1] == res[1][1][0]  # adjacent slices
    for _, _, total, total2 in res:  # every rank holds the sum
        assert total == pytest.approx(want, rel=1e-12)
        assert total2 == pytest.approx(want2, rel=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 1e-6)])
def test_gpu_shards_sum_to_the_unsharded_calculator(precision, tol):
    from aspartik_gb300.calculator import Calculator
    from tests.cases import dna_case

    c = dna_case(48, 3000, seed=56, model="gtr", alpha=0.5, num_categories=4)
    args = lists(c.tree.parents, c.tree.heights)

    def make(leaves, weights):
        g = Calculator.GB300(0, precision).make4(leaves, leaves.shape[1], num_categories=4)
        g.set_weights(weights)
        g.set_reversible(c.rates, c.pi)
        g.set_gamma(0.5)
        return g

    whole = make(c.leaves, c.weights)
    whole.propose_lengths(*args, 1.0)
    want = whole.log_likelihood()
    parts = []
    for r in range(3):
        sl, sw = shard_patterns(c.leaves, c.weights, r, 3)
        g = make(sl, sw)
        g.propose_lengths(*args, 1.0)
        parts.append(g.log_likelihood())
        g.close()
    whole.close()
    assert sum(parts) == pytest.approx(want, rel=tol)
