"""One chain's likelihood with its site patterns split across ranks.

Patterns are independent until the final weighted sum
(likelihood/mod.rs:134-139; gamma.rs:155-169), so rank r of N holds a
calculator over a contiguous slice of the patterns (same tree, model and
dirty lists on every rank), evaluates its share of sum_p w_p lnL_p, and one
scalar all-reduce (sum) per evaluation gives the chain's log-likelihood.
Accept and reject stay local.  The exchange is the only communication: the
dirty lists, edge lengths and model parameters are the same on every rank
because every rank runs the same deterministic proposal stream.
"""

from __future__ import annotations

import numpy as np


def shard_bounds(num_patterns: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of rank's contiguous pattern slice, balanced to within one
    pattern; every rank gets at least one pattern."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank or world size")
    if num_patterns < world:
        raise ValueError("fewer patterns than ranks")
    base, extra = divmod(num_patterns, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_patterns(leaves: np.ndarray, weights: np.ndarray, rank: int, world: int):
    """This rank's (leaves [L][p], weights [p]) slice."""
    lo, hi = shard_bounds(leaves.shape[1], rank, world)
    return np.ascontiguousarray(leaves[:, lo:hi]), np.ascontiguousarray(weights[lo:hi])


class ShardedLikelihood:
    """A calculator over this rank's pattern slice plus the sum across
    ranks.  `make_calc(leaves, weights)` builds the rank's calculator (a
    GpuCalculator on this rank's GPU, or any object with propose_lengths /
    log_likelihood / accept / reject); `group` is a torch.distributed group
    (None: the default group; no group at all with world size 1)."""

    def __init__(self, make_calc, leaves: np.ndarray, weights: np.ndarray,
                 rank: int, world: int, group=None):
        self.rank, self.world, self.group = rank, world, group
        self.bounds = shard_bounds(leaves.shape[1], rank, world)
        sl, sw = shard_patterns(leaves, weights, rank, world)
        self.calc = make_calc(sl, sw)

    def propose_lengths(self, internals, children, lengths, clock_rate: float = 1.0):
        self.calc.propose_lengths(internals, children, lengths, clock_rate)

    def local_log_likelihood(self) -> float:
        return float(self.calc.log_likelihood())

    def log_likelihood(self) -> float:
        local = self.local_log_likelihood()
        if self.world == 1:
            return local
        import torch
        import torch.distributed as dist

        t = torch.tensor([local], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
        return float(t.item())

    def accept(self) -> None:
        self.calc.accept()

    def reject(self) -> None:
        self.calc.reject()
