"""Dirty lists for whole-tree and single-path evaluations.

Produces what ``DatedTree::partials_lists`` (crates/b3/src/parameters/
tree.rs:398-461) returns for the two evaluations the benchmark times: every
internal dirty (after ``mark_all_edges_updated``, tree.rs:382-386), and the
path from one internal node to the root (after ``set_height`` of that node,
tree.rs:516-527).  Internals come children-first (breadth-first from the root,
reversed) and each child pair is sorted (min, max).
"""

from __future__ import annotations

from collections import deque

import numpy as np

TOMBSTONE = 0xFFFFFFFF


class Topology:
    def __init__(self, parents: np.ndarray, heights: np.ndarray):
        self.parents = np.asarray(parents, dtype=np.int64)
        self.heights = np.asarray(heights, dtype=np.float64)
        n = self.parents.size
        self.L = (n + 1) // 2
        self.children = np.full((self.L - 1, 2), -1, dtype=np.int64)
        self.root = -1
        for node, par in enumerate(self.parents):
            if par == TOMBSTONE:
                self.root = node
                continue
            k = par - self.L
            if self.children[k, 0] < 0:
                self.children[k, 0] = node
            else:
                self.children[k, 1] = node

    def edge_length(self, e: int) -> float:
        return float(self.heights[self.parents[e]] - self.heights[e])

    def _lists(self, dirty: set) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        order = [self.root]
        queue = deque([self.root])
        while queue:
            v = queue.popleft()
            for ch in self.children[v - self.L]:
                if ch >= self.L and ch in dirty:
                    order.append(int(ch))
                    queue.append(int(ch))
        order.reverse()
        internals = np.array(order, dtype=np.uint32)
        ch = np.sort(self.children[internals.astype(np.int64) - self.L], axis=1)
        lengths = self.heights[internals][:, None] - self.heights[ch]
        return internals, ch.astype(np.uint32), np.ascontiguousarray(lengths)

    def full(self):
        """Lists of a whole-tree evaluation."""
        return self._lists(set(range(self.L, 2 * self.L - 1)))

    def path(self, node: int):
        """Lists after the height of internal ``node`` changed."""
        dirty = set()
        v = int(node)
        while v != TOMBSTONE and v >= 0:
            dirty.add(v)
            p = self.parents[v]
            v = -1 if p == TOMBSTONE else int(p)
        return self._lists(dirty)

    def internal_children(self, internals: np.ndarray) -> int:
        ch = self.children[np.asarray(internals, dtype=np.int64) - self.L]
        return int((ch >= self.L).sum())


def algorithmic_bytes(top: Topology, internals: np.ndarray, num_patterns: int,
                      num_categories: int, states: int, w: int, e_b: int, w_p: int) -> int:
    """Bytes one evaluation must move at minimum: per listed node and
    (pattern, category) the partial written, each internal child's partial
    read (a tip child: its one-byte code), the scale exponents written and
    read; the root partial read; per pattern its weight and site result; per
    listed node the two child transition matrices of every category."""
    C, P, S = num_categories, num_patterns, states
    n = len(internals)
    ch = top.children[np.asarray(internals, dtype=np.int64) - top.L]
    n_int_children = int((ch >= top.L).sum())
    n_tip_children = 2 * n - n_int_children
    per_cp = (n * S * w + n_int_children * S * w + n_tip_children * 1
              + e_b * (n + n_int_children))
    return int(C * P * per_cp + C * P * S * w + P * (4 + 8) + n * 2 * C * S * S * w_p)
