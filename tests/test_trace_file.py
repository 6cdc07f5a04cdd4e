"""Trace files in the reference's TraceWriter layout
(callback/trace_writer.rs): columns, types, metadata and the tree round trip
(on the CPU with a stand-in chain), and the native driver's samples (GPU)."""

import numpy as np
import pytest

from tests.cases import dna_case


class FakeChain:
    """Samples of a 5-node tree in the shape Mcmc.samples() returns."""

    class settings:
        model = "gtr"
        clock_categories = 3

    def __init__(self, n=7):
        rng = np.random.default_rng(1)
        self.parents = np.tile(np.array([3, 3, 4, 4, 0xFFFFFFFF], dtype=np.uint32), (n, 1))
        self.heights = np.zeros((n, 5))
        self.heights[:, 3] = rng.uniform(0.1, 0.5, n)
        self.heights[:, 4] = self.heights[:, 3] + rng.uniform(0.1, 0.5, n)
        self.n = n

    def samples(self):
        n = self.n
        return {"step": np.arange(1, n + 1, dtype=np.uint64) * 10, "parents": self.parents,
                "heights": self.heights, "kappa": np.full(n, 2.0), "alpha": np.full(n, 0.5),
                "birth_rate": np.linspace(1, 2, n), "rates": np.ones((n, 6)),
                "frequencies": np.full((n, 4), 0.25), "clock_sd": np.full(n, 0.3)}

    def trace(self, name):
        return {"lnl": -np.arange(self.n) - 100.0, "prior": np.full(self.n, -5.0)}[name]


def test_trace_file_layout_and_tree_round_trip(tmp_path):
    pa = pytest.importorskip("pyarrow")
    import pyarrow.ipc as ipc

    from aspartik_gb300.trace import read_trees, write_trace

    fake = FakeChain()
    path = tmp_path / "trace.arrow"
    assert write_trace(path, fake) == fake.n
    table = ipc.open_file(str(path)).read_all()
    names = table.schema.names
    assert names[:4] == ["step", "posterior", "prior", "likelihood"]
    for col in ("tree:parents", "tree:heights", "tree:length", "tree:height", "rates",
                "frequencies", "clock_sd", "birth_rate", "alpha"):
        assert col in names, col
    assert table.schema.field("step").type == pa.uint64()
    assert table.schema.field("tree:parents").type == pa.list_(pa.uint32(), 5)
    assert all(not f.nullable for f in table.schema)
    meta = table.schema.metadata
    assert set(meta) >= {b"aspartik", b"os", b"arch", b"time"}
    np.testing.assert_array_equal(table["posterior"].to_numpy(),
                                  fake.trace("lnl") + fake.trace("prior"))
    parents, heights = read_trees(path)
    np.testing.assert_array_equal(parents, fake.parents)
    np.testing.assert_array_equal(heights, fake.heights)
    h = fake.heights
    # edges 0-3, 1-3 (h3 each), 2-4 (h4), 3-4 (h4 - h3)
    want_len = 2 * h[:, 3] + h[:, 4] + (h[:, 4] - h[:, 3])
    np.testing.assert_allclose(table["tree:length"].to_numpy(), want_len)
    np.testing.assert_allclose(table["tree:height"].to_numpy(), h[:, 4])


@pytest.mark.gpu
def test_native_samples_match_chain_state_and_traces():
    from aspartik_gb300.mcmc import Mcmc, McmcSettings

    c = dna_case(12, 200, seed=91, model="gtr", alpha=0.5, num_categories=4)
    s = McmcSettings(model="gtr", precision="f64", num_categories=4, sample_every=10,
                     weights=dict(subtree_slide=5, narrow_exchange=5, scale_alpha=1,
                                  delta_rates=1, tree_scale=1))
    m = Mcmc(c.leaves, c.weights, c.tree.parents, c.tree.heights, s)
    m.set_parameters(rates=c.rates, frequencies=c.pi, alpha=0.5, birth_rate=1.0)
    m.run(1000)
    smp = m.samples()
    assert smp["step"].tolist() == list(range(10, 1001, 10))
    parents, heights, lnl, _ = m.chain_state(0)
    np.testing.assert_array_equal(smp["parents"][-1], parents)
    np.testing.assert_array_equal(smp["heights"][-1], heights)
    np.testing.assert_array_equal(smp["alpha"], m.trace("alpha"))
    np.testing.assert_array_equal(smp["rates"][:, 0], m.trace("kappa_or_rate0"))
    root = np.argmax(smp["parents"] == 0xFFFFFFFF, axis=1)
    np.testing.assert_array_equal(smp["heights"][np.arange(root.size), root],
                                  m.trace("root_height"))
    assert m.trace("lnl")[-1] == lnl
    m.close()
