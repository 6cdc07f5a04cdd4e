// handle.cpp -- tree-level C ABI (include/b3g.h, "tree-level handle").
//
// The call sequence b3's MCMC makes around its likelihood
// (likelihood/dna.rs:68-124, likelihood/gamma.rs:97-169, tree.rs:357-461,
// 975-994), with the tree mirrored inside the library: the caller loads its
// tree state (b3g_set_tree), marks the edges its move changed
// (b3g_mark_edges / b3g_mark_all, as tree.rs:357-386), proposes any subset
// of chains (b3g_propose, asynchronous: every chain has its own calculator
// and CUDA stream, so the chains' evaluations run concurrently), reads the
// log-likelihoods and decides per chain (b3g_accept / b3g_reject).  The
// dirty list is built from the mirrored tree exactly as partials_lists
// builds it (children first, root last, sorted child pairs, tree.rs:398-461)
// and evaluated by the calculator's propose_lengths.
#include "calculator.hpp"
#include "tree.hpp"

#include <cmath>
#include <memory>
#include <new>
#include <stdexcept>
#include <vector>

namespace b3g {
void set_last_error(const char *message);

class Handle {
      public:
	Handle(const b3g_config &cfg, const uint8_t *tips,
	       const uint32_t *weights, uint32_t chains)
	    : L_(cfg.num_leaves), S_(cfg.num_states), C_(cfg.num_categories)
	{
		if (chains == 0 || chains > 64)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "between 1 and 64 chains");
		chain_.resize(chains);
		for (auto &ch : chain_) {
			ch.calc = std::make_unique<Calculator>(cfg, tips);
			ch.calc->set_weights(weights);
		}
	}

	uint32_t chains() const { return (uint32_t)chain_.size(); }

	void set_model(uint32_t c, uint32_t S, const double *V,
		       const double *Vinv, const double *lambda,
		       const double *pi, const double *cat_rates, uint32_t C)
	{
		Chain &ch = at(c);
		if (S != S_ || C != C_)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "states and categories must match the handle");
		if (!V || !Vinv || !lambda || !pi || !cat_rates)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "null model array");
		// Q = V diag(lambda) V^-1 for the short-branch shortcut
		std::vector<double> Q((size_t)S * S, 0.0);
		for (uint32_t i = 0; i < S; ++i)
			for (uint32_t j = 0; j < S; ++j) {
				double s = 0.0;
				for (uint32_t k = 0; k < S; ++k)
					s += V[i * S + k] * lambda[k] * Vinv[k * S + j];
				Q[(size_t)i * S + j] = s;
			}
		ch.calc->set_eigen(V, Vinv, lambda, Q.data(), pi, 1);
		ch.calc->set_category_rates(cat_rates);
	}

	void set_tree(uint32_t c, const uint32_t *parents, const double *heights,
		      double clock_rate)
	{
		Chain &ch = at(c);
		if (!parents || !heights)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "null tree array");
		if (!(clock_rate > 0.0) || !std::isfinite(clock_rate))
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "clock rate must be positive and finite");
		std::unique_ptr<DatedTree> t;
		try {
			t = std::make_unique<DatedTree>(parents, heights, 2 * L_ - 1);
		} catch (const std::invalid_argument &e) {
			throw Error(B3G_ERR_INVALID_ARGUMENT, e.what());
		}
		if (!t->validate())
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "not a valid dated tree");
		ch.tree = std::move(t);
		ch.clock = clock_rate;
		if (!ch.has_accepted) {
			ch.acc_parents.assign(parents, parents + 2 * L_ - 1);
			ch.acc_heights.assign(heights, heights + 2 * L_ - 1);
			ch.acc_clock = clock_rate;
			ch.has_accepted = true;
		}
	}

	void mark_edges(uint32_t c, const uint32_t *edges, uint32_t n)
	{
		Chain &ch = with_tree(c);
		if (n && !edges)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "null edges");
		for (uint32_t i = 0; i < n; ++i) {
			if (edges[i] >= 2 * L_ - 1 || edges[i] == ch.tree->root())
				throw Error(B3G_ERR_INVALID_ARGUMENT,
					    "no such edge (edge id = child node id)");
		}
		for (uint32_t i = 0; i < n; ++i)
			ch.tree->mark_edge_updated(edges[i]);
	}

	void mark_all(uint32_t c) { with_tree(c).tree->mark_all_edges_updated(); }

	void propose(uint64_t mask)
	{
		if (chains() < 64 && (mask >> chains()))
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "chain mask names a chain that does not exist");
		for (uint32_t c = 0; c < chains(); ++c)
			if ((mask >> c) & 1u)
				with_tree(c);
		for (uint32_t c = 0; c < chains(); ++c) {
			if (!((mask >> c) & 1u))
				continue;
			Chain &ch = chain_[c];
			ch.tree->partials_lists(internals_, children_, lengths_);
			ch.calc->propose_lengths(internals_.data(), children_.data(),
						 (uint32_t)internals_.size(),
						 lengths_.data(), ch.clock);
			ch.pending = true;
			ch.have = false;
		}
	}

	void wait()
	{
		for (uint32_t c = 0; c < chains(); ++c)
			if (chain_[c].pending)
				lnl(c);
	}

	double lnl(uint32_t c)
	{
		Chain &ch = at(c);
		if (ch.pending) {
			ch.value = ch.calc->log_likelihood();
			ch.pending = false;
			ch.have = true;
		}
		if (!ch.have)
			throw Error(B3G_ERR_STATE, "chain has no evaluated proposal");
		return ch.value;
	}

	void site_lnl(uint32_t c, double *out)
	{
		if (!out)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		lnl(c);
		at(c).calc->site_log_likelihoods(out);
	}

	void accept(uint32_t c)
	{
		Chain &ch = with_tree(c);
		if (ch.pending)
			lnl(c);
		ch.calc->accept();
		ch.tree->accept();
		ch.acc_parents = ch.tree->parents();
		ch.acc_heights = ch.tree->heights();
		ch.acc_clock = ch.clock;
	}

	void reject(uint32_t c)
	{
		Chain &ch = with_tree(c);
		if (ch.pending)
			lnl(c);
		ch.calc->reject();
		// back to the last accepted tree, nothing marked
		ch.tree = std::make_unique<DatedTree>(ch.acc_parents.data(),
						      ch.acc_heights.data(),
						      2 * L_ - 1);
		ch.clock = ch.acc_clock;
		ch.have = false;
	}

      private:
	struct Chain {
		std::unique_ptr<Calculator> calc;
		std::unique_ptr<DatedTree> tree;
		double clock = 1.0, acc_clock = 1.0, value = 0.0;
		std::vector<uint32_t> acc_parents;
		std::vector<double> acc_heights;
		bool has_accepted = false, pending = false, have = false;
	};
	Chain &at(uint32_t c)
	{
		if (c >= chains())
			throw Error(B3G_ERR_INVALID_ARGUMENT, "no such chain");
		return chain_[c];
	}
	Chain &with_tree(uint32_t c)
	{
		Chain &ch = at(c);
		if (!ch.tree)
			throw Error(B3G_ERR_STATE, "b3g_set_tree first");
		return ch;
	}

	uint32_t L_, S_, C_;
	std::vector<Chain> chain_;
	std::vector<uint32_t> internals_, children_;
	std::vector<double> lengths_;
};

} // namespace b3g

namespace {

template <typename F> b3g_status guarded(F &&f)
{
	try {
		f();
		b3g::set_last_error("");
		return B3G_OK;
	} catch (const b3g::Error &e) {
		b3g::set_last_error(e.what());
		return e.status;
	} catch (const std::bad_alloc &) {
		b3g::set_last_error("host allocation failed");
		return B3G_ERR_OUT_OF_MEMORY;
	} catch (const std::exception &e) {
		b3g::set_last_error(e.what());
		return B3G_ERR_STATE;
	} catch (...) {
		b3g::set_last_error("unknown error");
		return B3G_ERR_STATE;
	}
}

b3g::Handle *handle_of(b3g_handle *h)
{
	if (!h)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null handle");
	return reinterpret_cast<b3g::Handle *>(h);
}

} // namespace

extern "C" {

B3G_API b3g_status b3g_create(const b3g_config *config, const uint8_t *tips,
			      const uint32_t *weights, uint32_t num_chains,
			      b3g_handle **out)
{
	return guarded([&] {
		if (!config || !tips || !weights || !out)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null argument");
		*out = nullptr;
		*out = reinterpret_cast<b3g_handle *>(
			new b3g::Handle(*config, tips, weights, num_chains));
	});
}

B3G_API void b3g_destroy(b3g_handle *h)
{
	delete reinterpret_cast<b3g::Handle *>(h);
}

B3G_API b3g_status b3g_set_model(b3g_handle *h, uint32_t chain, uint32_t S,
				 const double *V, const double *Vinv,
				 const double *lambda, const double *pi,
				 const double *cat_rates, uint32_t C)
{
	return guarded([&] {
		handle_of(h)->set_model(chain, S, V, Vinv, lambda, pi, cat_rates, C);
	});
}

B3G_API b3g_status b3g_set_tree(b3g_handle *h, uint32_t chain,
				const uint32_t *parents, const double *heights,
				double clock_rate)
{
	return guarded([&] {
		handle_of(h)->set_tree(chain, parents, heights, clock_rate);
	});
}

B3G_API b3g_status b3g_mark_edges(b3g_handle *h, uint32_t chain,
				  const uint32_t *edges, uint32_t n)
{
	return guarded([&] { handle_of(h)->mark_edges(chain, edges, n); });
}

B3G_API b3g_status b3g_mark_all(b3g_handle *h, uint32_t chain)
{
	return guarded([&] { handle_of(h)->mark_all(chain); });
}

B3G_API b3g_status b3g_propose(b3g_handle *h, uint64_t chains_mask)
{
	return guarded([&] { handle_of(h)->propose(chains_mask); });
}

B3G_API b3g_status b3g_wait(b3g_handle *h)
{
	return guarded([&] { handle_of(h)->wait(); });
}

B3G_API b3g_status b3g_lnl(b3g_handle *h, uint32_t chain, double *out)
{
	return guarded([&] {
		if (!out)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*out = handle_of(h)->lnl(chain);
	});
}

B3G_API b3g_status b3g_site_lnl(b3g_handle *h, uint32_t chain, double *out)
{
	return guarded([&] { handle_of(h)->site_lnl(chain, out); });
}

B3G_API b3g_status b3g_accept(b3g_handle *h, uint32_t chain)
{
	return guarded([&] { handle_of(h)->accept(chain); });
}

B3G_API b3g_status b3g_reject(b3g_handle *h, uint32_t chain)
{
	return guarded([&] { handle_of(h)->reject(chain); });
}

} // extern "C"
