// mcmc_state.cpp -- checkpoint of the native MCMC driver (b3g_mcmc_dump /
// b3g_mcmc_load).
//
// Counterpart of Mcmc::dump (crates/b3/src/mcmc.rs:251-268), which writes a
// tag, a protocol version, the current step, the posterior, every
// parameter, the scheduler and the RNG.  This driver's state differs from
// the reference's (its own operators, xoshiro256** RNGs, several chains), so
// this exact checkpoint has its own layout (mcmc_verbatim.cpp writes and
// reads one chain in the reference's); it holds everything later steps
// depend on:
//
//   "B3GMCST1", u32 version = 2, u32 chains, leaves, model, categories,
//   clock categories, precision, reserved
//   u64 step, swaps tried, swaps accepted; u32 tuning rounds, reserved
//   u64 swap RNG state[4]
//   per operator: u64 accepts, rejects, aborts, prior rejects, window
//   accepts, window rejects; f64 tuning
//   per chain: u32 index, run-walk tile, run-walk block, leaves; f64 beta,
//   lnL, prior, kappa, alpha, birth rate, clock sd; u32 n, f64 rates[n];
//   u32 n, f64 frequencies[n]; u64 RNG state[4]; u32 parents[2L-1];
//   u32 children[2L-2] (each internal's children in the order the
//   operators walk them); f64 heights[2L-1]; with a relaxed clock u32 edge
//   categories[2L-1]
//   u64 FNV-1a hash of everything before it
//
// Native byte order; a checkpoint is read back on the same kind of host.
// Delayed-acceptance runs are not checkpointed (their surrogate, pilot and
// drift window are not part of the format).
#include "mcmc.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

namespace b3g {

namespace {

constexpr char kMagic[8] = {'B', '3', 'G', 'M', 'C', 'S', 'T', '1'};
constexpr uint32_t kVersion = 2; // 2: fourteen operator kinds, child order

uint64_t fnv1a(const uint8_t *p, size_t n)
{
	uint64_t h = 1469598103934665603ull;
	for (size_t i = 0; i < n; ++i) {
		h ^= p[i];
		h *= 1099511628211ull;
	}
	return h;
}

struct Writer {
	std::vector<uint8_t> &out;
	template <typename T> void put(const T &v)
	{
		const uint8_t *p = reinterpret_cast<const uint8_t *>(&v);
		out.insert(out.end(), p, p + sizeof(T));
	}
	template <typename T> void put_n(const T *v, size_t n)
	{
		const uint8_t *p = reinterpret_cast<const uint8_t *>(v);
		out.insert(out.end(), p, p + n * sizeof(T));
	}
};

struct Reader {
	const uint8_t *p;
	size_t left;
	template <typename T> T get()
	{
		T v;
		take(&v, sizeof(T));
		return v;
	}
	template <typename T> void get_n(T *v, size_t n) { take(v, n * sizeof(T)); }
	void take(void *dst, size_t n)
	{
		if (n > left)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "checkpoint is truncated");
		std::memcpy(dst, p, n);
		p += n;
		left -= n;
	}
};

} // namespace

std::vector<uint8_t> Mcmc::dump() const
{
	if (cfg_.da_pilot_steps)
		throw Error(B3G_ERR_STATE,
			    "delayed-acceptance runs are not checkpointed");
	for (const auto &chp : chains_)
		if (chp->launched || chp->model_sent || chp->alpha_sent)
			throw Error(B3G_ERR_STATE, "checkpoint between steps only");
	std::vector<uint8_t> buf;
	Writer w{buf};
	w.put_n(kMagic, 8);
	const uint32_t L = chains_[0]->tree->num_leaves();
	const uint32_t head[8] = {kVersion, (uint32_t)chains_.size(), L,
				  cfg_.model, cfg_.num_categories,
				  cfg_.clock_categories, cfg_.precision, 0u};
	w.put_n(head, 8);
	w.put(step_);
	w.put(swaps_tried_);
	w.put(swaps_accepted_);
	w.put(tune_rounds_);
	w.put(uint32_t(0));
	uint64_t rs[4];
	swap_rng_.get_state(rs);
	w.put_n(rs, 4);
	for (uint32_t k = 0; k < kOpCount; ++k) {
		const OpStats &o = ops_[k];
		const uint64_t c[6] = {o.accepts, o.rejects, o.aborts,
				       o.prior_rejects, o.window_accepts,
				       o.window_rejects};
		w.put_n(c, 6);
		w.put(o.tuning);
	}
	for (const auto &chp : chains_) {
		const Chain &ch = *chp;
		const uint32_t h[4] = {ch.index, ch.calc->runs_tile(),
				       ch.calc->runs_block(), ch.tree->num_leaves()};
		w.put_n(h, 4);
		const double v[7] = {ch.beta,       ch.lnl_cache, ch.prior_cache,
				     ch.kappa.v,    ch.alpha.v,   ch.birth_rate.v,
				     ch.clock_sd.v};
		w.put_n(v, 7);
		w.put((uint32_t)ch.rates.v.size());
		w.put_n(ch.rates.v.data(), ch.rates.v.size());
		w.put((uint32_t)ch.freqs.v.size());
		w.put_n(ch.freqs.v.data(), ch.freqs.v.size());
		ch.rng.get_state(rs);
		w.put_n(rs, 4);
		w.put_n(ch.tree->parents().data(), ch.tree->num_nodes());
		w.put_n(ch.tree->children().data(), ch.tree->children().size());
		w.put_n(ch.tree->heights().data(), ch.tree->num_nodes());
		if (cfg_.clock_categories)
			w.put_n(ch.edge_cat.data(), ch.tree->num_nodes());
	}
	w.put(fnv1a(buf.data(), buf.size()));
	return buf;
}

void Mcmc::load(const uint8_t *state, size_t size)
{
	if (cfg_.da_pilot_steps)
		throw Error(B3G_ERR_STATE,
			    "delayed-acceptance runs are not checkpointed");
	if (!state || size < 8 + 8)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "checkpoint is truncated");
	uint64_t stored;
	std::memcpy(&stored, state + size - 8, 8);
	if (fnv1a(state, size - 8) != stored)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "checkpoint is corrupted (hash mismatch)");
	Reader r{state, size - 8};
	char magic[8];
	r.get_n(magic, 8);
	if (std::memcmp(magic, kMagic, 8) != 0)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "not a b3g MCMC checkpoint");
	uint32_t head[8];
	r.get_n(head, 8);
	if (head[0] != kVersion)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "unknown checkpoint version " + std::to_string(head[0]));
	const uint32_t L = chains_[0]->tree->num_leaves();
	if (head[1] != chains_.size() || head[2] != L || head[3] != cfg_.model ||
	    head[4] != cfg_.num_categories || head[5] != cfg_.clock_categories ||
	    head[6] != cfg_.precision)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "checkpoint of a different configuration (chains, "
			    "leaves, model, categories, clock or precision)");
	const uint64_t step = r.get<uint64_t>();
	const uint64_t tried = r.get<uint64_t>();
	const uint64_t accepted = r.get<uint64_t>();
	const uint32_t rounds = r.get<uint32_t>();
	(void)r.get<uint32_t>();
	uint64_t swap_rs[4];
	r.get_n(swap_rs, 4);
	OpStats ops[kOpCount];
	for (uint32_t k = 0; k < kOpCount; ++k) {
		uint64_t c[6];
		r.get_n(c, 6);
		ops[k].accepts = c[0];
		ops[k].rejects = c[1];
		ops[k].aborts = c[2];
		ops[k].prior_rejects = c[3];
		ops[k].window_accepts = c[4];
		ops[k].window_rejects = c[5];
		ops[k].tuning = r.get<double>();
	}
	struct Saved {
		uint32_t h[4];
		double v[7];
		std::vector<double> rates, freqs;
		uint64_t rs[4];
		std::vector<uint32_t> parents, children, cats;
		std::vector<double> heights;
		std::unique_ptr<DatedTree> tree;
	};
	std::vector<Saved> saved(chains_.size());
	for (size_t i = 0; i < saved.size(); ++i) {
		Saved &sv = saved[i];
		const uint32_t nodes = chains_[i]->tree->num_nodes();
		r.get_n(sv.h, 4);
		if (sv.h[3] != chains_[i]->tree->num_leaves())
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "checkpoint of a different alignment (leaves)");
		r.get_n(sv.v, 7);
		uint32_t n = r.get<uint32_t>();
		if (n > 6)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "bad rates in checkpoint");
		sv.rates.resize(n);
		r.get_n(sv.rates.data(), n);
		n = r.get<uint32_t>();
		if (n != 4)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "bad frequencies in checkpoint");
		sv.freqs.resize(n);
		r.get_n(sv.freqs.data(), n);
		r.get_n(sv.rs, 4);
		sv.parents.resize(nodes);
		sv.children.resize(nodes - 1);
		sv.heights.resize(nodes);
		r.get_n(sv.parents.data(), nodes);
		r.get_n(sv.children.data(), nodes - 1);
		r.get_n(sv.heights.data(), nodes);
		if (cfg_.clock_categories) {
			sv.cats.resize(nodes);
			r.get_n(sv.cats.data(), nodes);
		}
		try {
			sv.tree = std::make_unique<DatedTree>(sv.parents.data(),
							      sv.heights.data(), nodes);
		} catch (const std::invalid_argument &e) {
			throw Error(B3G_ERR_INVALID_ARGUMENT, e.what());
		}
		if (!sv.tree->validate())
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "checkpoint holds an invalid tree");
		if (!sv.tree->set_child_order(sv.children.data()))
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "checkpoint's child order contradicts its parents");
		for (uint32_t v = 0; v < (uint32_t)sv.cats.size(); ++v)
			if (sv.cats[v] >= cfg_.clock_categories &&
			    v != sv.tree->root())
				throw Error(B3G_ERR_INVALID_ARGUMENT,
					    "clock category out of range");
	}
	if (r.left != 0)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "trailing bytes in checkpoint");

	// apply: every chain gets its state back and is evaluated whole
	for (size_t i = 0; i < chains_.size(); ++i) {
		Chain &ch = *chains_[i];
		Saved &sv = saved[i];
		ch.calc->set_runs_shape(sv.h[1], sv.h[2]);
		ch.index = sv.h[0];
		ch.beta = sv.v[0];
		ch.kappa.v = sv.v[3];
		ch.alpha.v = sv.v[4];
		ch.birth_rate.v = sv.v[5];
		ch.clock_sd.v = sv.v[6];
		for (Real *x : {&ch.kappa, &ch.alpha, &ch.birth_rate, &ch.clock_sd})
			x->accept();
		ch.rates.v = sv.rates;
		ch.freqs.v = sv.freqs;
		ch.rates.accept();
		ch.freqs.accept();
		ch.rng.set_state(sv.rs);
		ch.tree = std::move(sv.tree);
		if (cfg_.clock_categories) {
			ch.edge_cat = sv.cats;
			clock_rates(ch);
		}
		ch.cat_changed = false;
		send_model(ch, true);
		if (cfg_.num_categories > 1)
			ch.calc->set_gamma(ch.alpha.v);
		lists(ch);
		ch.calc->propose_lengths(ch.internals.data(), ch.children.data(),
					 (uint32_t)ch.internals.size(),
					 ch.lengths.data(), 1.0);
	}
	for (size_t i = 0; i < chains_.size(); ++i) {
		Chain &ch = *chains_[i];
		const double lnl = ch.calc->log_likelihood();
		ch.calc->accept();
		ch.tree->accept();
		ch.launched = ch.model_sent = ch.alpha_sent = false;
		const double want = saved[i].v[1];
		// the same partials, summed in the order of a whole-tree launch
		if (!(std::fabs(lnl - want) <= 1e-12 * std::max(1.0, std::fabs(want))))
			throw Error(B3G_ERR_STATE,
				    "checkpoint does not match this alignment: its "
				    "log-likelihood differs from the recomputed one");
		ch.lnl_cache = want;
		ch.prior_cache = saved[i].v[2];
	}
	step_ = step;
	swaps_tried_ = tried;
	swaps_accepted_ = accepted;
	tune_rounds_ = rounds;
	swap_rng_.set_state(swap_rs);
	for (uint32_t k = 0; k < kOpCount; ++k)
		ops_[k] = ops[k];
	tuned_ = true;
	for (auto &t : trace_)
		t.clear();
	for (auto &t : chain_trace_)
		t.clear();
	sample_steps_.clear();
	sample_parents_.clear();
	sample_heights_.clear();
	sample_params_.clear();
}

} // namespace b3g
