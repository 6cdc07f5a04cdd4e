// mcmc_verbatim.cpp -- one chain's state in the reference's own state-file
// layout (b3g_mcmc_dump_verbatim / b3g_mcmc_load_verbatim).
//
// Mcmc::dump and load_state (crates/b3/src/mcmc.rs:175-219, 251-268) write
// and read, through the verbatim layout (verbatim.hpp):
//
//   tag 62 33 b3 44 (mcmc.rs:19), u32 protocol version 19 (lib.rs:29),
//   u64 current step, f64 posterior,
//   every parameter in the Mcmc's order: a Real is one f64, a RealVector
//   its f64 values, a DatedTree a u32 slice of parents (root: u32::MAX) and
//   an f64 slice of heights, a ClassVector its u32 classes,
//   every operator in the scheduler's order: u32 accepts and u32 rejects
//   since its last tuning, then its tuning (f64) if it has one,
//   the RNG: u128 state and u128 stream of its PCG64.
//
// The parameter and operator lists are the caller's (they come from the
// reference configuration the file is exchanged with).  This driver's
// generator is xoshiro256**, not PCG64: a dump writes the chain's four
// state words as the two u128 values (the low bit of the stream set, as a
// PCG increment is odd), and a load reseeds the chain's generator from the
// four words through splitmix64, so a loaded chain is a valid continuation
// but not the writer's random stream.  The exact checkpoint of this driver
// is b3g_mcmc_dump.
#include "mcmc.hpp"
#include "verbatim.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

namespace b3g {

namespace {

constexpr uint8_t kStateTag[4] = {0x62, 0x33, 0xb3, 0x44};
constexpr uint32_t kStateVersion = 19;

void check_layout(const McmcConfig &cfg, const uint32_t *params, uint32_t np,
		  const VerbatimOp *ops, uint32_t nops)
{
	if ((np && !params) || (nops && !ops))
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null parameter or operator list");
	bool seen[kVpCount] = {};
	for (uint32_t i = 0; i < np; ++i) {
		const uint32_t p = params[i];
		if (p >= kVpCount)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "unknown state parameter");
		if (seen[p])
			throw Error(B3G_ERR_INVALID_ARGUMENT, "state parameter listed twice");
		seen[p] = true;
		if ((p == kVpKappa && cfg.model != 0) || (p == kVpRates && cfg.model != 1))
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "kappa belongs to HKY chains, exchangeabilities to GTR");
		if (p == kVpAlpha && cfg.num_categories < 2)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "alpha needs Gamma categories");
		if ((p == kVpClockSd || p == kVpClockCategories) && !cfg.clock_categories)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "relaxed-clock parameters need a relaxed clock");
	}
	for (uint32_t i = 0; i < nops; ++i)
		if (ops[i].op >= kOpCount || ops[i].has_tuning > 1)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "bad state operator");
}

uint64_t mix64(uint64_t x)
{
	x += 0x9E3779B97F4A7C15ull;
	x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
	x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
	return x ^ (x >> 31);
}

} // namespace

std::vector<uint8_t> Mcmc::dump_verbatim(uint32_t chain, const uint32_t *params,
					 uint32_t num_params, const VerbatimOp *ops,
					 uint32_t num_ops) const
{
	if (chain >= chains_.size())
		throw Error(B3G_ERR_INVALID_ARGUMENT, "chain out of range");
	check_layout(cfg_, params, num_params, ops, num_ops);
	const Chain &ch = *chains_[chain];
	if (ch.launched || ch.model_sent || ch.alpha_sent)
		throw Error(B3G_ERR_STATE, "state between steps only");
	verbatim::Writer w;
	w.tag(kStateTag, 4);
	w.u32(kStateVersion);
	w.u64(step_);
	w.f64(ch.lnl_cache + ch.prior_cache);
	const DatedTree &t = *ch.tree;
	for (uint32_t i = 0; i < num_params; ++i) {
		switch (params[i]) {
		case kVpTree:
			w.slice_u32(t.parents().data(), t.num_nodes());
			w.slice_f64(t.heights().data(), t.num_nodes());
			break;
		case kVpBirthRate:
			w.f64(ch.birth_rate.v);
			break;
		case kVpKappa:
			w.f64(ch.kappa.v);
			break;
		case kVpAlpha:
			w.f64(ch.alpha.v);
			break;
		case kVpRates:
			for (const double x : ch.rates.v)
				w.f64(x);
			break;
		case kVpFreqs:
			for (const double x : ch.freqs.v)
				w.f64(x);
			break;
		case kVpClockSd:
			w.f64(ch.clock_sd.v);
			break;
		case kVpClockCategories:
			for (uint32_t v = 0; v < t.num_nodes(); ++v)
				w.u32(ch.edge_cat[v]);
			break;
		}
	}
	for (uint32_t i = 0; i < num_ops; ++i) {
		const OpStats &o = ops_[ops[i].op];
		w.u32((uint32_t)std::min<uint64_t>(o.window_accepts, UINT32_MAX));
		w.u32((uint32_t)std::min<uint64_t>(o.window_rejects, UINT32_MAX));
		if (ops[i].has_tuning)
			w.f64(o.tuning);
	}
	uint64_t rs[4];
	ch.rng.get_state(rs);
	w.u128(rs[0], rs[1]);
	w.u128(rs[2] | 1u, rs[3]);
	return w.bytes();
}

void Mcmc::load_verbatim(uint32_t chain, const uint32_t *params, uint32_t num_params,
			 const VerbatimOp *ops, uint32_t num_ops, const uint8_t *state,
			 size_t size)
{
	if (chain >= chains_.size())
		throw Error(B3G_ERR_INVALID_ARGUMENT, "chain out of range");
	check_layout(cfg_, params, num_params, ops, num_ops);
	if (!state)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null state");
	Chain &ch = *chains_[chain];
	if (ch.launched || ch.model_sent || ch.alpha_sent)
		throw Error(B3G_ERR_STATE, "state between steps only");
	const uint32_t nodes = ch.tree->num_nodes();
	// parse everything before changing anything (load_state, mcmc.rs:183-219)
	std::vector<uint32_t> parents, cats;
	std::vector<double> heights, rates, freqs;
	double reals[kVpCount] = {};
	uint64_t step = 0, rng_words[4] = {};
	std::vector<uint32_t> accepts(num_ops), rejects(num_ops);
	std::vector<double> tunings(num_ops, 0.0);
	try {
		verbatim::Reader r(state, size);
		if (!r.tag(kStateTag, 4))
			throw Error(B3G_ERR_INVALID_ARGUMENT, "not a b3 state file");
		const uint32_t version = r.u32();
		if (version != kStateVersion)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "Cannot load state: protocol version v" +
					    std::to_string(version) +
					    " is incompatible with the currently "
					    "supported version v" +
					    std::to_string(kStateVersion) + ".");
		step = r.u64();
		(void)r.f64(); // the posterior: re-evaluated below
		for (uint32_t i = 0; i < num_params; ++i) {
			switch (params[i]) {
			case kVpTree:
				parents = r.slice_u32();
				heights = r.slice_f64();
				if (parents.size() != nodes || heights.size() != nodes)
					throw Error(B3G_ERR_INVALID_ARGUMENT,
						    "state tree has another number of nodes");
				break;
			case kVpRates:
				rates.resize(6);
				for (double &x : rates)
					x = r.f64();
				break;
			case kVpFreqs:
				freqs.resize(4);
				for (double &x : freqs)
					x = r.f64();
				break;
			case kVpClockCategories:
				cats.resize(nodes);
				for (uint32_t &c : cats)
					c = r.u32();
				break;
			default:
				reals[params[i]] = r.f64();
			}
		}
		for (uint32_t i = 0; i < num_ops; ++i) {
			accepts[i] = r.u32();
			rejects[i] = r.u32();
			if (ops[i].has_tuning)
				tunings[i] = r.f64();
		}
		r.u128(rng_words[0], rng_words[1]);
		r.u128(rng_words[2], rng_words[3]);
		if (r.left() != 0)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    std::to_string(r.left()) +
					    " bytes after the state's RNG: its parameter "
					    "or operator list differs from this one");
	} catch (const Error &) {
		throw;
	} catch (const std::runtime_error &e) { // the reader: a short state
		throw Error(B3G_ERR_INVALID_ARGUMENT, e.what());
	}
	std::unique_ptr<DatedTree> tree;
	if (!parents.empty()) {
		try {
			tree = std::make_unique<DatedTree>(parents.data(), heights.data(),
							   nodes);
		} catch (const std::invalid_argument &e) {
			throw Error(B3G_ERR_INVALID_ARGUMENT, e.what());
		}
		if (!tree->validate())
			throw Error(B3G_ERR_INVALID_ARGUMENT, "state holds an invalid tree");
	}
	const uint32_t root = tree ? tree->root() : ch.tree->root();
	for (uint32_t v = 0; v < (uint32_t)cats.size(); ++v)
		if (cats[v] >= cfg_.clock_categories && v != root)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "clock category out of range");
	for (uint32_t i = 0; i < num_params; ++i) {
		const uint32_t p = params[i];
		bool ok = true;
		if (p == kVpRates)
			for (const double x : rates)
				ok = ok && std::isfinite(x) && x > 0.0;
		else if (p == kVpFreqs)
			for (const double x : freqs)
				ok = ok && std::isfinite(x) && x > 0.0;
		else if (p != kVpTree && p != kVpClockCategories)
			ok = std::isfinite(reals[p]) && reals[p] > 0.0;
		if (!ok)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "state parameter not finite and positive");
	}
	for (uint32_t i = 0; i < num_ops; ++i)
		if (ops[i].has_tuning && !(std::isfinite(tunings[i]) && tunings[i] > 0.0))
			throw Error(B3G_ERR_INVALID_ARGUMENT, "bad operator tuning in state");

	// apply
	for (uint32_t i = 0; i < num_params; ++i) {
		switch (params[i]) {
		case kVpTree:
			ch.tree = std::move(tree);
			break;
		case kVpBirthRate:
			ch.birth_rate.v = reals[kVpBirthRate];
			break;
		case kVpKappa:
			ch.kappa.v = reals[kVpKappa];
			break;
		case kVpAlpha:
			ch.alpha.v = reals[kVpAlpha];
			break;
		case kVpRates:
			ch.rates.v = rates;
			break;
		case kVpFreqs:
			ch.freqs.v = freqs;
			break;
		case kVpClockSd:
			ch.clock_sd.v = reals[kVpClockSd];
			break;
		case kVpClockCategories:
			ch.edge_cat = cats;
			break;
		}
	}
	for (Real *x : {&ch.kappa, &ch.alpha, &ch.birth_rate, &ch.clock_sd})
		x->accept();
	ch.rates.accept();
	ch.freqs.accept();
	if (cfg_.clock_categories)
		clock_rates(ch);
	ch.cat_changed = false;
	for (uint32_t i = 0; i < num_ops; ++i) {
		OpStats &o = ops_[ops[i].op];
		o.window_accepts = accepts[i];
		o.window_rejects = rejects[i];
		if (ops[i].has_tuning)
			o.tuning = tunings[i];
	}
	step_ = step;
	uint64_t rs[4];
	for (int k = 0; k < 4; ++k)
		rs[k] = mix64(rng_words[k] ^ mix64((uint64_t)k));
	ch.rng.set_state(rs);
	// update calculators and priors, then accept (mcmc.rs:205-218)
	send_model(ch, true);
	if (cfg_.num_categories > 1)
		ch.calc->set_gamma(ch.alpha.v);
	lists(ch);
	ch.calc->propose_lengths(ch.internals.data(), ch.children.data(),
				 (uint32_t)ch.internals.size(), ch.lengths.data(), 1.0);
	ch.lnl_cache = ch.calc->log_likelihood();
	ch.calc->accept();
	ch.tree->accept();
	ch.prior_cache = prior(ch);
	ch.launched = ch.model_sent = ch.alpha_sent = false;
}

} // namespace b3g
