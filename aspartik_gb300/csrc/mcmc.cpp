// mcmc.cpp -- native MCMC driver (see mcmc.hpp).
#include "mcmc.hpp"

#include <cstdlib>
#include "host_math.hpp"

#include <algorithm>
#include <cmath>
#include <limits>

namespace b3g {

// ---------------------------------------------------------------------------
// RNG

namespace {

uint64_t splitmix64(uint64_t &x)
{
	uint64_t z = (x += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

const double kNegInf = -std::numeric_limits<double>::infinity();

double lognormal_lnpdf(double x, double mu, double sigma)
{
	if (!(x > 0.0))
		return kNegInf;
	const double z = (std::log(x) - mu) / sigma;
	return -std::log(x * sigma * std::sqrt(2.0 * M_PI)) - 0.5 * z * z;
}

// SymmetricDirichlet (crates/b3/src/priors/dirichlet.rs:22-36): the
// concentration is sum / k; the values are not required to sum to 1
double sym_dirichlet_lnpdf(const std::vector<double> &x, double sum)
{
	const double k = static_cast<double>(x.size());
	const double a = sum / k;
	double out = std::lgamma(sum) - k * std::lgamma(a);
	for (const double v : x)
		out += (a - 1.0) * std::log(v);
	return out;
}

} // namespace

Rng::Rng(uint64_t seed)
{
	uint64_t x = seed;
	for (auto &w : s_)
		w = splitmix64(x);
}

uint64_t Rng::next()
{
	const uint64_t result = rotl(s_[1] * 5, 7) * 9;
	const uint64_t t = s_[1] << 17;
	s_[2] ^= s_[0];
	s_[3] ^= s_[1];
	s_[1] ^= s_[2];
	s_[0] ^= s_[3];
	s_[2] ^= t;
	s_[3] = rotl(s_[3], 45);
	return result;
}

double Rng::uniform() { return (next() >> 11) * 0x1.0p-53; }

uint32_t Rng::below(uint32_t n)
{
	return static_cast<uint32_t>((static_cast<unsigned __int128>(next()) * n) >> 64);
}

// ---------------------------------------------------------------------------

Mcmc::Mcmc(const McmcConfig &cfg, uint32_t L, uint32_t P,
	   const uint8_t *samples, const uint32_t *weights,
	   const uint32_t *parents, const double *heights)
    : Mcmc(cfg, std::vector<Problem>{Problem{L, P, samples, weights, parents, heights}})
{
}

Mcmc::Mcmc(const McmcConfig &cfg, const std::vector<Problem> &problems)
    : cfg_(cfg), swap_rng_(cfg.seed ^ 0x5EEDu)
{
	if (cfg.num_chains < 1 || cfg.num_chains > 256)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "num_chains must be 1..256");
	if (problems.empty() || cfg.num_chains % problems.size() != 0)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "num_chains must be a multiple of the number of problems");
	num_problems_ = (uint32_t)problems.size();
	if (num_problems_ > 1 && cfg.da_pilot_steps)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "delayed acceptance needs a single problem (one surrogate "
			    "per alignment)");
	if (cfg.model > 1)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "model must be 0 (HKY) or 1 (GTR)");
	if (cfg.launch > kLaunchIndependent)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "unknown launch mode");
	for (uint32_t k = 0; k < kOpCount; ++k) {
		if (!(cfg.weights[k] >= 0.0) || !std::isfinite(cfg.weights[k]))
			throw Error(B3G_ERR_INVALID_ARGUMENT, "bad operator weight");
		weight_total_ += cfg.weights[k];
	}
	if (!(weight_total_ > 0.0))
		throw Error(B3G_ERR_INVALID_ARGUMENT, "all operator weights are 0");
	// DeltaExchange starts at tuning 0.75 like the scale operators
	for (auto &o : ops_)
		o.tuning = 0.75;
	const uint32_t group = cfg.num_chains / num_problems_;
	for (uint32_t i = 0; i < cfg.num_chains; ++i) {
		const Problem &pr = problems[i / group];
		if (!pr.samples || !pr.weights || !pr.parents || !pr.heights)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "null problem array");
		b3g_config cc{};
		cc.num_leaves = pr.L;
		cc.num_patterns = pr.P;
		cc.num_states = 4;
		cc.num_categories = cfg.num_categories;
		cc.precision = cfg.precision;
		cc.scale_ln = 30;
		cc.device = cfg.device;
		auto ch = std::make_unique<Chain>(cfg.seed + 0x9E37u * (i + 1));
		try {
			ch->tree = std::make_unique<DatedTree>(pr.parents, pr.heights,
							       2 * pr.L - 1);
		} catch (const std::exception &e) {
			throw Error(B3G_ERR_INVALID_ARGUMENT, e.what());
		}
		ch->calc = std::make_unique<Calculator>(cc, pr.samples);
		ch->calc->set_timing(false); // the driver reads no kernel timings
		ch->calc->set_weights(pr.weights);
		ch->beta = 1.0 / (1.0 + cfg.heat * (i % group));
		ch->index = i;
		ch->problem = i / group;
		ch->kappa.v = 2.0;
		ch->alpha.v = 0.5;
		ch->birth_rate.v = 1.0;
		ch->rates.v.assign(6, 1.0);
		ch->freqs.v.assign(4, 0.25);
		if (cfg.clock_categories) {
			const uint32_t nodes = 2 * pr.L - 1;
			ch->edge_cat.resize(nodes);
			for (uint32_t v = 0; v < nodes; ++v)
				ch->edge_cat[v] = v % cfg.clock_categories;
			ch->clock_sd.v = 0.3;
			clock_rates(*ch);
		}
		chains_.push_back(std::move(ch));
	}
	set_parameters(2.0, nullptr, nullptr, 0.5, 1.0);
	// every chain of a step in one graph-replayed batched launch (FP32
	// chosen form, several chains), or each chain's launches on its own
	// stream, the launches of a step running concurrently
	bool use_batch = cfg.launch == kLaunchBatch;
	if (const char *env = std::getenv("B3G_MCMC_BATCH"))
		if (cfg.launch != kLaunchIndependent)
			use_batch = std::atoi(env) != 0;
	if (use_batch && (cfg.precision != B3G_PRECISION_F32 || chains_.size() < 2))
		use_batch = false;
	if (use_batch) {
		std::vector<Calculator *> calcs;
		for (auto &ch : chains_)
			calcs.push_back(ch->calc.get());
		batch_ = std::make_unique<Batch>(calcs.data(), (uint32_t)calcs.size());
		batch_lnl_.assign(calcs.size(), 0.0);
	}
	uint32_t threads = cfg.host_threads;
	if (const char *env = std::getenv("B3G_MCMC_THREADS"))
		threads = (uint32_t)std::max(0, std::atoi(env));
	// automatic: a thread for every four chains, at most 8; the batched
	// mode's host work per chain is a few copies, so it keeps to the
	// calling thread unless asked otherwise
	// (independent stepping: a thread per chain, at most 8)
	if (threads == 0)
		threads = batch_ ? 1u
			  : std::min<uint32_t>(
				    {cfg.launch == kLaunchIndependent
					     ? (uint32_t)chains_.size()
					     : ((uint32_t)chains_.size() + 3) / 4,
				     8u, std::max(1u, std::thread::hardware_concurrency())});
	threads = std::min<uint32_t>(threads, (uint32_t)chains_.size());
	if (threads > 1) {
		const int dev = cfg.device;
		pool_ = std::make_unique<HostPool>(threads, [dev] {
			check_cuda(cudaSetDevice(dev), "cudaSetDevice");
		});
	}
}

double Mcmc::send_model(Chain &ch, bool mark_all)
{
	if (cfg_.model == 1) {
		ch.calc->set_reversible(ch.rates.v.data(), ch.freqs.v.data(), 1);
	} else {
		double V[16], Vi[16], lam[4], Q[16];
		hky_eigen(ch.kappa.v, ch.freqs.v.data(), V, Vi, lam, Q);
		ch.calc->set_eigen(V, Vi, lam, Q, ch.freqs.v.data(), 1);
	}
	if (mark_all)
		ch.tree->mark_all_edges_updated();
	return 0.0;
}

void Mcmc::set_parameters(double kappa, const double *rates,
			  const double *freqs, double alpha, double birth_rate)
{
	for (auto &chp : chains_) {
		Chain &ch = *chp;
		ch.kappa.v = kappa;
		if (rates)
			ch.rates.v.assign(rates, rates + 6);
		if (freqs)
			ch.freqs.v.assign(freqs, freqs + 4);
		ch.alpha.v = alpha;
		ch.birth_rate.v = birth_rate;
		send_model(ch, true);
		if (cfg_.num_categories > 1)
			ch.calc->set_gamma(alpha);
		// DnaLikelihood::new: mark all, evaluate, accept (dna.rs:34-66)
		lists(ch);
		ch.calc->propose_lengths(ch.internals.data(), ch.children.data(),
					 (uint32_t)ch.internals.size(),
					 ch.lengths.data(), 1.0);
	}
	for (auto &chp : chains_) {
		Chain &ch = *chp;
		ch.lnl_cache = ch.calc->log_likelihood();
		ch.calc->accept();
		ch.tree->accept();
		ch.prior_cache = prior(ch);
		ch.launched = ch.model_sent = ch.alpha_sent = false;
	}
	// the launch configuration for this alignment and GPU, tuned once on
	// the whole tree (trial proposals are rejected)
	if (cfg_.precision == B3G_PRECISION_F32 && !tuned_) {
		for (auto &chp : chains_)
			chp->calc->autotune(chp->internals.data(), chp->children.data(),
					    (uint32_t)chp->internals.size(),
					    chp->lengths.data(), 1.0);
		tuned_ = true;
	}
}

// Yule (priors/yule.rs:23-40), LogNormal parameter priors and symmetric
// Dirichlet priors as _b3_config sets them up (config/__init__.py:660-730);
// the Gamma shape gets LogNormal(0, 1).
double Mcmc::prior(const Chain &ch) const
{
	const DatedTree &t = *ch.tree;
	const double lam = ch.birth_rate.v;
	double out = static_cast<double>(t.num_internals()) * std::log(lam);
	for (uint32_t v = t.num_leaves(); v < t.num_nodes(); ++v) {
		const double diff = -lam * t.height(v);
		out += diff;
		if (v == t.root())
			out += diff;
	}
	out += lognormal_lnpdf(lam, 1.0, 1.5);
	if (cfg_.model == 0) {
		out += lognormal_lnpdf(ch.kappa.v, 1.0, 1.25);
	} else {
		out += sym_dirichlet_lnpdf(ch.rates.v, 6.0);
	}
	out += sym_dirichlet_lnpdf(ch.freqs.v, 1.0);
	if (cfg_.num_categories > 1)
		out += lognormal_lnpdf(ch.alpha.v, 0.0, 1.0);
	if (cfg_.clock_categories) {
		// relaxed-clock sd ~ Exponential(mean 1/3); categories uniform
		const double sd = ch.clock_sd.v;
		out += sd > 0.0 ? std::log(3.0) - 3.0 * sd : kNegInf;
	}
	return std::isnan(out) ? kNegInf : out;
}

void Mcmc::clock_rates(Chain &ch)
{
	ch.clock_rates.resize(cfg_.clock_categories);
	lognormal_categories(ch.clock_sd.v, (int)cfg_.clock_categories,
			     ch.clock_rates.data());
}

void Mcmc::lists(Chain &ch)
{
	ch.tree->partials_lists(ch.internals, ch.children, ch.lengths);
	if (!cfg_.clock_categories)
		return;
	// RelaxedClock::get_rate (clock.rs:118-122): edge id = child node
	for (size_t k = 0; k < ch.lengths.size(); ++k)
		ch.lengths[k] *= ch.clock_rates[ch.edge_cat[ch.children[k]]];
}

void Mcmc::set_clock(double sd, const uint32_t *categories)
{
	const uint32_t K = cfg_.clock_categories;
	if (!K)
		throw Error(B3G_ERR_STATE, "the chains use a strict clock");
	if (!(sd > 0.0) || !std::isfinite(sd))
		throw Error(B3G_ERR_INVALID_ARGUMENT, "clock sd must be finite and > 0");
	if (categories && num_problems_ > 1)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "per-node clock categories need a single problem");
	for (auto &chp : chains_) {
		Chain &ch = *chp;
		const uint32_t nodes = ch.tree->num_nodes();
		for (uint32_t v = 0; v < nodes; ++v) {
			const uint32_t c = categories ? categories[v] : v % K;
			if (c >= K && v != ch.tree->root())
				throw Error(B3G_ERR_INVALID_ARGUMENT,
					    "clock category out of range");
			ch.edge_cat[v] = c < K ? c : 0;
		}
		ch.clock_sd.v = sd;
		clock_rates(ch);
	}
}

namespace {

// intersections (operators/_subtree_slide.py): the nodes under `node`
// whose parent edge crosses `height`
void intersections(const DatedTree &t, uint32_t node, double height,
		   std::vector<uint32_t> &out)
{
	if (t.height(node) < height) {
		out.push_back(node);
		return;
	}
	if (!t.is_leaf(node)) {
		intersections(t, t.left(node), height, out);
		intersections(t, t.right(node), height, out);
	}
}

uint32_t random_nonroot(const DatedTree &t, Rng &rng)
{
	uint32_t v;
	do
		v = rng.below(t.num_nodes());
	while (v == t.root());
	return v;
}

// Moves whose likelihood is a whole-tree evaluation: every edge length or
// the substitution model changes.
bool is_global_move(uint32_t op)
{
	return op == kOpTreeScale || op == kOpUpDown || op == kOpScaleKappa ||
	       op == kOpScaleAlpha || op == kOpDeltaRates || op == kOpDeltaFreqs;
}

} // namespace

// One proposal per operator kind, restating python/aspartik/b3/operators.
void Mcmc::propose(Chain &ch)
{
	DatedTree &t = *ch.tree;
	double u = ch.rng.uniform() * weight_total_;
	uint32_t op = 0;
	for (; op + 1 < kOpCount; ++op) {
		if (u < cfg_.weights[op])
			break;
		u -= cfg_.weights[op];
	}
	while (cfg_.weights[op] == 0.0 && op > 0)
		--op;
	ch.op = op;
	ch.hastings = 0.0;
	ch.status = 0;
	ch.screenable = false;
	ch.screened = false;
	// delayed acceptance screens the moves that need a whole-tree
	// evaluation; their surrogate inputs before the move
	const bool global = cfg_.da_pilot_steps && is_global_move(op);
	if (global)
		features(ch, ch.feat_old);
	const double f = ops_[op].tuning;
	auto scale_factor = [&]() {
		// sample_range(f, 1 / f, Uniform(0, 1)) (operators/_util.py)
		return f + (1.0 / f - f) * ch.rng.uniform();
	};
	switch (op) {
	case kOpTreeScale: { // _tree_scale.py
		const double s = scale_factor();
		t.scale(s);
		ch.hastings = std::log(s) * (double(t.num_internals()) - 2.0);
		break;
	}
	case kOpScaleKappa:
	case kOpScaleAlpha:
	case kOpScaleBirthRate: { // _param_scale.py ScaleReal
		Real &r = op == kOpScaleKappa ? ch.kappa
			  : op == kOpScaleAlpha ? ch.alpha
						: ch.birth_rate;
		const double s = scale_factor();
		r.set(r.v * s);
		ch.hastings = -std::log(s);
		break;
	}
	case kOpDeltaRates:
	case kOpDeltaFreqs: { // _delta_exchange.py
		RealVec &vec = op == kOpDeltaRates ? ch.rates : ch.freqs;
		const double delta = ch.rng.uniform() * (1.0 - f) / 10.0;
		const uint32_t n = (uint32_t)vec.v.size();
		uint32_t d1 = ch.rng.below(n), d2 = d1;
		while (d2 == d1)
			d1 = ch.rng.below(n);
		vec.set(d1, vec.v[d1] - delta);
		vec.set(d2, vec.v[d2] + delta);
		break;
	}
	case kOpNarrowExchange: { // _tree_exchange.py BeastNarrowExchange
		if (t.num_internals() < 2) {
			ch.status = 1;
			break;
		}
		uint32_t node;
		do
			node = ch.rng.below(t.num_nodes());
		while (node == t.root() || t.parent_of(node) == t.root());
		const uint32_t parent = t.parent_of(node);
		const uint32_t gp = t.parent_of(parent);
		const uint32_t uncle = t.other_child(gp, parent);
		if (t.height(uncle) < t.height(parent)) {
			if (!t.swap_parents(node, uncle))
				ch.status = 1;
		} else {
			ch.status = 1;
		}
		break;
	}
	case kOpSubtreeSlide: { // _subtree_slide.py
		if (t.num_internals() < 2) {
			ch.status = 1;
			break;
		}
		const uint32_t node = random_nonroot(t, ch.rng);
		const uint32_t parent = t.parent_of(node);
		const uint32_t gp = t.parent_of(parent);
		const uint32_t sibling = t.other_child(parent, node);
		// distribution Uniform(-0.5, 0.5) times the tuning factor
		const double delta = (ch.rng.uniform() - 0.5) * f;
		const double old_h = t.height(parent);
		const double new_h = old_h + delta;
		std::vector<uint32_t> dest;
		if (delta > 0.0) {
			if (gp != kTombstone && t.height(gp) < new_h) {
				uint32_t new_child = parent, new_parent = gp;
				while (t.height(new_parent) < new_h) {
					new_child = new_parent;
					new_parent = t.parent_of(new_child);
					if (new_parent == kTombstone)
						break;
				}
				if (new_parent == kTombstone) {
					t.replace_child(parent, sibling, new_child);
					t.replace_child(gp, parent, sibling);
					t.set_root(parent);
				} else {
					t.replace_child(parent, sibling, new_child);
					t.replace_child(gp, parent, sibling);
					t.replace_child(new_parent, new_child, parent);
				}
				intersections(t, new_child, old_h, dest);
				ch.hastings = -std::log(double(dest.size()));
			}
		} else {
			if (t.height(node) > new_h) {
				ch.status = 1;
				break;
			}
			if (t.height(sibling) > new_h) {
				intersections(t, sibling, new_h, dest);
				if (dest.empty()) {
					ch.status = 1;
					break;
				}
				const uint32_t new_child = dest[ch.rng.below((uint32_t)dest.size())];
				const uint32_t new_parent = t.parent_of(new_child);
				if (gp == kTombstone) {
					t.replace_child(parent, sibling, new_child);
					t.replace_child(new_parent, new_child, parent);
					t.set_root(sibling);
				} else {
					t.replace_child(parent, sibling, new_child);
					t.replace_child(gp, parent, sibling);
					t.replace_child(new_parent, new_child, parent);
				}
				// The forward move picks one of |dest| destinations and
				// the reverse (upward) move is deterministic, so
				// q(x | x') / q(x' | x) = |dest|.  The reference's
				// _subtree_slide.py:94 returns -log(len(destinations))
				// here, which biases the tree; that sign is not copied
				// (BEAST's SubtreeSlideOperator uses +log).
				ch.hastings = std::log(double(dest.size()));
			}
		}
		t.set_height(parent, new_h);
		break;
	}
	case kOpRelaxedCategory: { // one edge's class (clock.rs:107-112)
		const uint32_t K = cfg_.clock_categories;
		if (K < 2) {
			ch.status = 1;
			break;
		}
		const uint32_t e = random_nonroot(t, ch.rng);
		uint32_t c = ch.rng.below(K - 1);
		if (c >= ch.edge_cat[e])
			++c;
		ch.cat_edge = e;
		ch.cat_old = ch.edge_cat[e];
		ch.edge_cat[e] = c;
		ch.cat_changed = true;
		t.mark_edge_updated(e);
		break;
	}
	case kOpScaleClockSd: { // ScaleReal on the sd; every rate changes
		if (!cfg_.clock_categories) {
			ch.status = 1;
			break;
		}
		const double s = scale_factor();
		ch.clock_sd.set(ch.clock_sd.v * s);
		ch.hastings = -std::log(s);
		clock_rates(ch);
		t.mark_all_edges_updated();
		break;
	}
	case kOpNodeSlide: { // _node_slide.py: uniform between parent and children
		if (t.num_internals() < 2) {
			ch.status = 1;
			break;
		}
		// random_nonroot_internal (tree.rs:799-809)
		uint32_t node;
		do
			node = t.num_leaves() + ch.rng.below(t.num_internals());
		while (node == t.root());
		const double upper = t.height(t.parent_of(node));
		const double lower = std::max(t.height(t.left(node)), t.height(t.right(node)));
		t.set_height(node, (upper - lower) * ch.rng.uniform() + lower);
		break;
	}
	case kOpRootSlide: { // _root.py: root height scaled above its older child
		const uint32_t root = t.root();
		const double s = scale_factor();
		const double lower = std::max(t.height(t.left(root)), t.height(t.right(root)));
		t.set_height(root, (t.height(root) - lower) * s + lower);
		ch.hastings = -std::log(s);
		break;
	}
	case kOpUpDown: { // _updown.py with up = the tree, down = the birth rate
		const double s = scale_factor();
		t.scale(s);
		ch.birth_rate.set(ch.birth_rate.v / s);
		// log(s) (dims up - dims down - 2): DatedTree::scale counts the
		// internals, Real::scale one value (tree.rs:335-348, real.rs:31)
		ch.hastings = std::log(s) * (double(t.num_internals()) - 1.0 - 2.0);
		break;
	}
	case kOpWideExchange: { // _tree_exchange.py BeastWideExchange
		const uint32_t a = random_nonroot(t, ch.rng);
		uint32_t b;
		do
			b = random_nonroot(t, ch.rng);
		while (b == a);
		const uint32_t pa = t.parent_of(a), pb = t.parent_of(b);
		if (pa != pb && a != pb && b != pa && t.height(a) < t.height(pb) &&
		    t.height(b) < t.height(pa)) {
			if (!t.swap_parents(a, b))
				ch.status = 1;
		} else {
			ch.status = 1;
		}
		break;
	}
	default:
		ch.status = 1;
	}
	if (global && ch.status == 0) {
		features(ch, ch.feat_new);
		ch.screenable = true;
	}
}

// The body of DnaLikelihood/GammaLikelihood::likelihood (dna.rs:68-100,
// gamma.rs:97-169) up to the asynchronous launch.
void Mcmc::launch(Chain &ch)
{
	const bool model_changed =
		ch.kappa.changed || ch.rates.changed || ch.freqs.changed;
	if (model_changed) {
		send_model(ch, true);
		ch.model_sent = true;
	}
	if (ch.alpha.changed && cfg_.num_categories > 1) {
		ch.calc->set_gamma(ch.alpha.v);
		ch.alpha_sent = true;
		ch.tree->mark_all_edges_updated();
	}
	if (!ch.tree->is_changed()) {
		ch.launched = false;
		ch.lnl_new = ch.lnl_cache;
		return;
	}
	lists(ch);
	if (batch_)
		ch.calc->stage_lengths(ch.internals.data(), ch.children.data(),
				       (uint32_t)ch.internals.size(),
				       ch.lengths.data(), 1.0);
	else
		ch.calc->propose_lengths(ch.internals.data(), ch.children.data(),
					 (uint32_t)ch.internals.size(),
					 ch.lengths.data(), 1.0);
	ch.launched = true;
}

// Surrogate inputs of the chain's current state (see kDaInputs).
void Mcmc::features(const Chain &ch, float *out) const
{
	const DatedTree &t = *ch.tree;
	auto lg = [](double x) { return (float)std::log(std::max(x, 1e-300)); };
	double inner = 0.0, outer = 0.0;
	for (uint32_t v = 0; v < t.num_nodes(); ++v) {
		if (v == t.root())
			continue;
		(t.is_leaf(v) ? outer : inner) += t.edge_length(v);
	}
	out[0] = lg(inner + outer);
	out[1] = lg(t.root_height());
	out[2] = lg(inner);
	out[3] = lg(outer);
	out[4] = cfg_.num_categories > 1 ? lg(ch.alpha.v) : 0.0f;
	for (uint32_t k = 0; k < 6; ++k)
		out[5 + k] = cfg_.model == 1 ? lg(ch.rates.v[k])
					     : (k == 0 ? lg(ch.kappa.v) : 0.0f);
	for (uint32_t k = 0; k < 3; ++k)
		out[11 + k] = (float)ch.freqs.v[k];
}

// Stage one of delayed acceptance (Christen and Fox, "Markov chain Monte
// Carlo using an approximation", J. Comput. Graph. Stat. 14(4), 2005): the
// proposal passes with probability min(1, r*), r* its MH ratio with the
// surrogate difference in place of the exact log-likelihood difference.
// Every pending screenable proposal of the step goes through one surrogate
// launch, before any chain's evaluation is queued (a launch behind them
// would wait for their blocks).
void Mcmc::screen_all()
{
	screen_idx_.clear();
	for (size_t i = 0; i < chains_.size(); ++i)
		if (chains_[i]->status == 0 && chains_[i]->screenable)
			screen_idx_.push_back((uint32_t)i);
	screen_chains(screen_idx_, 0, screen_xn_, screen_xo_, screen_out_);
}

void Mcmc::screen_chains(const std::vector<uint32_t> &idx, uint32_t ctx,
			 std::vector<float> &xn, std::vector<float> &xo,
			 std::vector<float> &out)
{
	const uint32_t n = (uint32_t)idx.size();
	if (n == 0)
		return;
	xn.resize((size_t)n * kDaInputs);
	xo.resize((size_t)n * kDaInputs);
	out.resize(n);
	for (uint32_t j = 0; j < n; ++j) {
		const Chain &ch = *chains_[idx[j]];
		for (uint32_t k = 0; k < kDaInputs; ++k) {
			xn[j * kDaInputs + k] = (ch.feat_new[k] - in_mean_[k]) * in_scale_[k];
			xo[j * kDaInputs + k] = (ch.feat_old[k] - in_mean_[k]) * in_scale_[k];
		}
	}
	surrogate_->deltas(ctx, xn.data(), xo.data(), n, out.data());
	for (uint32_t j = 0; j < n; ++j) {
		Chain &ch = *chains_[idx[j]];
		ch.da_delta = out_scale_ * (double)out[j];
		const double log_r1 =
			ch.beta * (ch.da_delta + ch.prior_new - ch.prior_cache) + ch.hastings;
		if (log_r1 > std::log(ch.rng.uniform()))
			ch.screened = true;
		else
			ch.status = 3;
	}
}

void Mcmc::train_surrogate()
{
	// independent stepping: the chains' pilot pairs, in chain order
	for (auto &chp : chains_) {
		Chain &ch = *chp;
		pilot_old_.insert(pilot_old_.end(), ch.pilot_old.begin(), ch.pilot_old.end());
		pilot_new_.insert(pilot_new_.end(), ch.pilot_new.begin(), ch.pilot_new.end());
		pilot_delta_.insert(pilot_delta_.end(), ch.pilot_delta.begin(),
				    ch.pilot_delta.end());
		ch.pilot_old.clear();
		ch.pilot_new.clear();
		ch.pilot_delta.clear();
	}
	const size_t n = pilot_delta_.size();
	if (n < 64) { // too few pairs: stay with the exact chain
		da_.fallback = 1;
		return;
	}
	for (uint32_t k = 0; k < kDaInputs; ++k) {
		double s = 0.0, s2 = 0.0;
		for (size_t i = 0; i < n; ++i) {
			const double a = pilot_old_[i * kDaInputs + k];
			const double b = pilot_new_[i * kDaInputs + k];
			s += a + b;
			s2 += a * a + b * b;
		}
		const double mean = s / (2.0 * n);
		const double var = std::max(s2 / (2.0 * n) - mean * mean, 0.0);
		in_mean_[k] = (float)mean;
		in_scale_[k] = var > 1e-20 ? (float)(1.0 / std::sqrt(var)) : 0.0f;
	}
	double m = 0.0, m2 = 0.0;
	for (const float d : pilot_delta_) {
		m += d;
		m2 += (double)d * d;
	}
	const double dvar = m2 / n - (m / n) * (m / n);
	out_scale_ = dvar > 1e-12 ? std::sqrt(dvar) : 1.0;
	std::vector<float> xo(pilot_old_.size()), xn(pilot_new_.size()), dl(n);
	for (size_t i = 0; i < n; ++i) {
		for (uint32_t k = 0; k < kDaInputs; ++k) {
			xo[i * kDaInputs + k] =
				(pilot_old_[i * kDaInputs + k] - in_mean_[k]) * in_scale_[k];
			xn[i * kDaInputs + k] =
				(pilot_new_[i * kDaInputs + k] - in_mean_[k]) * in_scale_[k];
		}
		dl[i] = (float)(pilot_delta_[i] / out_scale_);
	}
	surrogate_ = std::make_unique<Mlp>(kDaInputs, cfg_.da_hidden, cfg_.seed ^ 0xDAu,
					   cfg_.device);
	da_.train_loss = surrogate_->train(xn.data(), xo.data(), dl.data(),
					   (uint32_t)n, cfg_.da_epochs, 512, 1e-3f,
					   cfg_.seed ^ 0x7Au);
	da_active_ = true;
	drift_.assign(200, 0.0);
	drift_pos_ = 0;
	for (auto &chp : chains_) {
		chp->da_on = true;
		chp->drift.assign(200, 0.0);
		chp->drift_pos = 0;
	}
	if (pool_ && cfg_.launch == kLaunchIndependent)
		surrogate_->ensure_contexts(pool_->size());
}

void Mcmc::prepare(Chain &ch)
{
	propose(ch);
	if (ch.status != 0)
		return;
	ch.prior_new = prior(ch);
	if (ch.prior_new == kNegInf)
		ch.status = 2; // mcmc.rs:331-335
}

// Metropolis-Hastings and finalize_step (mcmc.rs:337-393); for a screened
// proposal, stage two of delayed acceptance: min(1, r / r*).  Touches the
// chain alone; tally() gathers the statistics.
void Mcmc::settle(Chain &ch)
{
	bool accept = false;
	ch.evaluated = ch.finite = false;
	if (ch.status == 0) {
		const double lnl = !ch.launched ? ch.lnl_cache
				   : batch_    ? batch_lnl_[ch.index]
					       : ch.calc->log_likelihood();
		ch.lnl_new = lnl;
		ch.evaluated = ch.launched;
		if (lnl != kNegInf && !std::isnan(lnl)) {
			ch.finite = true;
			ch.dlnl = lnl - ch.lnl_cache;
			if (ch.screened) {
				const double err = ch.dlnl - ch.da_delta;
				accept = ch.beta * err > std::log(ch.rng.uniform());
			} else {
				const double new_post = lnl + ch.prior_new;
				const double old_post = ch.lnl_cache + ch.prior_cache;
				const double ratio =
					ch.beta * (new_post - old_post) + ch.hastings;
				accept = ratio > std::log(ch.rng.uniform());
			}
		}
	}
	ch.accepted = accept;
	if (accept) {
		ch.tree->accept();
		ch.kappa.accept();
		ch.alpha.accept();
		ch.birth_rate.accept();
		ch.rates.accept();
		ch.freqs.accept();
		ch.clock_sd.accept();
		ch.cat_changed = false;
		if (ch.launched)
			ch.calc->accept();
		ch.lnl_cache = ch.lnl_new;
		ch.prior_cache = ch.prior_new;
	} else {
		const bool restore_model = ch.model_sent;
		const bool restore_alpha = ch.alpha_sent;
		ch.tree->reject();
		ch.kappa.reject();
		ch.alpha.reject();
		ch.birth_rate.reject();
		ch.rates.reject();
		ch.freqs.reject();
		if (ch.clock_sd.changed) {
			ch.clock_sd.reject();
			clock_rates(ch);
		}
		if (ch.cat_changed) {
			ch.edge_cat[ch.cat_edge] = ch.cat_old;
			ch.cat_changed = false;
		}
		if (ch.launched)
			ch.calc->reject();
		if (restore_model)
			send_model(ch, false);
		if (restore_alpha)
			ch.calc->set_gamma(ch.alpha.v);
	}
	ch.launched = false;
	ch.model_sent = false;
	ch.alpha_sent = false;
}

// In chain order, so the counters, the drift window and the surrogate's
// pilot pairs do not depend on the host threads.
// The step's statistics of one chain into `sink`: the driver's own
// counters, drift window and pilot pairs (lockstep) or the chain's
// (independent stepping).
void Mcmc::tally_into(const Chain &ch, const TallySink &sink)
{
	OpStats &st = sink.ops[ch.op];
	DaStats &da = *sink.da;
	if (ch.evaluated)
		++da.exact_evaluations;
	if (ch.status == 3)
		++da.stage1_rejects;
	if (ch.status == 0 && ch.finite) {
		if (ch.screened) {
			++(ch.accepted ? da.stage2_accepts : da.stage2_rejects);
			// drift of the screen: RMS of the last window of errors
			std::vector<double> &drift = *sink.drift;
			const double err = ch.dlnl - ch.da_delta;
			drift[(*sink.drift_pos)++ % drift.size()] = err * err;
			if (*sink.drift_pos >= drift.size()) {
				double sum = 0.0;
				for (const double e2 : drift)
					sum += e2;
				da.drift_rms = std::sqrt(sum / drift.size());
				if (cfg_.da_drift_limit > 0.0 && da.drift_rms > cfg_.da_drift_limit) {
					*sink.screening = false; // back to the exact chain
					da.fallback = 1;
				}
			}
		}
		// pilot pairs for the surrogate
		if (ch.screenable && cfg_.da_pilot_steps && !surrogate_ && da_.fallback == 0 &&
		    std::isfinite(ch.dlnl)) {
			sink.pilot_old->insert(sink.pilot_old->end(), ch.feat_old,
					       ch.feat_old + kDaInputs);
			sink.pilot_new->insert(sink.pilot_new->end(), ch.feat_new,
					       ch.feat_new + kDaInputs);
			sink.pilot_delta->push_back((float)ch.dlnl);
			++da.pilot_pairs;
		}
	}
	if (ch.status == 1)
		++st.aborts;
	else if (ch.status == 2)
		++st.prior_rejects;
	if (ch.accepted) {
		++st.accepts;
		++st.window_accepts;
	} else if (ch.status == 0 || ch.status == 3) {
		++st.rejects;
		++st.window_rejects;
	}
}

void Mcmc::tally(const Chain &ch)
{
	tally_into(ch, TallySink{ops_, &da_, &drift_, &drift_pos_, &da_active_, &pilot_old_,
				 &pilot_new_, &pilot_delta_});
}

// Metropolis coupling: adjacent temperatures exchange with probability
// min(1, exp((b_i - b_j) (post_j - post_i))); the betas move, not the states.
void Mcmc::swap_temperatures()
{
	const uint32_t group = (uint32_t)chains_.size() / num_problems_;
	if (group < 2)
		return;
	std::vector<uint32_t> by_beta(group);
	for (uint32_t g = 0; g < num_problems_; ++g) {
		for (uint32_t i = 0; i < group; ++i)
			by_beta[i] = g * group + i;
		std::sort(by_beta.begin(), by_beta.end(), [&](uint32_t a, uint32_t b) {
			return chains_[a]->beta > chains_[b]->beta;
		});
		const uint32_t k = swap_rng_.below(group - 1);
		Chain &a = *chains_[by_beta[k]];
		Chain &b = *chains_[by_beta[k + 1]];
		const double pa = a.lnl_cache + a.prior_cache;
		const double pb = b.lnl_cache + b.prior_cache;
		const double lr = (a.beta - b.beta) * (pb - pa);
		++swaps_tried_;
		if (lr > std::log(swap_rng_.uniform())) {
			std::swap(a.beta, b.beta);
			++swaps_accepted_;
		}
	}
}

// Operator tuning toward 0.234 acceptance (operators/mod.rs:165-193) with a
// rate that decays as 1/sqrt(round).
void Mcmc::tune()
{
	++tune_rounds_;
	const double r = 1.0 / std::sqrt(static_cast<double>(tune_rounds_));
	for (uint32_t k = 0; k < kOpCount; ++k) {
		OpStats &o = ops_[k];
		if (k == kOpNarrowExchange || k == kOpNodeSlide || k == kOpWideExchange)
			continue; // not tunable
		const double n = double(o.window_accepts + o.window_rejects);
		if (n == 0.0)
			continue;
		const double acc = double(o.window_accepts) / n;
		if (k == kOpSubtreeSlide) {
			// SubtreeSlide's factor multiplies the slide, so a larger
			// value is a bolder move: it grows when the acceptance is
			// above the target and shrinks below it, in log space (as
			// BEAST tunes its size), down to the node spacings of large
			// trees.  The reference applies the scale operators' rule
			// (operators/mod.rs:165-193, a larger factor being a smaller
			// move) to it as well, which drives a rarely accepted slide
			// to ever larger moves; that direction is not copied.
			o.tuning = std::clamp(o.tuning * std::exp(4.0 * r * (acc - 0.234)),
					      1e-6, 10.0);
		} else {
			o.tuning = std::clamp(o.tuning + r * (0.234 - acc), 0.01, 0.99);
		}
		o.window_accepts = o.window_rejects = 0;
	}
}

void Mcmc::set_tuning(uint32_t op, double tuning)
{
	if (op >= kOpCount)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "bad operator");
	const bool sub = op == kOpSubtreeSlide;
	if (!std::isfinite(tuning) || tuning < (sub ? 1e-6 : 0.01) ||
	    tuning > (sub ? 10.0 : 0.99))
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "tuning out of range (SubtreeSlide 1e-6..10, others 0.01..0.99)");
	ops_[op].tuning = tuning;
}

// The chain with the largest beta (the first of equals).
size_t Mcmc::cold_chain() const
{
	size_t cold = 0;
	for (size_t i = 1; i < chains_.size(); ++i)
		if (chains_[i]->beta > chains_[cold]->beta)
			cold = i;
	return cold;
}

void Mcmc::record_chain(size_t i, bool cold, uint64_t step)
{
	const Chain &ch = *chains_[i];
	const DatedTree &t = *ch.tree;
	double length = 0.0;
	for (uint32_t v = 0; v < t.num_nodes(); ++v)
		if (v != t.root())
			length += t.edge_length(v);
	const double f[8] = {ch.lnl_cache,
			     ch.prior_cache,
			     ch.lnl_cache + ch.prior_cache,
			     t.root_height(),
			     cfg_.model == 0 ? ch.kappa.v : ch.rates.v[0],
			     ch.alpha.v,
			     length,
			     cfg_.clock_categories ? ch.clock_sd.v : 0.0};
	for (uint32_t k = 0; k < 8; ++k)
		chain_trace_[i * 8 + k].push_back(f[k]);
	if (!cold)
		return;
	for (uint32_t k = 0; k < 8; ++k)
		trace_[k].push_back(f[k]);
	// the whole sample for trace files: tree and parameters
	sample_steps_.push_back(step);
	for (uint32_t v = 0; v < t.num_nodes(); ++v) {
		sample_parents_.push_back(t.parent_of(v));
		sample_heights_.push_back(t.height(v));
	}
	const double p[kSampleParams] = {
		ch.kappa.v,    ch.alpha.v,    ch.birth_rate.v, ch.rates.v[0],
		ch.rates.v[1], ch.rates.v[2], ch.rates.v[3],   ch.rates.v[4],
		ch.rates.v[5], ch.freqs.v[0], ch.freqs.v[1],   ch.freqs.v[2],
		ch.freqs.v[3], cfg_.clock_categories ? ch.clock_sd.v : 0.0};
	sample_params_.insert(sample_params_.end(), p, p + kSampleParams);
}

void Mcmc::record()
{
	chain_trace_.resize(chains_.size() * 8);
	const size_t cold = cold_chain();
	for (size_t i = 0; i < chains_.size(); ++i)
		record_chain(i, i == cold, step_);
}

void Mcmc::run(uint64_t steps)
{
	if (cfg_.launch == kLaunchIndependent) {
		run_independent(steps);
		return;
	}
	const uint32_t n = (uint32_t)chains_.size();
	// chain i on host thread i % T, each thread's chains in order
	auto each = [&](auto &&fn) {
		if (!pool_) {
			for (auto &ch : chains_)
				fn(*ch);
			return;
		}
		const uint32_t T = pool_->size();
		pool_->run([&](uint32_t w) {
			for (uint32_t i = w; i < n; i += T)
				fn(*chains_[i]);
		});
	};
	auto launch_pending = [&](Chain &ch) {
		if (ch.status == 0)
			launch(ch);
	};
	for (uint64_t s = 0; s < steps; ++s) {
		// the surrogate screens the step's proposals between their
		// preparation and the first launch; without it each thread goes
		// straight from a chain's proposal to its launch
		const bool screening = da_active_;
		if (screening) {
			each([&](Chain &ch) { prepare(ch); });
			screen_all();
		}
		if (batch_) {
			each([&](Chain &ch) {
				if (!screening)
					prepare(ch);
				launch_pending(ch);
			});
			bool any = false;
			for (auto &ch : chains_)
				any = any || ch->launched;
			if (any) {
				batch_->run();
				batch_->log_likelihoods(batch_lnl_.data());
				batch_ms_ += batch_->last_ms();
				++batch_runs_;
			}
			each([&](Chain &ch) { settle(ch); });
		} else {
			// every chain's device work is queued before any result is
			// read: by each thread for its own chains
			const uint32_t T = pool_ ? pool_->size() : 1;
			auto job = [&](uint32_t w) {
				for (uint32_t i = w; i < n; i += T) {
					if (!screening)
						prepare(*chains_[i]);
					launch_pending(*chains_[i]);
				}
				for (uint32_t i = w; i < n; i += T)
					settle(*chains_[i]);
			};
			if (pool_)
				pool_->run(job);
			else
				job(0);
		}
		for (auto &ch : chains_)
			tally(*ch);
		++step_;
		if (cfg_.da_pilot_steps && step_ == cfg_.da_pilot_steps && !surrogate_)
			train_surrogate();
		if (cfg_.swap_every && step_ % cfg_.swap_every == 0)
			swap_temperatures();
		if (cfg_.tune_every && step_ % cfg_.tune_every == 0)
			tune();
		if (cfg_.sample_every && step_ % cfg_.sample_every == 0)
			record();
	}
}

// Independent stepping.  Between two synchronisation points (an MC3 swap
// attempt, an operator tuning, the end of the delayed-acceptance pilot,
// the end of the call)
// every host thread advances its own chains on their own, reading only
// what stays fixed there (operator tunings, the surrogate, the
// configuration, the temperatures) and counting into the chains' own
// accumulators; at the point the counts are merged (integers: their order
// does not matter) and the driver swaps, tunes or trains.  Pilot pairs are concatenated in chain order
// when the surrogate is trained, and each chain keeps its own drift window.
// So the results depend neither on the thread count nor on how the steps
// are split into calls.
void Mcmc::run_independent(uint64_t steps)
{
	const uint32_t T = pool_ ? pool_->size() : 1;
	chain_trace_.resize(chains_.size() * 8);
	uint64_t left = steps;
	while (left > 0) {
		uint64_t k = left;
		if (cfg_.tune_every)
			k = std::min<uint64_t>(k, cfg_.tune_every - step_ % cfg_.tune_every);
		if (cfg_.da_pilot_steps && !surrogate_ && step_ < cfg_.da_pilot_steps)
			k = std::min<uint64_t>(k, cfg_.da_pilot_steps - step_);
		if (cfg_.swap_every)
			k = std::min<uint64_t>(k, cfg_.swap_every - step_ % cfg_.swap_every);
		const uint64_t at = step_;
		auto job = [&](uint32_t w) { window(w, T, at, k); };
		if (pool_)
			pool_->run(job);
		else
			job(0);
		merge_own();
		step_ += k;
		left -= k;
		if (cfg_.da_pilot_steps && step_ == cfg_.da_pilot_steps && !surrogate_)
			train_surrogate();
		if (cfg_.swap_every && step_ % cfg_.swap_every == 0)
			swap_temperatures();
		if (cfg_.tune_every && step_ % cfg_.tune_every == 0)
			tune();
		if (cfg_.sample_every && step_ % cfg_.sample_every == 0)
			record();
	}
}

void Mcmc::window(uint32_t w, uint32_t threads, uint64_t first_step, uint64_t count)
{
	const uint32_t n = (uint32_t)chains_.size();
	const size_t cold = cold_chain();
	std::vector<uint32_t> mine, idx;
	for (uint32_t i = w; i < n; i += threads)
		mine.push_back(i);
	std::vector<float> xn, xo, out;
	const bool screening = da_active_ && surrogate_;
	for (uint64_t s = 0; s < count; ++s) {
		const uint64_t step = first_step + s + 1;
		for (const uint32_t i : mine)
			prepare(*chains_[i]);
		if (screening) {
			idx.clear();
			for (const uint32_t i : mine) {
				const Chain &ch = *chains_[i];
				if (ch.da_on && ch.status == 0 && ch.screenable)
					idx.push_back(i);
			}
			screen_chains(idx, w, xn, xo, out);
		}
		for (const uint32_t i : mine)
			if (chains_[i]->status == 0)
				launch(*chains_[i]);
		for (const uint32_t i : mine) {
			settle(*chains_[i]);
			tally_own(*chains_[i]);
		}
		// a sample at the window's last step is taken at the
		// synchronisation point, after a swap there (as in lockstep)
		if (cfg_.sample_every && step % cfg_.sample_every == 0 && s + 1 < count)
			for (const uint32_t i : mine)
				record_chain(i, i == cold, step);
	}
}

// tally() into the chain's own accumulators, with its own drift window.
void Mcmc::tally_own(Chain &ch)
{
	tally_into(ch, TallySink{ch.acc_ops, &ch.acc_da, &ch.drift, &ch.drift_pos, &ch.da_on,
				 &ch.pilot_old, &ch.pilot_new, &ch.pilot_delta});
}

void Mcmc::merge_own()
{
	for (auto &chp : chains_) {
		Chain &ch = *chp;
		for (uint32_t k = 0; k < kOpCount; ++k) {
			OpStats &o = ops_[k];
			const OpStats &a = ch.acc_ops[k];
			o.accepts += a.accepts;
			o.rejects += a.rejects;
			o.aborts += a.aborts;
			o.prior_rejects += a.prior_rejects;
			o.window_accepts += a.window_accepts;
			o.window_rejects += a.window_rejects;
			ch.acc_ops[k] = OpStats{};
		}
		const DaStats &a = ch.acc_da;
		da_.pilot_pairs += a.pilot_pairs;
		da_.stage1_rejects += a.stage1_rejects;
		da_.stage2_accepts += a.stage2_accepts;
		da_.stage2_rejects += a.stage2_rejects;
		da_.exact_evaluations += a.exact_evaluations;
		da_.fallback |= a.fallback;
		da_.drift_rms = std::max(da_.drift_rms, a.drift_rms);
		ch.acc_da.pilot_pairs = ch.acc_da.stage1_rejects = 0;
		ch.acc_da.stage2_accepts = ch.acc_da.stage2_rejects = 0;
		ch.acc_da.exact_evaluations = 0;
	}
}

double Mcmc::check_full_recompute()
{
	double worst = 0.0;
	for (auto &chp : chains_) {
		Chain &ch = *chp;
		ch.tree->mark_all_edges_updated();
		lists(ch);
		ch.calc->propose_lengths(ch.internals.data(), ch.children.data(),
					 (uint32_t)ch.internals.size(),
					 ch.lengths.data(), 1.0);
		const double full = ch.calc->log_likelihood();
		ch.calc->reject();
		ch.tree->reject();
		const double rel = std::fabs(full - ch.lnl_cache) /
				   std::max(1.0, std::fabs(full));
		worst = std::max(worst, rel);
	}
	return worst;
}

void Mcmc::op_stats(uint32_t op, uint64_t out[4], double *tuning) const
{
	const OpStats &o = ops_[op];
	out[0] = o.accepts;
	out[1] = o.rejects;
	out[2] = o.aborts;
	out[3] = o.prior_rejects;
	*tuning = o.tuning;
}

void Mcmc::chain_state(uint32_t chain, uint32_t *parents, double *heights,
		       double *lnl, double *beta) const
{
	const Chain &ch = *chains_.at(chain);
	std::copy(ch.tree->parents().begin(), ch.tree->parents().end(), parents);
	std::copy(ch.tree->heights().begin(), ch.tree->heights().end(), heights);
	*lnl = ch.lnl_cache;
	*beta = ch.beta;
}

} // namespace b3g
