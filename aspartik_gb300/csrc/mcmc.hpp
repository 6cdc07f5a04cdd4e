// mcmc.hpp -- native MCMC driver around the device likelihood.
//
// Restates the step of b3's engine (crates/b3/src/mcmc.rs:314-393):
// operator proposal -> prior (reject at -inf before any likelihood work) ->
// likelihood -> Metropolis-Hastings -> accept or reject of every parameter,
// the tree and the likelihood.  Operators follow python/aspartik/b3/
// operators (TreeScale, ScaleReal, SubtreeSlide, BeastNarrowExchange,
// BeastWideExchange, NodeSlide, RootSlide, UpDown, DeltaExchange) and the
// priors python/aspartik/b3/config/__init__.py:660-800 (Yule, LogNormal,
// SymmetricDirichlet).  Beyond the reference it
// runs several chains at once (independent replicates or Metropolis-coupled
// temperatures) and evaluates the proposals of all chains before reading
// any result back, so their GPU work overlaps.
#pragma once

#include "batch.hpp"
#include "calculator.hpp"
#include "host_pool.hpp"
#include "mlp.hpp"
#include "tree.hpp"

#include <cstdint>
#include <memory>
#include <vector>

namespace b3g {

// xoshiro256** (Blackman and Vigna), seeded through splitmix64
class Rng {
      public:
	explicit Rng(uint64_t seed);
	uint64_t next();
	double uniform();            // [0, 1)
	uint32_t below(uint32_t n);  // [0, n)
	void get_state(uint64_t out[4]) const
	{
		for (int k = 0; k < 4; ++k)
			out[k] = s_[k];
	}
	void set_state(const uint64_t in[4])
	{
		for (int k = 0; k < 4; ++k)
			s_[k] = in[k];
	}

      private:
	uint64_t s_[4];
};

struct Real {
	double v = 0.0, backup = 0.0;
	bool changed = false;
	void set(double x)
	{
		if (!changed) {
			backup = v;
			changed = true;
		}
		v = x;
	}
	void accept() { changed = false; }
	void reject()
	{
		if (changed)
			v = backup;
		changed = false;
	}
};

struct RealVec {
	std::vector<double> v, backup;
	bool changed = false;
	void set(size_t i, double x)
	{
		if (!changed) {
			backup = v;
			changed = true;
		}
		v[i] = x;
	}
	void accept() { changed = false; }
	void reject()
	{
		if (changed)
			v = backup;
		changed = false;
	}
};

enum OpKind : uint32_t {
	kOpTreeScale = 0,
	kOpSubtreeSlide,
	kOpNarrowExchange,
	kOpScaleKappa,
	kOpScaleAlpha,
	kOpScaleBirthRate,
	kOpDeltaRates,
	kOpDeltaFreqs,
	kOpRelaxedCategory, // one edge's relaxed-clock category
	kOpScaleClockSd,    // the relaxed clock's LogNormal sd
	kOpNodeSlide,       // one internal height between parent and children
	kOpRootSlide,       // the root height, scaled above its older child
	kOpUpDown,          // tree heights up, birth rate down (or reverse)
	kOpWideExchange,    // parents of two random nodes swapped
	kOpCount
};

struct OpStats {
	uint64_t accepts = 0, rejects = 0, aborts = 0, prior_rejects = 0;
	uint64_t window_accepts = 0, window_rejects = 0;
	double tuning = 0.75;
};

// One alignment of the driver with the start tree of its chains.
struct Problem {
	uint32_t L, P;
	const uint8_t *samples;
	const uint32_t *weights;
	const uint32_t *parents;
	const double *heights;
};

enum : uint32_t {
	kLaunchStreams = 0, // one launch per chain, each chain on its own stream
	kLaunchBatch = 1,   // every chain of a step in one graph-replayed batch
	// each chain on its own stream, and the chains advance independently
	// between the driver's synchronisation points (MC3 swap attempts,
	// operator tuning, the end of the delayed-acceptance pilot, the end of
	// a run)
	kLaunchIndependent = 2,
};

// Parameters of a state file in the reference's layout (Mcmc::dump,
// crates/b3/src/mcmc.rs:251-268), in the order its Mcmc lists them.
enum VerbatimParam : uint32_t {
	kVpTree = 0,         // DatedTree: parents, heights (tree.rs:1012-1016)
	kVpBirthRate,        // Real: f64 (real.rs:59-62)
	kVpKappa,            // Real
	kVpAlpha,            // Real
	kVpRates,            // RealVector: 6 f64 (real_vector.rs:77-82)
	kVpFreqs,            // RealVector: 4 f64
	kVpClockSd,          // Real
	kVpClockCategories,  // ClassVector: u32 per node (class_vector.rs:82-87)
	kVpCount
};

// One operator of the reference's scheduler: which of this driver's
// operator kinds it is, and whether it has a tuning parameter (its dump then
// carries one, operators/mod.rs:208-219).
struct VerbatimOp {
	uint32_t op;
	uint32_t has_tuning;
};

struct McmcConfig {
	uint32_t num_chains;
	uint32_t num_categories;
	uint32_t precision;
	uint32_t model; // 0 HKY, 1 GTR
	uint64_t seed;
	double heat;          // beta_i = 1 / (1 + heat * i)
	uint32_t swap_every;  // steps between swap attempts, 0 = never
	uint32_t sample_every;
	uint32_t tune_every;  // steps between operator tunings, 0 = never
	int32_t device;
	double weights[kOpCount];
	// delayed acceptance (0 pilot steps: off)
	uint32_t da_pilot_steps;
	uint32_t da_epochs;
	uint32_t da_hidden;
	double da_drift_limit;
	uint32_t clock_categories; // 0: strict clock
	uint32_t launch;           // kLaunch*
	// host threads that step the chains (0: one for every four chains, one
	// per chain with independent stepping, at most 8 and at most the
	// hardware threads, and the calling thread alone in the batched launch
	// mode; 1: the calling thread alone); the results do not depend on it
	uint32_t host_threads;
};

// Inputs of the surrogate, for the moves that re-evaluate the whole tree
// (tree scale, up-down, kappa, alpha, exchangeabilities, frequencies): 5
// length summaries of the tree (log of the tree length, the root height,
// the internal and the external edge lengths' sums, and log alpha) and 9
// model parameters (log exchangeabilities or log kappa, three frequencies).
constexpr uint32_t kDaInputs = 14;

// Parameters of one sample: kappa, alpha, birth rate, 6 exchangeabilities,
// 4 frequencies, relaxed-clock sd.
constexpr uint32_t kSampleParams = 14;

struct DaStats {
	uint64_t pilot_pairs = 0, stage1_rejects = 0, stage2_accepts = 0,
		 stage2_rejects = 0, exact_evaluations = 0, fallback = 0;
	double train_loss = 0.0, drift_rms = 0.0;
};

struct Chain {
	std::unique_ptr<DatedTree> tree;
	std::unique_ptr<Calculator> calc;
	Rng rng;
	Real kappa, alpha, birth_rate;
	RealVec rates, freqs;
	// relaxed clock: category of every edge (by child node), LogNormal sd
	// and the category rates it gives
	std::vector<uint32_t> edge_cat;
	bool cat_changed = false;
	uint32_t cat_edge = 0, cat_old = 0; // the proposal's change
	Real clock_sd;
	std::vector<double> clock_rates;
	double beta = 1.0;
	uint32_t index = 0;
	uint32_t problem = 0; // the alignment, and the chain's temperature group
	double lnl_cache = 0.0, lnl_new = 0.0;
	double prior_cache = 0.0, prior_new = 0.0;
	bool launched = false;   // a device evaluation is pending
	bool model_sent = false; // the device holds a not yet accepted model
	bool alpha_sent = false;
	// per-step state
	uint32_t op = 0;
	double hastings = 0.0;
	int status = 0; // 0 pending, 1 abort, 2 prior reject, 3 stage-1 reject
	bool screenable = false; // a whole-tree move with surrogate inputs
	bool screened = false; // passed stage one of delayed acceptance
	double da_delta = 0.0; // surrogate f(x_new) - f(x_old)
	float feat_old[kDaInputs], feat_new[kDaInputs];
	// the step's outcome, for the statistics gathered in chain order
	bool accepted = false;
	bool evaluated = false; // an exact evaluation was read
	bool finite = false;    // ... and gave a finite log-likelihood
	double dlnl = 0.0;      // its difference to the current state's
	std::vector<uint32_t> internals, children;
	std::vector<double> lengths;
	// independent stepping: the chain's own statistics since the last
	// synchronisation point (merged into the driver's there), its pilot
	// pairs (concatenated in chain order for training), and its own
	// delayed-acceptance drift window and screening switch
	OpStats acc_ops[kOpCount];
	DaStats acc_da;
	std::vector<float> pilot_old, pilot_new, pilot_delta;
	std::vector<double> drift;
	size_t drift_pos = 0;
	bool da_on = false;
	explicit Chain(uint64_t seed) : rng(seed) {}
};

class Mcmc {
      public:
	Mcmc(const McmcConfig &cfg, uint32_t L, uint32_t P,
	     const uint8_t *samples, const uint32_t *weights,
	     const uint32_t *parents, const double *heights);
	// Several alignments: num_chains / problems.size() chains per problem,
	// chain i on problem i / that count at temperature index i % that count
	// (MC3 swaps only between chains of one problem).
	Mcmc(const McmcConfig &cfg, const std::vector<Problem> &problems);

	void set_clock(double sd, const uint32_t *categories);
	void set_parameters(double kappa, const double *rates,
			    const double *freqs, double alpha,
			    double birth_rate);
	void run(uint64_t steps);
	// cold-chain trace: 0 lnL, 1 prior, 2 posterior, 3 root height,
	// 4 kappa or rates[0], 5 alpha, 6 tree length
	const std::vector<double> &trace(uint32_t field) const
	{
		return trace_[field];
	}
	// the same fields for each chain in chain order (chain i's state,
	// whatever temperature MC3 swaps have given it)
	const std::vector<double> &chain_trace(uint32_t chain, uint32_t field) const
	{
		return chain_trace_.at((size_t)chain * 8 + field);
	}
	size_t chain_trace_size() const { return chain_trace_.size(); }
	void op_stats(uint32_t op, uint64_t out[4], double *tuning) const;
	// the operator's tuning parameter (a start value, e.g. carried over
	// from a burn-in run)
	void set_tuning(uint32_t op, double tuning);
	// samples: steps[n], parents[n][nodes], heights[n][nodes],
	// parameters[n][kSampleParams]
	uint64_t num_samples() const { return sample_steps_.size(); }
	const std::vector<uint64_t> &sample_steps() const { return sample_steps_; }
	const std::vector<uint32_t> &sample_parents() const { return sample_parents_; }
	const std::vector<double> &sample_heights() const { return sample_heights_; }
	const std::vector<double> &sample_params() const { return sample_params_; }
	const DaStats &da_stats() const { return da_; }
	uint64_t swaps_accepted() const { return swaps_accepted_; }
	uint64_t swaps_tried() const { return swaps_tried_; }
	uint64_t steps_done() const { return step_; }
	// Full recompute of every chain from scratch against its cached value;
	// returns the largest relative difference.  Between steps only.
	double check_full_recompute();
	void chain_state(uint32_t chain, uint32_t *parents, double *heights,
			 double *lnl, double *beta) const;
	uint32_t num_chains() const { return (uint32_t)chains_.size(); }
	uint32_t chain_nodes(uint32_t chain) const
	{
		return chains_.at(chain)->tree->num_nodes();
	}
	uint32_t num_problems() const { return num_problems_; }
	bool batched() const { return batch_ != nullptr; }
	// device time of the batched launches so far (ms) and their count
	double batch_device_ms() const { return batch_ms_; }
	uint64_t batch_launches() const { return batch_runs_; }
	// Checkpoint (mcmc_state.cpp): everything later steps depend on, between
	// steps; load needs a driver built with the same configuration and
	// data and continues bit for bit as the dumped run would have.
	std::vector<uint8_t> dump() const;
	void load(const uint8_t *state, size_t size);
	// A state in the reference's own layout (mcmc_verbatim.cpp) for one
	// chain: its parameters in the order `params` gives, the operators'
	// statistics and tunings in the order `ops` gives, the step and the
	// chain's posterior; load takes such a state (written by either) into
	// the chain and the driver's step and operators, and re-evaluates.
	std::vector<uint8_t> dump_verbatim(uint32_t chain, const uint32_t *params,
					   uint32_t num_params, const VerbatimOp *ops,
					   uint32_t num_ops) const;
	void load_verbatim(uint32_t chain, const uint32_t *params,
			   uint32_t num_params, const VerbatimOp *ops,
			   uint32_t num_ops, const uint8_t *state, size_t size);

      private:
	void propose(Chain &ch);
	// the tree's dirty lists with the per-edge lengths (relaxed clock:
	// times the edge's category rate)
	void lists(Chain &ch);
	void clock_rates(Chain &ch);
	double prior(const Chain &ch) const;
	void sync_model(Chain &ch);
	void launch(Chain &ch);
	// propose and prior (any host thread)
	void prepare(Chain &ch);
	// read the result, Metropolis-Hastings, accept or reject the chain's
	// state (any host thread)
	void settle(Chain &ch);
	// the step's statistics of one chain (calling thread, chain order)
	void tally(const Chain &ch);
	struct TallySink {
		OpStats *ops; // [kOpCount]
		DaStats *da;
		std::vector<double> *drift;
		size_t *drift_pos;
		bool *screening; // cleared when the drift exceeds its limit
		std::vector<float> *pilot_old, *pilot_new, *pilot_delta;
	};
	void tally_into(const Chain &ch, const TallySink &sink);
	// independent stepping (kLaunchIndependent): `steps` steps in windows
	// between synchronisation points; a window's steps of the chains of
	// host thread w; the same statistics as tally() into the chain's own
	// accumulators; their merge at a synchronisation point
	void run_independent(uint64_t steps);
	void window(uint32_t w, uint32_t threads, uint64_t first_step, uint64_t count);
	void tally_own(Chain &ch);
	void merge_own();
	// screening of the listed chains' pending proposals through surrogate
	// inference context ctx (one launch)
	void screen_chains(const std::vector<uint32_t> &idx, uint32_t ctx,
			   std::vector<float> &xn, std::vector<float> &xo,
			   std::vector<float> &out);
	// chain i's trace fields (and, for the cold chain, its sample) at
	// step `step`
	void record_chain(size_t i, bool cold, uint64_t step);
	size_t cold_chain() const;
	void swap_temperatures();
	void tune();
	void record();
	double send_model(Chain &ch, bool mark_all);
	void features(const Chain &ch, float *out) const;
	void screen_all();
	void train_surrogate();

	McmcConfig cfg_;
	uint32_t num_problems_ = 1;
	std::vector<std::unique_ptr<Chain>> chains_;
	// host threads of the step (none: the calling thread alone)
	std::unique_ptr<HostPool> pool_;
	// the step's screened chains and the surrogate's inputs and outputs
	std::vector<uint32_t> screen_idx_;
	std::vector<float> screen_xn_, screen_xo_, screen_out_;
	double batch_ms_ = 0.0;
	uint64_t batch_runs_ = 0;
	// FP32 chosen form: every chain's proposal of a step is evaluated by
	// one graph replay of a batch
	std::unique_ptr<Batch> batch_;
	std::vector<double> batch_lnl_;
	OpStats ops_[kOpCount];
	double weight_total_ = 0.0;
	uint64_t step_ = 0;
	uint64_t swaps_tried_ = 0, swaps_accepted_ = 0;
	uint32_t tune_rounds_ = 0;
	Rng swap_rng_;
	std::vector<double> trace_[8];
	std::vector<std::vector<double>> chain_trace_; // [chain * 8 + field]
	// per sample: the step, the cold chain's tree (parents and heights of
	// every node) and its parameters (kSampleParams values)
	std::vector<uint64_t> sample_steps_;
	std::vector<uint32_t> sample_parents_;
	std::vector<double> sample_heights_, sample_params_;

	// delayed acceptance: pilot pairs, the trained surrogate, input and
	// output normalisation, the drift window of (exact - surrogate)
	std::unique_ptr<Mlp> surrogate_;
	bool da_active_ = false;
	std::vector<float> pilot_old_, pilot_new_, pilot_delta_;
	float in_mean_[kDaInputs] = {}, in_scale_[kDaInputs] = {};
	double out_scale_ = 1.0;
	std::vector<double> drift_;
	size_t drift_pos_ = 0;
	DaStats da_;
	bool tuned_ = false; // the calculators' launch configuration is tuned
};

} // namespace b3g
