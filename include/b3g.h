/*
 * b3g.h -- C ABI of the GB300 (sm_103a) Felsenstein-pruning likelihood.
 *
 * The library replaces the likelihood path of the b3 MCMC engine of
 * kaathewisegit/aspartik (crate b3).  Two levels are exported:
 *
 *  1. Calculator level -- a drop-in for `trait Calculator<f64>`
 *     (crates/b3/src/calculator/mod.rs:54-76) as built by
 *     `CalculatorConfig::make4` (mod.rs:159-200).  The caller passes exactly
 *     what the reference's calculators consume: the children-first dirty list
 *     from `DatedTree::partials_lists` (parameters/tree.rs:456-461), the child
 *     transition matrices gathered by `Transitions::write_matrices`
 *     (transitions.rs:62-72) and the base frequencies.
 *
 *  2. Likelihood level -- a drop-in for the body of
 *     `DnaLikelihood::likelihood` / `GammaLikelihood::likelihood`
 *     (likelihood/dna.rs:68-100, likelihood/gamma.rs:97-169).  The caller
 *     passes the dirty list and the time lengths of the child edges; the
 *     device builds P(t) = V diag(exp(lambda r t)) V^-1 for every category,
 *     prunes, rescales, mixes the rate categories and returns the weighted
 *     root log-likelihood as one double.
 *
 * Conventions: every call returns a b3g_status; no exception crosses the ABI;
 * b3g_last_error() gives the message of the calling thread's last failure.
 * A handle belongs to one host thread at a time.  Device pointers are never
 * exposed.  Node ids follow the reference: leaves 0..L-1, internals L..2L-2,
 * edge id = child node id (tree.rs:728-736).  Matrices are row-major with
 * P[i][j] = Prob(i -> j).
 */
#ifndef B3G_H
#define B3G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define B3G_API __attribute__((visibility("default")))
#else
#define B3G_API
#endif

typedef enum b3g_status {
	B3G_OK = 0,
	B3G_ERR_INVALID_ARGUMENT = 1, /* bad size, index or order */
	B3G_ERR_OUT_OF_MEMORY = 2,    /* device or pinned host allocation */
	B3G_ERR_CUDA = 3,             /* CUDA runtime error */
	B3G_ERR_TIMEOUT = 4,          /* a bounded device wait gave up */
	B3G_ERR_NUMERIC = 5,          /* NaN/inf in a model input */
	B3G_ERR_STATE = 6             /* call out of order */
} b3g_status;

/* Arithmetic of the partial likelihoods. */
enum {
	/* Plain form: FP64 partials with the reference's e^scale_ln rescaling
	 * (calculator/cpu4.rs:403-433). */
	B3G_PRECISION_F64 = 0,
	/* Chosen form: FP32 partials renormalised by an exact power of two at
	 * every node, integer exponents per (node, pattern, category), FP64
	 * log-scale bookkeeping and a compensated FP64 site sum. */
	B3G_PRECISION_F32 = 1
};

typedef struct b3g_config {
	uint32_t num_leaves;     /* L >= 2 */
	uint32_t num_patterns;   /* P >= 1, site patterns after deduplication */
	uint32_t num_states;     /* 4 (DNA) or 20 (protein, <= 8 categories) */
	uint32_t num_categories; /* C in 1..16 rate categories */
	uint32_t precision;      /* B3G_PRECISION_* */
	uint32_t scale_ln;       /* FP64 form: rescale threshold e^-scale_ln;
				    the reference default is 30
				    (calculator/mod.rs:103-110) */
	int32_t device;          /* CUDA device ordinal */
	uint32_t reserved;       /* must be 0 */
} b3g_config;

typedef struct b3g_calculator b3g_calculator;
typedef struct b3g_batch b3g_batch;
typedef struct b3g_handle b3g_handle;

/* Message of the calling thread's last failed call ("" if none). */
B3G_API const char *b3g_last_error(void);
/* Library version string. */
B3G_API const char *b3g_version(void);

/* ---- construction ------------------------------------------------------
 * Replaces CalculatorConfig::make4 (calculator/mod.rs:159-200) and
 * Cpu4Calculator::new / CudaPartialsCalculator::new (cpu4.rs:108-165,
 * cuda_partials/mod.rs:171-284).  `samples` is the leaf-major
 * [num_leaves][num_patterns] array of 4-bit IUPAC codes that `deduplicate`
 * produces (likelihood/mod.rs:74-132); single bases map to states 0..3 and
 * every other code to "unknown" (cpu4.rs:117-124).  With num_states = 20
 * (no reference counterpart) the samples are state indices 0..19 and any
 * other value is unknown.  Partials start zeroed. */
B3G_API b3g_status b3g_calculator_create(const b3g_config *config,
					 const uint8_t *samples,
					 b3g_calculator **out);
B3G_API void b3g_calculator_destroy(b3g_calculator *calc);
B3G_API uint32_t b3g_calculator_num_patterns(const b3g_calculator *calc);

/* ---- calculator level (trait Calculator<f64>) ---------------------------
 * Replaces Calculator::propose (cpu4.rs:39-76, cuda_partials/mod.rs:63-101).
 *   internals[n]          children-first dirty internals, root last
 *   children[n][2]        child node ids of each listed internal
 *   matrices[n][2][C][4][4] transition matrices of the left and right child
 *                         edge per rate category (C = 1: the reference's
 *                         [n*2][4][4] layout)
 *   frequencies[4]        base frequencies (Transitions::frequencies)
 * The launch is asynchronous; results are read by the calls below. */
B3G_API b3g_status b3g_calculator_propose(b3g_calculator *calc,
					  const uint32_t *internals,
					  const uint32_t *children, uint32_t n,
					  const double *matrices,
					  const double *frequencies);
/* Calculator::likelihoods: per-pattern log-likelihoods with the scaling
 * removed, [C][P] (C = 1: [P]).  Blocks until the last proposal is done. */
B3G_API b3g_status b3g_calculator_likelihoods(b3g_calculator *calc,
					      double *out);
/* Calculator::accept / reject (cpu4.rs:78-90, sk/src/editbuf.rs:48-65):
 * selector flips only, no device copies. */
B3G_API b3g_status b3g_calculator_accept(b3g_calculator *calc);
B3G_API b3g_status b3g_calculator_reject(b3g_calculator *calc);

/* ---- likelihood level (DnaLikelihood / GammaLikelihood) -----------------
 * Pattern weights from deduplicate (likelihood/mod.rs:74-132). Default 1. */
B3G_API b3g_status b3g_calculator_set_weights(b3g_calculator *calc,
					      const uint32_t *weights);
/* Substitution model given as an eigensystem, e.g. the analytic HKY one
 * (substitution.rs:336-388): Q = V diag(lambda) V^-1, all row-major.  With
 * `shortcuts` set, d > 20 gives rows equal to the frequencies and d < 1e-10
 * gives I + Q d with a unit diagonal, as HKY/GTR::write_transition do
 * (substitution.rs:403-420, 571-588). */
B3G_API b3g_status b3g_calculator_set_eigen(b3g_calculator *calc,
					    const double *V,
					    const double *Vinv,
					    const double *lambda,
					    const double *Q,
					    const double *frequencies,
					    int shortcuts);
/* Reversible model from symmetric exchangeabilities in upper-triangle
 * row-major order (AC, AG, AT, CG, CT, GT for DNA: GTR::update_matrices,
 * substitution.rs:502-555) and frequencies.  Q is normalised to mean rate 1,
 * decomposed on the host in FP64 (symmetric Jacobi) and uploaded. */
B3G_API b3g_status b3g_calculator_set_reversible(b3g_calculator *calc,
						 const double *rates,
						 const double *frequencies,
						 int shortcuts);
/* Rate multipliers per category, [C] (default all 1). */
B3G_API b3g_status b3g_calculator_set_category_rates(b3g_calculator *calc,
						     const double *rates);
/* Median-discretised Gamma(alpha) rates, normalised to mean 1
 * (update_categories, likelihood/gamma.rs:205-225). */
B3G_API b3g_status b3g_calculator_set_gamma(b3g_calculator *calc,
					    double alpha);
/* Dirty-path evaluation from edge time lengths.  lengths[n][2] are the time
 * lengths (parent height - child height) of the left and right child edge of
 * each listed internal; the transition distance of category c is
 * length * (clock_rate * rate_c), as GammaLikelihood computes it
 * (gamma.rs:126-134).  Asynchronous. */
B3G_API b3g_status b3g_calculator_propose_lengths(b3g_calculator *calc,
						  const uint32_t *internals,
						  const uint32_t *children,
						  uint32_t n,
						  const double *lengths,
						  double clock_rate);
/* Weighted root log-likelihood of the last proposal: sum over patterns of
 * weight * (log-sum-exp over categories + ln(1/C)); for C = 1 this is
 * weighted_sum (likelihood/mod.rs:134-139).  Blocks. */
B3G_API b3g_status b3g_calculator_log_likelihood(b3g_calculator *calc,
						 double *out);
/* Per-pattern mixed log-likelihoods of the last proposal, [P].  Blocks. */
B3G_API b3g_status b3g_calculator_site_log_likelihoods(b3g_calculator *calc,
						       double *out);
/* CUDA events around every evaluation, for the timing calls below (off by
 * default: each costs a few microseconds of host time per evaluation). */
B3G_API b3g_status b3g_calculator_set_timing(b3g_calculator *calc, int on);
/* Device time of the last proposal in milliseconds, from CUDA events on the
 * calculator's stream: the transition-matrix kernel and the pruning kernel
 * (which includes the root reduction).  Needs timing on.  Blocks. */
B3G_API b3g_status b3g_calculator_last_timing(b3g_calculator *calc,
					      float *transition_ms,
					      float *prune_ms);
/* Sums of those device times over every proposal since the last reset, and
 * the number of proposals.  The events live in a ring that is harvested
 * without stalling back-to-back proposals.  Blocks until all are done. */
B3G_API b3g_status b3g_calculator_timing_totals(b3g_calculator *calc,
						int reset,
						double *transition_ms,
						double *prune_ms,
						uint64_t *proposals);
/* Bytes the last proposal copied host -> device (its staged dirty list,
 * schedule runs, frequencies and lengths or matrices). */
B3G_API b3g_status b3g_calculator_last_upload_bytes(b3g_calculator *calc,
						    uint64_t *bytes);
/* Kernels the last evaluation launched on the calculator's stream (one
 * fused launch for a short FP32 list or a run walk that builds its own
 * tables; tables + pruning otherwise; three for 20 states on the tensor
 * cores). */
B3G_API b3g_status b3g_calculator_last_launches(b3g_calculator *calc,
						uint32_t *kernels);
/* Device time between two markers on the calculator's stream: span_begin
 * records the first, span_end records the second, waits and returns the
 * elapsed milliseconds. */
B3G_API b3g_status b3g_calculator_span_begin(b3g_calculator *calc);
B3G_API b3g_status b3g_calculator_span_end(b3g_calculator *calc, float *ms);

/* Autotuner (no counterpart in the reference).  Times a representative list
 * (normally the whole tree) with each launch configuration of this
 * calculator's form and keeps the fastest: patterns per tile of the
 * run-synchronous walk (16, 32, 64 or 128, with 512- or 1,024-thread
 * blocks; a thread owns two pattern columns of one category, so a warp
 * spans four, two, one or one categories; four-state FP32), or tensor
 * cores (one or two thread groups per CTA) against CUDA cores (20-state
 * FP32).
 * Every trial proposal is rejected, so
 * call it between steps; the accepted state is unchanged.  `choice`
 * receives the tile, or 1 (tensor cores) / 0 (CUDA cores); the FP64 form
 * has nothing to tune and returns 0. */
B3G_API b3g_status b3g_calculator_autotune(b3g_calculator *calc,
					   const uint32_t *internals,
					   const uint32_t *children, uint32_t n,
					   const double *lengths,
					   double clock_rate, uint32_t *choice);

/* ---- batched evaluation ----------------------------------------------------
 * Many calculators (chains: replicates or heated copies, each with its own
 * alignment, tree and model) evaluated by one launch.  Members stage their
 * proposals with b3g_calculator_stage_lengths (same arguments as
 * b3g_calculator_propose_lengths, host work only); b3g_batch_run replays one
 * CUDA graph that copies every member's staged block, builds all transition
 * tables with one kernel and prunes every member's pattern tiles with one
 * persistent kernel (tiles handed out by an atomic counter, costliest member
 * first); b3g_batch_log_likelihoods waits and returns one value per member
 * (NaN for members with nothing staged).  Members must use the FP32 chosen
 * form and one device; a calculator belongs to at most one batch; accept and
 * reject stay per member. */
B3G_API b3g_status b3g_batch_create(b3g_calculator *const *members,
				    uint32_t count, b3g_batch **out);
B3G_API void b3g_batch_destroy(b3g_batch *batch);
B3G_API b3g_status b3g_calculator_stage_lengths(b3g_calculator *calc,
						const uint32_t *internals,
						const uint32_t *children,
						uint32_t n,
						const double *lengths,
						double clock_rate);
B3G_API b3g_status b3g_batch_run(b3g_batch *batch);
B3G_API b3g_status b3g_batch_log_likelihoods(b3g_batch *batch, double *out);
/* Device time of the last replay (events inside the graph), ms. */
B3G_API b3g_status b3g_batch_last_ms(b3g_batch *batch, float *ms);

/* Rates of k relaxed-clock categories: quantiles (i + 1/2) / k of a
 * mean-one LogNormal with log-scale sd (clock.rs:66-84). */
B3G_API b3g_status b3g_lognormal_categories(double sd, uint32_t k,
					    double *rates);

/* ---- site-pattern compression on the device ---------------------------------
 * Replaces deduplicate (crates/b3/src/likelihood/mod.rs:74-132) for large
 * alignments: msa is [num_sequences][num_sites] (row per sequence, host
 * memory); the unique columns in first-occurrence order go to
 * leaves[num_sequences][*num_patterns] (capacity num_sequences * num_sites),
 * their site counts to weights (capacity num_sites) and every site's pattern
 * to site_to_pattern[num_sites].  dna_gaps != 0 maps code 0 (gap) to 0b1111
 * as the reference does for DNA; 0 keeps codes (protein state indices).
 * device_ms (may be NULL) receives the device time of the compression.
 * Allocates and frees its own device memory (ingest time, not per step). */
B3G_API b3g_status b3g_deduplicate(const uint8_t *msa, uint32_t num_sequences,
				   uint32_t num_sites, int dna_gaps,
				   int32_t device, uint8_t *leaves,
				   uint32_t *weights, uint32_t *site_to_pattern,
				   uint32_t *num_patterns, float *device_ms);

/* ---- per-pattern class mixture ---------------------------------------------
 * Replaces HeteroLikelihood (crates/b3/src/likelihood/hetero.rs:97-168): K
 * classes, each a calculator over the same patterns with its own substitution
 * model and clock (the caller proposes each member with its own edge lengths
 * and model); pattern p belongs to class c(p) and the log-likelihood is
 * sum_p w_p lnL_{c(p)}(p), weights taken from the first member.  Members
 * must be evaluated and accepted before the mixture is built.  Per step:
 * propose the members whose tree, model or clock changed and/or
 * b3g_hetero_set_classes, then b3g_hetero_log_likelihood, then exactly one
 * of b3g_hetero_accept / _reject (which accept or reject the evaluated
 * members too).  A member not evaluated in the step contributes its accepted
 * per-pattern values, so a step that changes only the classes prunes
 * nothing.  At most 16 classes. */
typedef struct b3g_hetero b3g_hetero;
B3G_API b3g_status b3g_hetero_create(b3g_calculator *const *members,
				     uint32_t count, b3g_hetero **out);
B3G_API void b3g_hetero_destroy(b3g_hetero *h);
/* classes[num_patterns], each < count. */
B3G_API b3g_status b3g_hetero_set_classes(b3g_hetero *h,
					  const uint32_t *classes);
B3G_API b3g_status b3g_hetero_log_likelihood(b3g_hetero *h, double *out);
B3G_API b3g_status b3g_hetero_accept(b3g_hetero *h);
B3G_API b3g_status b3g_hetero_reject(b3g_hetero *h);

/* ---- native MCMC driver ---------------------------------------------------
 * The caller side of the path: b3's MCMC step (crates/b3/src/mcmc.rs:
 * 314-393) in C++ -- operator proposal, prior (reject at -inf before any
 * likelihood work), device likelihood, Metropolis-Hastings, accept/reject
 * of tree, parameters and calculator -- with the operators of
 * python/aspartik/b3/operators (TreeScale, SubtreeSlide, BeastNarrowExchange,
 * BeastWideExchange, NodeSlide, RootSlide, UpDown, ScaleReal, DeltaExchange;
 * SubtreeSlide's downward Hastings term is +log of the destination count,
 * where the reference's Python operator has -log, and its slide size is
 * tuned toward 0.234 acceptance, growing when accepted more often, where
 * the reference's tuning rule drives it the other way) and the priors of the reference's config
 * recipe (Yule, LogNormal, SymmetricDirichlet).  Several chains run at once
 * (replicates, or Metropolis-coupled temperatures beta_i = 1/(1 + heat*i));
 * every chain's device work of a step is queued before any result is read.
 * The model is HKY (kappa + frequencies) or GTR (6 exchangeabilities +
 * frequencies), optionally with Gamma rate categories (shape alpha). */
typedef struct b3g_mcmc b3g_mcmc;

enum { B3G_MODEL_HKY = 0, B3G_MODEL_GTR = 1 };

enum {
	B3G_OP_TREE_SCALE = 0,
	B3G_OP_SUBTREE_SLIDE = 1,
	B3G_OP_NARROW_EXCHANGE = 2,
	B3G_OP_SCALE_KAPPA = 3,
	B3G_OP_SCALE_ALPHA = 4,
	B3G_OP_SCALE_BIRTH_RATE = 5,
	B3G_OP_DELTA_RATES = 6,
	B3G_OP_DELTA_FREQUENCIES = 7,
	B3G_OP_RELAXED_CATEGORY = 8, /* one edge's relaxed-clock rate category */
	B3G_OP_SCALE_CLOCK_SD = 9,   /* the relaxed clock's LogNormal sd */
	B3G_OP_NODE_SLIDE = 10,      /* NodeSlide (operators/_node_slide.py) */
	B3G_OP_ROOT_SLIDE = 11,      /* RootSlide (operators/_root.py) */
	B3G_OP_UP_DOWN = 12,         /* UpDown(tree, birth rate), _updown.py */
	B3G_OP_WIDE_EXCHANGE = 13,   /* BeastWideExchange, _tree_exchange.py */
	B3G_OP_COUNT = 14
};

/* Trace fields of the cold chain, sampled every sample_every steps. */
enum {
	B3G_TRACE_LNL = 0,
	B3G_TRACE_PRIOR = 1,
	B3G_TRACE_POSTERIOR = 2,
	B3G_TRACE_ROOT_HEIGHT = 3,
	B3G_TRACE_KAPPA_OR_RATE0 = 4,
	B3G_TRACE_ALPHA = 5,
	B3G_TRACE_TREE_LENGTH = 6,
	B3G_TRACE_CLOCK_SD = 7
};

typedef struct b3g_mcmc_config {
	uint32_t num_chains;     /* 1..256 */
	uint32_t num_categories; /* 1 = no Gamma */
	uint32_t precision;      /* B3G_PRECISION_* */
	uint32_t model;          /* B3G_MODEL_* */
	uint64_t seed;
	double heat;             /* 0 = independent replicates */
	uint32_t swap_every;     /* steps between swap attempts, 0 = never */
	uint32_t sample_every;   /* steps between trace samples, 0 = never */
	uint32_t tune_every;     /* steps between operator tunings, 0 = never */
	int32_t device;
	double op_weights[B3G_OP_COUNT];
	/* Delayed acceptance (no counterpart in the reference): after
	 * da_pilot_steps exact steps a surrogate (14 inputs: log tree length,
	 * root height, internal and external edge-length sums and alpha, and
	 * 9 model parameters; da_hidden units per hidden layer) is trained for
	 * da_epochs on the pilot's pairs of the moves that re-evaluate the
	 * whole tree (tree scale, up-down, kappa, alpha, exchangeabilities,
	 * frequencies) and screens those moves afterwards; the exact
	 * likelihood stays the second-stage test, so the target distribution
	 * is unchanged.  Screening stops for good when the RMS of
	 * (exact - surrogate) over the last 200 screened proposals exceeds
	 * da_drift_limit (0: never).  da_pilot_steps = 0 turns it off. */
	uint32_t da_pilot_steps;
	uint32_t da_epochs;
	uint32_t da_hidden;
	uint32_t da_reserved; /* must be 0 */
	double da_drift_limit;
	/* Relaxed clock (RelaxedClock, crates/b3/src/clock.rs:41-134): 0 =
	 * strict clock; k > 0 = every edge has one of k rate categories whose
	 * rates are the median quantiles of a mean-one LogNormal with
	 * log-scale sd (prior Exponential, mean 1/3).  A category change
	 * marks only its edge for recomputation, an sd change every edge. */
	uint32_t clock_categories;
	/* B3G_MCMC_LAUNCH_STREAMS (0): each chain launches its own evaluations
	 * on its own stream and a step's launches run concurrently;
	 * B3G_MCMC_LAUNCH_BATCH (1, FP32 chosen form, several chains): every
	 * chain's evaluation of a step in one replay of a captured CUDA graph
	 * (b3g_batch_*: one staging copy, one persistent launch for the
	 * members' short lists, one for the long ones, one read-back);
	 * B3G_MCMC_LAUNCH_INDEPENDENT (2): as streams, but each host thread
	 * advances its chains on their own between the driver's
	 * synchronisation points (MC3 swap attempts, operator tuning, the end
	 * of the delayed-acceptance pilot, the end of b3g_mcmc_run), so no
	 * chain waits for another's evaluation in between; the
	 * chains' statistics are merged at those points, each chain keeps its
	 * own delayed-acceptance drift window, and the results depend neither
	 * on the thread count nor on how the steps are split into runs (they
	 * differ from the other modes' in the statistics and drift decisions
	 * only). */
	uint32_t launch;
	/* Host threads that step the chains, chain i on thread i % threads
	 * (independent stepping: automatically one per chain, at most 8):
	 * each proposes and launches its chains' evaluations, then reads
	 * their results; statistics are gathered in chain order, so the
	 * results are the same for every value.  0 = one for every four
	 * chains, at most 8 and at most the hardware threads (the calling
	 * thread alone in the batched launch mode, whose per-chain host work
	 * is a few copies); 1 = the calling thread alone (the environment
	 * variable B3G_MCMC_THREADS overrides it). */
	uint32_t host_threads;
} b3g_mcmc_config;

enum {
	B3G_MCMC_LAUNCH_STREAMS = 0,
	B3G_MCMC_LAUNCH_BATCH = 1,
	B3G_MCMC_LAUNCH_INDEPENDENT = 2
};

/* One alignment of a driver over several (b3g_mcmc_create_multi). */
typedef struct b3g_mcmc_problem {
	uint32_t num_leaves;
	uint32_t num_patterns;
	const uint8_t *samples;  /* [num_leaves][num_patterns] */
	const uint32_t *weights; /* [num_patterns] */
	const uint32_t *parents; /* [2 num_leaves - 1], root 0xFFFFFFFF */
	const double *heights;   /* [2 num_leaves - 1] */
} b3g_mcmc_problem;

/* parents[2L-1] (root: 0xFFFFFFFF) and heights[2L-1] give the start tree of
 * every chain; samples/weights as for b3g_calculator_create/_set_weights. */
B3G_API b3g_status b3g_mcmc_create(const b3g_mcmc_config *config,
				   uint32_t num_leaves, uint32_t num_patterns,
				   const uint8_t *samples,
				   const uint32_t *weights,
				   const uint32_t *parents,
				   const double *heights, b3g_mcmc **out);
/* Chains over several alignments (no counterpart in the reference, whose
 * Mcmc holds one likelihood): num_chains / num_problems chains per problem;
 * chain i runs problem i / that count at temperature index i % that count,
 * beta = 1 / (1 + heat * index), and MC3 swaps pair chains of one problem
 * only.  Delayed acceptance needs a single problem; traces and samples of
 * the cold chain are problem 0's, b3g_mcmc_chain_trace gives every chain. */
B3G_API b3g_status b3g_mcmc_create_multi(const b3g_mcmc_config *config,
					 uint32_t num_problems,
					 const b3g_mcmc_problem *problems,
					 b3g_mcmc **out);
/* Launch mode in use (1: batched graph) and, when batched, the device time
 * of all replays so far (ms) and their count. */
B3G_API b3g_status b3g_mcmc_launch_stats(b3g_mcmc *mcmc, uint32_t *batched,
					 double *device_ms, uint64_t *launches);
B3G_API void b3g_mcmc_destroy(b3g_mcmc *mcmc);
/* Start values (rates/frequencies may be NULL to keep the defaults). */
B3G_API b3g_status b3g_mcmc_set_parameters(b3g_mcmc *mcmc, double kappa,
					   const double *rates,
					   const double *frequencies,
					   double alpha, double birth_rate);
/* Relaxed clock start state (before b3g_mcmc_set_parameters): sd > 0 and
 * the category of every edge, categories[2L-1] indexed by the edge's child
 * node (the root's entry is ignored), or NULL for node % k. */
B3G_API b3g_status b3g_mcmc_set_clock(b3g_mcmc *mcmc, double sd,
				      const uint32_t *categories);
B3G_API b3g_status b3g_mcmc_run(b3g_mcmc *mcmc, uint64_t steps);
/* Whole samples of the cold chain (for trace files), up to `capacity`;
 * *count = all.  steps[n]; parents[n][2L-1] (root: 0xFFFFFFFF) and
 * heights[n][2L-1]; parameters[n][14] = kappa, alpha, birth rate, 6
 * exchangeabilities, 4 frequencies, relaxed-clock sd (0 if strict).  Any
 * output may be NULL. */
B3G_API b3g_status b3g_mcmc_samples(b3g_mcmc *mcmc, uint64_t *steps,
				    uint32_t *parents, double *heights,
				    double *parameters, uint64_t capacity,
				    uint64_t *count);
/* Copies up to `capacity` samples of a B3G_TRACE_* field; *count = all. */
B3G_API b3g_status b3g_mcmc_trace(b3g_mcmc *mcmc, uint32_t field,
				  double *out, uint64_t capacity,
				  uint64_t *count);
/* The same for one chain (0 .. num_chains - 1) in chain order, e.g. for
 * the summed ESS of independent replicates; with MC3 swaps a chain's trace
 * follows its state through the temperatures. */
B3G_API b3g_status b3g_mcmc_chain_trace(b3g_mcmc *mcmc, uint32_t chain,
					uint32_t field, double *out,
					uint64_t capacity, uint64_t *count);
/* counts = {accepts, rejects, aborts, prior rejects} of one operator. */
B3G_API b3g_status b3g_mcmc_operator_stats(b3g_mcmc *mcmc, uint32_t op,
					   uint64_t *counts, double *tuning);
/* Sets one operator's tuning parameter, e.g. to the values a burn-in run
 * reached (operators' set_tuning, python/aspartik/b3/__init__.py:109-119):
 * 0.01..0.99 for the scale and delta operators, 1e-6..10 for SubtreeSlide
 * (its slide size). */
B3G_API b3g_status b3g_mcmc_set_tuning(b3g_mcmc *mcmc, uint32_t op,
				       double tuning);
B3G_API b3g_status b3g_mcmc_swaps(b3g_mcmc *mcmc, uint64_t *tried,
				  uint64_t *accepted);
/* counts = {pilot pairs, stage-1 rejects, stage-2 accepts, stage-2 rejects,
 * exact evaluations, fallback (1 if screening stopped)};
 * values = {final training loss, last drift RMS}. */
B3G_API b3g_status b3g_mcmc_da_stats(b3g_mcmc *mcmc, uint64_t *counts,
				     double *values);
/* Checkpoint between runs (Mcmc::dump, mcmc.rs:251-268, in this driver's
 * own layout): the chains' trees, parameters, relaxed-clock categories,
 * cached likelihoods and priors, temperatures, RNG states and run-walk
 * launch shapes, the step counter, swap counters and RNG, the operators'
 * statistics and tuning.  b3g_mcmc_dump sets *size to the checkpoint's
 * bytes and writes it to out when out is not null (capacity >= *size).
 * b3g_mcmc_load takes a checkpoint into a driver created with the same
 * configuration and data (and its parameters set): every chain is evaluated
 * from scratch and checked against the saved likelihood, traces and samples
 * start empty, and later runs continue exactly as the dumped driver's
 * would.  Not for delayed-acceptance runs (B3G_ERR_STATE). */
B3G_API b3g_status b3g_mcmc_dump(b3g_mcmc *mcmc, uint8_t *out,
				 uint64_t capacity, uint64_t *size);
B3G_API b3g_status b3g_mcmc_load(b3g_mcmc *mcmc, const uint8_t *state,
				 uint64_t size);

/* State files in the reference's own layout (Mcmc::dump_state /
 * load_state, crates/b3/src/mcmc.rs:175-219, 251-268, written through
 * crates/verbatim: little-endian values padded to their size, slices with a
 * u32 length): tag 62 33 b3 44, u32 version 19, u64 step, f64 posterior,
 * the parameters in the reference Mcmc's order, each operator's u32
 * accepts and rejects since its last tuning and its f64 tuning if it has
 * one, the RNG as two u128 values.  The caller gives the reference
 * configuration's parameter order (B3G_STATE_*) and operator order (this
 * driver's B3G_OP_* kind of each, and whether it is tuned).  One chain's
 * parameters; the step and the operators' statistics and tunings are the
 * driver's.  The RNG section carries this driver's xoshiro256** words on
 * dump and reseeds the chain's generator on load (the reference's PCG64
 * stream is not reproduced); b3g_mcmc_dump is the exact checkpoint.  Load
 * re-evaluates the chain (likelihood and priors) and accepts, as
 * load_state does; a state of another version, tag, tree size or with
 * bytes left after its RNG is refused with nothing changed. */
enum {
	B3G_STATE_TREE = 0,             /* u32 parents slice, f64 heights slice */
	B3G_STATE_BIRTH_RATE = 1,       /* f64 */
	B3G_STATE_KAPPA = 2,            /* f64 (HKY) */
	B3G_STATE_ALPHA = 3,            /* f64 (Gamma categories) */
	B3G_STATE_RATES = 4,            /* 6 f64 (GTR) */
	B3G_STATE_FREQUENCIES = 5,      /* 4 f64 */
	B3G_STATE_CLOCK_SD = 6,         /* f64 (relaxed clock) */
	B3G_STATE_CLOCK_CATEGORIES = 7  /* u32 per node (relaxed clock) */
};
typedef struct b3g_state_operator {
	uint32_t op;         /* B3G_OP_* */
	uint32_t has_tuning; /* 0 or 1 */
} b3g_state_operator;
B3G_API b3g_status b3g_mcmc_dump_verbatim(b3g_mcmc *mcmc, uint32_t chain,
					  const uint32_t *params,
					  uint32_t num_params,
					  const b3g_state_operator *ops,
					  uint32_t num_ops, uint8_t *out,
					  uint64_t capacity, uint64_t *size);
B3G_API b3g_status b3g_mcmc_load_verbatim(b3g_mcmc *mcmc, uint32_t chain,
					  const uint32_t *params,
					  uint32_t num_params,
					  const b3g_state_operator *ops,
					  uint32_t num_ops, const uint8_t *state,
					  uint64_t size);
/* Re-evaluates every chain from scratch and returns the largest relative
 * difference to its incrementally maintained log-likelihood. */
B3G_API b3g_status b3g_mcmc_check(b3g_mcmc *mcmc, double *max_rel_diff);
B3G_API b3g_status b3g_mcmc_chain_state(b3g_mcmc *mcmc, uint32_t chain,
					uint32_t *parents, double *heights,
					double *lnl, double *beta);

/* ---- delayed-acceptance surrogate ------------------------------------------
 * No counterpart in the reference.  A fully connected network
 * inputs -> hidden -> hidden -> hidden -> 1 with GELU, FP32, trained and
 * evaluated by this library's own CUDA kernels.  Parameters are flat: layer
 * by layer, W [out][in] row-major then b [out].  The training objective is
 * mean_n (f(x_new,n) - f(x_old,n) - delta_n)^2 (Adam). */
typedef struct b3g_surrogate b3g_surrogate;
B3G_API b3g_status b3g_surrogate_create(uint32_t inputs, uint32_t hidden,
					uint64_t seed, int32_t device,
					b3g_surrogate **out);
B3G_API void b3g_surrogate_destroy(b3g_surrogate *s);
B3G_API uint32_t b3g_surrogate_num_params(const b3g_surrogate *s);
B3G_API b3g_status b3g_surrogate_get_params(b3g_surrogate *s, float *out);
B3G_API b3g_status b3g_surrogate_set_params(b3g_surrogate *s,
					    const float *in);
/* f(x) for n rows x[n][inputs]. */
B3G_API b3g_status b3g_surrogate_forward(b3g_surrogate *s, const float *x,
					 uint32_t n, float *out);
/* Loss of the pair objective and its gradient (flat, parameter order). */
B3G_API b3g_status b3g_surrogate_loss_grad(b3g_surrogate *s,
					   const float *x_new,
					   const float *x_old,
					   const float *delta, uint32_t n,
					   float *loss, float *grad);
B3G_API b3g_status b3g_surrogate_train(b3g_surrogate *s, const float *x_new,
				       const float *x_old, const float *delta,
				       uint32_t n, uint32_t epochs,
				       uint32_t batch, float lr, uint64_t seed,
				       float *final_loss);
/* f(x_new) - f(x_old) for one pair (one fused launch: a cluster of 8
 * blocks holds the hidden layers in distributed shared memory). */
B3G_API b3g_status b3g_surrogate_delta(b3g_surrogate *s, const float *x_new,
				       const float *x_old, float *out);
/* The same for n pairs (1..256) in one launch, a cluster per pair; x_new
 * and x_old [n][inputs], out[n].  The MCMC driver screens every chain's
 * proposal of a step with one call. */
B3G_API b3g_status b3g_surrogate_deltas(b3g_surrogate *s, const float *x_new,
					const float *x_old, uint32_t n,
					float *out);

/* ---- allocation-free pruning --------------------------------------------
 * This entry point has no counterpart in the reference.
 *
 * It is for callers that must not have this library allocate device memory:
 * a host program whose every device buffer comes from its own allocator or
 * pool (for example a Rust CUDA wrapper that owns the calculator's buffers,
 * as the reference's CUDA calculators own theirs), or code that runs where a
 * cudaMalloc/cudaFree is not allowed or would stall the whole device, such
 * as a loop that is being recorded into a CUDA graph or a latency-critical
 * MCMC step.  The caller passes every input and output as device memory in
 * the layouts below; the only working memory of the call, one double per
 * thread block plus a completion counter, is a fixed array compiled into
 * the library (B3G_NOALLOC_MAX_BLOCKS blocks, 128 KiB + 256 bytes), which
 * every GPU that loads the library holds until the process exits.
 *
 * Limits and rules:
 *  - At most B3G_NOALLOC_MAX_BLOCKS blocks: ldp / tile with tile = 128
 *    patterns for 1 category, 64 for 2, 32 for more (so up to 2,097,152
 *    padded patterns for 1 category, 524,288 for 4).  Larger problems are
 *    rejected with B3G_ERR_INVALID_ARGUMENT.
 *  - Runs on the calling thread's current device; `stream` (a cudaStream_t,
 *    or NULL for the default stream) must belong to it.  The call is
 *    asynchronous.
 *  - The first call on a device looks up the array's device address (once
 *    per device); make that first call before any stream capture begins.
 *  - All calls in the process share the one array per device, and each call
 *    clears its counter first: calls that can overlap on the GPU (different
 *    streams without ordering between them) race and must not be issued.
 *  - The device data is trusted: the caller guarantees that every slot,
 *    leaf and tip code in `ops` and `tips` lies inside the buffers.
 *
 * Layouts (ldp = padded pattern count, a multiple of 128; C categories;
 * R = double for B3G_PRECISION_F64, float for B3G_PRECISION_F32):
 *   tips        u8  [L][ldp]   states 0..3, 4 = unknown (padding: 4)
 *   partials    R   [slots][C][ldp][4]
 *   scales      i32 [slots][C][ldp]
 *   ops         b3g_node_op [n], children-first, root last
 *   tables      R   [n][2][C][5][4]: for entry i, side s (0 left, 1 right),
 *               category c: element [k][j] = P(t)[j][k] for k < 4 and 1 for
 *               k = 4 (P(t) transposed, then a row of ones)
 *   frequencies f64 [4]
 *   weights     u32 [ldp] (0 on padding)
 *   site_lnl    f64 [ldp] out: per-pattern mixed log-likelihood
 *   lnl         f64 [1]   out: weighted sum over patterns
 */
#define B3G_NOALLOC_MAX_BLOCKS 16384u
#define B3G_TIP 0x80000000u /* b3g_node_op child: B3G_TIP | leaf id */

typedef struct b3g_node_op {
	uint32_t out;   /* output slot */
	uint32_t left;  /* child slot, or B3G_TIP | leaf id */
	uint32_t right; /* child slot, or B3G_TIP | leaf id */
	uint32_t run;   /* entries from this one on that are mutually
			   independent (1 is always valid) */
} b3g_node_op;

typedef struct b3g_prune_buffers {
	const uint8_t *tips;
	void *partials;
	int32_t *scales;
	const b3g_node_op *ops;
	const void *tables;
	const double *frequencies;
	const uint32_t *weights;
	double *site_lnl;
	double *lnl;
	uint32_t n;              /* entries in ops, >= 1 */
	uint32_t ldp;            /* padded patterns, multiple of 128 */
	uint32_t num_categories; /* 1..16 */
	uint32_t precision;      /* B3G_PRECISION_* */
	uint32_t scale_ln;       /* FP64 form rescale exponent */
	uint32_t reserved;       /* must be 0 */
} b3g_prune_buffers;

B3G_API b3g_status b3g_prune_noalloc(const b3g_prune_buffers *buffers,
				     void *stream);

/* ---- tree-level handle -------------------------------------------------
 * The call sequence b3's MCMC makes around its likelihood
 * (likelihood/dna.rs:68-124, likelihood/gamma.rs:97-169) with the tree
 * mirrored inside the library, for 1..64 chains over one alignment: load the
 * tree (parents[2L-1], root 0xFFFFFFFF, and heights[2L-1], as
 * tree.rs:906-930), mark the edges a move changed (edge id = child node
 * id, tree.rs:357-386), propose a set of chains (asynchronous; each chain
 * has its own calculator and stream, so the chains run concurrently), read
 * the log-likelihoods, then accept or reject each proposed chain.  The dirty
 * list is built from the mirrored tree as partials_lists builds it
 * (tree.rs:398-461).  A reject returns the chain's tree to its last
 * accepted state (the first tree loaded counts as accepted).  One host
 * thread per handle. */
B3G_API b3g_status b3g_create(const b3g_config *config, const uint8_t *tips,
			      const uint32_t *weights, uint32_t num_chains,
			      b3g_handle **out);
B3G_API void b3g_destroy(b3g_handle *h);
/* V, Vinv row-major S x S, lambda[S], pi[S], cat_rates[C] (mean one);
 * S and C must match the handle's configuration. */
B3G_API b3g_status b3g_set_model(b3g_handle *h, uint32_t chain, uint32_t S,
				 const double *V, const double *Vinv,
				 const double *lambda, const double *pi,
				 const double *cat_rates, uint32_t C);
B3G_API b3g_status b3g_set_tree(b3g_handle *h, uint32_t chain,
				const uint32_t *parents, const double *heights,
				double clock_rate);
B3G_API b3g_status b3g_mark_edges(b3g_handle *h, uint32_t chain,
				  const uint32_t *edges, uint32_t n);
B3G_API b3g_status b3g_mark_all(b3g_handle *h, uint32_t chain);
/* bit c of chains_mask: evaluate chain c */
B3G_API b3g_status b3g_propose(b3g_handle *h, uint64_t chains_mask);
B3G_API b3g_status b3g_wait(b3g_handle *h);
B3G_API b3g_status b3g_lnl(b3g_handle *h, uint32_t chain, double *out);
/* per-pattern lnL (categories mixed, scaling removed), [num_patterns] */
B3G_API b3g_status b3g_site_lnl(b3g_handle *h, uint32_t chain, double *out);
B3G_API b3g_status b3g_accept(b3g_handle *h, uint32_t chain);
B3G_API b3g_status b3g_reject(b3g_handle *h, uint32_t chain);

#ifdef __cplusplus
}
#endif

#endif
