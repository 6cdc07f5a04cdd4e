// calculator.hpp -- host side of one device-resident pruning store.
//
// Mirrors the reference's calculator life cycle (crates/b3/src/calculator/
// mod.rs:33-76): propose -> likelihoods -> accept | reject.  The host keeps
// only the EditBuf selectors (sk/src/editbuf.rs:8-105) and the staging
// buffers; partials, scale counts, tips, weights, the model and every
// per-step table live in HBM.  Accept and reject are selector flips: the
// cumulative scale counts are per slot, so nothing is copied on the device.
#pragma once

#include "../../include/b3g.h"
#include "b3g_device.cuh"

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

namespace b3g {

struct Error : std::runtime_error {
	b3g_status status;
	Error(b3g_status s, const std::string &m)
	    : std::runtime_error(m), status(s)
	{
	}
};

void check_cuda(cudaError_t e, const char *what);

class Calculator {
      public:
	Calculator(const b3g_config &cfg, const uint8_t *samples);
	~Calculator();
	Calculator(const Calculator &) = delete;
	Calculator &operator=(const Calculator &) = delete;

	uint32_t num_patterns() const { return P_; }
	uint32_t num_leaves() const { return L_; }
	uint32_t num_categories() const { return C_; }
	int device() const { return device_; }

	// calculator level
	void propose_matrices(const uint32_t *internals,
			      const uint32_t *children, uint32_t n,
			      const double *matrices, const double *freqs);
	void likelihoods(double *out);
	void accept();
	void reject();

	// likelihood level
	void set_weights(const uint32_t *w);
	void set_eigen(const double *V, const double *Vinv,
		       const double *lambda, const double *Q,
		       const double *pi, int shortcuts);
	void set_reversible(const double *rates, const double *pi,
			    int shortcuts);
	void set_category_rates(const double *rates);
	void set_gamma(double alpha);
	void propose_lengths(const uint32_t *internals,
			     const uint32_t *children, uint32_t n,
			     const double *lengths, double clock_rate);
	double log_likelihood();
	void site_log_likelihoods(double *out);
	void last_timing(float *transition_ms, float *prune_ms);
	void timing_totals(bool reset, double *transition_ms, double *prune_ms,
			   uint64_t *proposals);
	void span_begin();
	float span_end();
	uint64_t last_upload_bytes() const { return last_upload_bytes_; }
	uint32_t last_launches() const { return last_launches_; }
	// launch shape of the run walk (patterns per tile, threads per block),
	// as the autotuner leaves it; a checkpoint restores it so that whole-
	// tree sums keep their order
	uint32_t runs_tile() const { return runs_tile_; }
	uint32_t runs_block() const { return runs_block_; }
	void set_runs_shape(uint32_t tile, uint32_t block)
	{
		if ((tile != 16 && tile != 32 && tile != 64 && tile != 128) ||
		    (block != 512 && block != 1024) || tile * C_ > 512 ||
		    (block == 1024 && tile * C_ >= 512))
			throw Error(B3G_ERR_INVALID_ARGUMENT, "no such run-walk shape");
		runs_tile_ = tile;
		runs_block_ = block;
	}
	uint32_t autotune(const uint32_t *internals, const uint32_t *children,
			  uint32_t n, const double *lengths, double clock_rate);

	// Batched evaluation: validate and stage a dirty-path evaluation
	// without launching; a Batch evaluates all staged members at once.
	void stage_lengths(const uint32_t *internals, const uint32_t *children,
			   uint32_t n, const double *lengths, double clock_rate);
	friend class Batch;
	friend class Hetero;

      private:
	void validate_lists(const uint32_t *internals,
			    const uint32_t *children, uint32_t n);
	void stage_ops(const uint32_t *internals, const uint32_t *children,
		       uint32_t n);
	void launch(uint32_t n, bool matrices_mode, double clock_rate,
		    bool want_cat);
	void launch_direct(uint32_t n, double clock_rate);
	void wait_stage();
	bool upload_pending_ = false; // an upload from h_stage_ may be in flight
	// The fused short-list kernel and the run walk write their results
	// into mapped host memory (the blocks' sums, h_bsums_ below; without
	// it the word h_lnl_).  Before such a launch with no earlier
	// evaluation in flight, the host stores sentinels there and
	// log_likelihood polls for the result instead of synchronising the
	// stream; otherwise (or on any other path) it synchronises.
	uint32_t in_flight_ = 0; // evaluations launched since the last wait
	bool poll_result_ = false;
	void arm_poll();
	bool wait_mapped(double &value);
	// FP32 four-state walks (run walk, fused short list): every block writes
	// its sum into the mapped array h_bsums_ and the host folds them in the
	// device fold's order, so no block waits for a ticket and no last block
	// folds.  host_fold_blocks_: the last launch's block count (0: its
	// result is a single word).
	double *h_bsums_ = nullptr, *d_bsums_ = nullptr;
	uint32_t host_fold_blocks_ = 0;
	void arm_host_fold(uint32_t blocks);
	bool wait_host_sums();
	double fold_host_sums() const;
	struct TimingSlot;
	void launch20(uint32_t n, bool matrices_mode, double clock_rate,
		      bool want_cat, TimingSlot &slot);
	void upload_model();
	void release();

	// shape
	uint32_t L_ = 0, I_ = 0, P_ = 0, ldp_ = 0, S_ = 0, C_ = 0, tile_ = 0;
	bool f32_ = false;
	uint32_t scale_ln_ = 0;
	int device_ = -1;

	// host state
	std::vector<uint8_t> selectors_; // EditBuf over internals
	std::vector<uint32_t> stamp_;    // per-node epoch stamps
	std::vector<uint32_t> pos_;      // list position of each listed node
	std::vector<uint32_t> run_of_;   // start of the run of each entry
	// run walk: shared-memory slot of each listed output, indexed by the
	// output's partial slot (kNoSlot outside assign_slots), and the pools
	std::vector<uint8_t> smem_of_;
	std::vector<uint8_t> free_slots_, pending_slots_;
	// dynamic shared memory a run-walk block may take: the SM's, halved
	// for 512-thread blocks (two per SM), less the reserved share
	uint32_t smem_per_sm_ = 0, smem_reserved_ = 0;
	uint32_t smem_budget(uint32_t block) const
	{
		const int64_t b = (int64_t)smem_per_sm_ / (1024 / block) -
				  (int64_t)smem_reserved_ - 256;
		return b > 0 ? (uint32_t)b : 0u;
	}
	// threads per block of the run walk (512 or 1024, autotuned)
	uint32_t runs_block_ = 512;
	bool use_slots_ = true;
	bool use_inline_ = true;
	size_t off_slots_ = 0;
	uint32_t assign_slots(uint32_t n, uint32_t capacity);
	uint32_t stamp_epoch_ = 0;
	uint32_t tip_children_ = 0;      // tip children in the staged list
	bool model_set_ = false;
	bool have_result_ = false;
	bool outstanding_ = false; // evaluated since the last accept/reject
	bool cat_valid_ = false;
	ModelDev model_host_{};

	// stream and events
	cudaStream_t stream_ = nullptr;
	cudaEvent_t ev_stage_free_ = nullptr, ev_model_free_ = nullptr;
	cudaEvent_t ev_span0_ = nullptr, ev_span1_ = nullptr;
	// per-proposal timing ring: events before the transition kernel,
	// between the kernels and after the pruning kernel
	static constexpr uint32_t kRing = 64;
	struct TimingSlot {
		cudaEvent_t k0 = nullptr, kmid = nullptr, k1 = nullptr;
		bool pending = false;
		bool direct = false; // fused launch: k0 .. k1, no kmid
	};
	TimingSlot ring_[kRing];
	uint64_t ring_next_ = 0;
	double acc_transition_ms_ = 0.0, acc_prune_ms_ = 0.0;
	uint64_t acc_count_ = 0;
	void harvest(TimingSlot &s);
	void record(cudaEvent_t e); // a timing event, when timing is on
	bool timing_ = false; // CUDA events around every evaluation (off: none)

      public:
	// Per-proposal device timing (events around the kernels).  On by
	// default; a driver that never reads it turns it off to save the
	// event calls on every launch.
	void set_timing(bool on) { timing_ = on; }

      private:

	// device buffers
	uint8_t *d_tips_ = nullptr;
	void *d_partials_ = nullptr;
	int32_t *d_scales_ = nullptr;
	uint32_t *d_weights_ = nullptr;
	double *d_site_ = nullptr;
	double *d_cat_ = nullptr;
	double *d_block_sums_ = nullptr;
	unsigned *d_ticket_ = nullptr;
	double *d_lnl_ = nullptr;
	ModelDev *d_model_ = nullptr;
	void *d_ptab_ = nullptr;
	unsigned char *d_stage_ = nullptr;

	// pinned host staging
	unsigned char *h_stage_ = nullptr;
	// a batch lends h_stage_ / d_stage_ a slice of its one contiguous
	// staging block (lengths-mode proposals only while it does); the
	// calculator's own buffers wait here and come back when it ends
	unsigned char *own_h_stage_ = nullptr, *own_d_stage_ = nullptr;
	ModelDev *h_model_ = nullptr;
	double *h_lnl_ = nullptr;
	double *d_lnl_host_ = nullptr; // device view of h_lnl_
	size_t stage_bytes_ = 0;
	size_t off_pi_ = 0, off_runs_ = 0, off_in_ = 0;
	uint32_t n_runs_ = 0;
	uint32_t max_run_ = 0; // entries of the widest run
	uint64_t last_upload_bytes_ = 0;
	uint32_t last_launches_ = 0; // kernels the last evaluation launched
	// batch membership: staged proposal and the event after which the
	// batch no longer reads this calculator's staging buffer
	bool in_batch_ = false;
	bool staged_ = false;
	uint32_t staged_n_ = 0;
	uint32_t staged_tips_smem_ = 0;
	uint32_t staged_tile_ = 64;
	// patterns per tile of the run-synchronous walk for the staged list:
	// path-like lists (runs of one entry) take 128 so that one entry fills
	// a 512-thread block
	uint32_t pick_tile(uint32_t n) const
	{
		const bool narrow_runs = 2 * n_runs_ > n;
		return (narrow_runs && 128 * C_ <= 512) ? 128u : runs_tile_;
	}
	double staged_clock_ = 1.0;
	cudaEvent_t batch_done_ = nullptr;
	// work was queued on this calculator's own stream since a batch last
	// synchronised with it (model uploads, eigen kernel, own proposals)
	bool stream_dirty_ = false;
	uint32_t num_sms_ = 1;
	uint32_t block_sums_cap_ = 0; // d_block_sums_ entries
	uint32_t runs_tile_ = 64;
	bool use_runs_ = false;
	bool use_direct_ = false;
	bool use_tc20_ = false;
	uint32_t tc20_groups_ = 0; // 0: per launch from the grid size
	bool tc20_groups_fixed_ = false; // set by B3G_TC20_GROUPS
	uint32_t tc20_cluster_ = 1;      // CTAs per work item when fixed
	bool tc20_cluster_fixed_ = false; // set by B3G_TC20_CLUSTER
	float *d_tc_tab_ = nullptr;     // 20-state MMA operand blocks
	double *d_root_val_ = nullptr;  // [C][ldp] root pi . x per category
	int32_t *d_root_exp_ = nullptr; // [C][ldp] its exponent
	unsigned *d_status_ = nullptr;  // bounded tensor-core waits
	unsigned *h_status_ = nullptr;
};

} // namespace b3g
