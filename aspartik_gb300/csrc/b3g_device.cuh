// b3g_device.cuh -- device-side layouts shared by the b3g kernels and the
// host orchestration.
//
// Device store of one calculator (one chain), all resident in HBM:
//   tips      u8  [L][ldp]                   state 0..S-1, S = unknown
//   partials  R   [2I][C][ldp][S]            slot = (v - L) * 2 + selector
//   scales    i32 [2I][C][ldp]               cumulative rescale count of the
//                                            subtree below the slot's node
//   ptab      R   [n][2][C][S+1][S]          per-step transposed transition
//                                            tables, row S = all ones
// ldp is the pattern count rounded up to a multiple of 128; padded patterns
// carry unknown tips and weight 0.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "index_width.hpp"

namespace b3g {

constexpr uint32_t kTipBit = 0x80000000u;
constexpr int kMaxStates = 20;
constexpr int kMaxCategories = 16;
constexpr uint32_t kPatternAlign = 128;

// Shared-memory slot code meaning "global memory only" (run walk).
constexpr uint32_t kNoSlot = 0xFFu;

// One entry of the children-first schedule: output slot and the two
// children, each either a partial slot or (kTipBit | leaf id).
struct NodeOp {
	uint32_t out;
	uint32_t left;
	uint32_t right;
	uint32_t pad;
};

// Substitution model resident on the device, written by the host (the
// eigensystem is given or decomposed on the host); matrices row-major with
// row stride `states`.
struct ModelDev {
	double V[kMaxStates * kMaxStates];
	double Vinv[kMaxStates * kMaxStates];
	double lambda[kMaxStates];
	double Q[kMaxStates * kMaxStates];
	double pi[kMaxStates];
	double cat_rates[kMaxCategories];
	uint32_t shortcuts;
	uint32_t states;
};

struct PtabParams {
	const double *lengths;  // [n][2] time lengths, or null
	const double *matrices; // [n][2][C][S][S], or null
	const ModelDev *model;
	double clock_rate;
	uint32_t n;
	uint32_t C;
	void *ptab; // R [n][2][C][S+1][S]
};

struct PruneParams {
	const uint8_t *tips;
	void *partials;
	int32_t *scales;
	const NodeOp *ops;
	const void *ptab;
	const double *pi;
	const uint32_t *weights;
	double *site_lnl;   // [ldp]
	double *cat_lnl;    // [C][ldp] or null
	double *block_sums; // [gridDim.x]
	unsigned *ticket;   // zero between launches
	double *lnl_out;    // [1]
	double *lnl_host;   // host-mapped word that also receives it, or null
	// host-mapped [gridDim.x], or null: each block writes its sum there and
	// the host folds them (no ticket, no last-block fold, no lnl_out)
	double *sums_host;
	uint32_t n;
	uint32_t ldp;
	uint32_t C;
	uint32_t scale_ln;
	uint32_t num_leaves; // rows of tips
	uint32_t tips_smem;  // stage the block's tip codes in shared memory
	// 64-bit element indices whatever num_leaves says (the slot ids come
	// from a caller whose buffers may hold more than 2 * num_leaves slots)
	uint32_t wide_index;
	// run-synchronous walk (prune4_runs_kernel): runs[0..n_runs] are the
	// first entries of the runs of mutually independent entries, then n
	const uint32_t *runs;
	uint32_t n_runs;
	uint32_t tile; // patterns per tile
	uint32_t ptab_smem; // stage the transition tables in shared memory
	// per entry: shared-memory slot of the output (bits 0-7) and of the
	// left (8-15) and right (16-23) child, kNoSlot where the value lives
	// in global memory only; null or n_slots 0: no slots
	const uint32_t *slots;
	uint32_t n_slots;
	// run walk that builds its own transition tables (tables_inline):
	// run r + 1's tables are built while run r is walked, into a double
	// buffer of max_run entries in shared memory, with ptab4_kernel's
	// arithmetic, from the edge lengths (or the given matrices)
	const ModelDev *model;
	const double *lengths;  // [n][2], or null
	const double *matrices; // [n][2][C][4][4], or null
	double clock_rate;
	uint32_t tables_inline;
	uint32_t max_run;
	uint32_t lengths_smem; // stage the lengths in shared memory
	double scale_threshold;
	double scale_mult;
	double log_inv_c;
};

// One member of a batch (many calculators evaluated by one launch).  The
// pointers are the member's own device store; written once per batch.
struct MemberDesc {
	const uint8_t *tips;
	float *partials;     // FP32 chosen form
	int32_t *scales;
	float *ptab;
	const uint8_t *stage; // the member's staged block (ops, pi, runs, lengths)
	const ModelDev *model;
	const uint32_t *weights;
	double *site_lnl;
	double *tile_sums;   // one per tile, owned by the batch
	unsigned *ticket;    // tiles finished, owned by the batch
	uint32_t off_pi, off_runs, off_in;
	uint32_t ldp, C, L, tile;
	double log_inv_c;
};

// Per step and member, written by the host before every batched launch.
struct MemberStep {
	uint32_t n;      // dirty entries (0: nothing to evaluate)
	uint32_t n_runs;
	uint32_t tips_smem;
	uint32_t tile; // patterns per tile for this step (divides ldp)
	// a short list (n <= kDirectMax, C of 1, 2 or 4): walked by the
	// batched short-list kernel instead of the run walk
	uint32_t direct;
	double clock_rate;
};

struct BatchParams {
	const MemberDesc *members;
	const MemberStep *steps;
	double *lnl_out;     // [members]
	unsigned *work_next; // work counters, zero before each launch: [0] the
			     // run walk's, [1..3] the short-list kernels' (4,
			     // 2 and 1 categories)
	uint32_t num_members;
	uint32_t smem_ops_bytes;  // shared memory reserved for ops + runs
	uint32_t smem_tips_bytes; // shared memory reserved for a tip tile
	uint32_t max_cols;
	uint32_t narrow; // every member indexes with 32 bits
	uint32_t smem_ptab_bytes; // shared memory reserved for staged tables
};

// A run of the schedule holds at most kRunCap / C entries (at least 8):
// the run walk builds one run's transition tables in shared memory.
constexpr uint32_t kRunCap = 128;

// Transition tables of one list fit shared memory at most this large.
constexpr uint32_t kPtabSmemBytes = 32u * 1024u;

// Fused single-launch evaluation of a short list (FP32 chosen form, four
// states, one, two or four categories): the schedule, the edge lengths and the root
// frequencies travel in the kernel parameters, so the launch needs no
// upload, no transition kernel and no read-back copy.
constexpr uint32_t kDirectMax = 48; // entries
struct DirectParams {
	const uint8_t *tips;
	void *partials;
	int32_t *scales;
	const uint32_t *weights;
	const ModelDev *model;
	double *site_lnl;   // [ldp]
	double *block_sums; // [gridDim.x]
	unsigned *ticket;   // zero between launches
	double *lnl_out;    // device copy of the result
	double *lnl_host;   // host-mapped pinned word, written by the last block
			    // (without a host fold)
	// host-mapped [gridDim.x], or null: each block writes its sum there and
	// the host folds them (then lnl_out and lnl_host are not written)
	double *sums_host;
	uint32_t n, ldp, L, C; // C: 1, 2 or 4 categories
	double clock_rate;
	double log_inv_c;
	double pi[4];
	// the model as the table builder reads it, converted on the host with
	// the same rounding: V, V^-1, lambda in FP32, the shortcuts flag at
	// [36]; and clock rate x category rate in FP64 (the model in global
	// memory is read only on the shortcut paths)
	float eig[40];
	double rate[4];
	NodeOp ops[kDirectMax];
	double lengths[2 * kDirectMax]; // [n][2] time lengths
	// where entry i's left (0) and right (1) child comes from (kSrc*)
	uint8_t src[kDirectMax][2];
};

// Sources of a child in the fused short-list walk, set by the host: a tip
// code, a clean partial (not an output of this list: loaded ahead), the
// previous or the second previous entry's output (registers), or an older
// output of this list (read back when needed).
enum : uint8_t { kSrcTip = 0, kSrcClean, kSrcPrev, kSrcPrev2, kSrcEarlier };

// Launchers (kernels4.cu).  Each returns the launch error.
cudaError_t launch_ptab4(const PtabParams &p, bool f32, cudaStream_t s);
cudaError_t launch_prune4(const PruneParams &p, bool f32, uint32_t tile,
			  cudaStream_t s);
// Run-synchronous FP32 walk: `ctas` persistent blocks over ldp / p.tile
// pattern tiles.  Needs p.runs; block sums sized for `ctas`.
// dynamic shared memory of prune4_runs_kernel for these parameters
size_t prune4_runs_smem(const PruneParams &p);
// block: 512 (two blocks per SM) or 1024 threads (one per SM)
cudaError_t launch_prune4_runs(const PruneParams &p, uint32_t ctas,
			       uint32_t block, cudaStream_t s);
// 20-state tensor-core path (prune20tc.cuh), FP32 chosen form.
struct Tc20Params {
	const uint8_t *tips;
	float *partials;
	int32_t *scales;
	const NodeOp *ops;
	const float *tab;    // [n][2][C][21][20] tip rows
	const float *tc_tab; // [n][2][C][2][768] hi/lo MMA operand blocks
	const double *pi;
	const uint32_t *weights;
	double *root_val;    // [C][ldp] pi . x at the root
	int32_t *root_exp;   // [C][ldp] its power-of-two exponent
	double *site_lnl;    // [ldp]
	double *cat_lnl;     // [C][ldp] or null
	double *block_sums;  // [ldp / 128]
	unsigned *ticket;    // zero between launches
	double *lnl_out;
	unsigned *status;    // set to 1 when a bounded tensor-core wait gave up
	uint32_t n, ldp, C, L;
	uint32_t ops_smem;   // stage the list in shared memory
	uint32_t tips_smem;  // stage the tile's tip codes in shared memory
	uint32_t groups;     // 128-thread groups per CTA (1 or 2)
	uint32_t cluster;    // CTAs per (tile, category) work item, 1..8
	double log_inv_c;
};
// Dynamic shared memory of one tensor-core pruning CTA.
size_t prune20tc_smem(uint32_t groups, bool ops_smem, uint32_t n, bool tips_smem,
		      uint32_t L);
// Tables of both kinds for the tensor-core path: p.ptab receives the FP32
// tip rows, tc_tab the operand blocks.
cudaError_t launch_ptab20tc(const PtabParams &p, float *tc_tab, cudaStream_t s);
// Pruning (one CTA of p.groups x 128 threads per 128-pattern tile and
// category, 4 / p.groups CTAs per SM) then the root's category mixing and
// fold.
cudaError_t launch_prune20tc(const Tc20Params &p, cudaStream_t s);
// 20-state path (prune20.cuh): transition tables [n][2][C][21][20] computed
// in FP64, then one thread per (pattern, category) column walks the list;
// blocks of 32 patterns x C (C <= 8) categories.
cudaError_t launch_ptab20(const PtabParams &p, bool f32, cudaStream_t s);
cudaError_t launch_prune20(const PruneParams &p, bool f32, cudaStream_t s);
// Fused short-list evaluation: `ctas` persistent blocks over ldp / 128
// pattern tiles; needs p.n <= kDirectMax and block sums sized for `ctas`.
cudaError_t launch_prune4_direct(const DirectParams &p, uint32_t ctas,
				 cudaStream_t s);
// Batched evaluation (FP32): transition tables of every member with work,
// then one persistent pruning launch over all members' pattern tiles.
// max_entries = largest member n * 2 * C.
cudaError_t launch_ptab4_batch(const BatchParams &p, uint32_t max_entries,
			       cudaStream_t s);
cudaError_t launch_prune4_batch(const BatchParams &p, uint32_t ctas,
				cudaStream_t s);
// Batched short lists: every member whose step is direct and has C
// categories (1, 2 or 4), `ctas` persistent blocks taking (member, tile)
// items from that category count's counter.
cudaError_t launch_prune4_direct_batch(const BatchParams &p, uint32_t C,
				       uint32_t ctas, cudaStream_t s);

} // namespace b3g
