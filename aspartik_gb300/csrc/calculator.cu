// calculator.cu -- host orchestration of one device-resident pruning store
// and the C ABI declared in include/b3g.h.
#include "calculator.hpp"
#include "host_fold.hpp"
#include "host_math.hpp"

#include <cmath>
#include <cstring>
#include <algorithm>
#include <cstdlib>
#include <new>

namespace b3g {

void check_cuda(cudaError_t e, const char *what)
{
	if (e == cudaSuccess)
		return;
	const b3g_status s = e == cudaErrorMemoryAllocation
				     ? B3G_ERR_OUT_OF_MEMORY
				     : B3G_ERR_CUDA;
	throw Error(s, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct DeviceGuard {
	int prev = -1;
	explicit DeviceGuard(int dev)
	{
		check_cuda(cudaGetDevice(&prev), "cudaGetDevice");
		if (prev != dev)
			check_cuda(cudaSetDevice(dev), "cudaSetDevice");
	}
	~DeviceGuard()
	{
		int cur = -1;
		if (cudaGetDevice(&cur) == cudaSuccess && cur != prev && prev >= 0)
			cudaSetDevice(prev);
	}
};

template <typename T> void dev_alloc(T *&p, size_t bytes, const char *what)
{
	void *v = nullptr;
	check_cuda(cudaMalloc(&v, bytes ? bytes : 1), what);
	p = static_cast<T *>(v);
}

// EditBuf::set_edited (sk/src/editbuf.rs:71-81)
inline void set_edited(uint8_t &m)
{
	if (!(m & 2u))
		m = static_cast<uint8_t>(((m & 1u) ^ 1u) | 2u);
}

} // namespace

Calculator::Calculator(const b3g_config &cfg, const uint8_t *samples)
{
	if (cfg.num_leaves < 2)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "num_leaves must be >= 2");
	if (cfg.num_patterns < 1)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "num_patterns must be >= 1");
	if (cfg.num_states != 4 && cfg.num_states != 20)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "num_states must be 4 (DNA) or 20 (protein)");
	if (cfg.num_states == 20 && cfg.num_categories > 8)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "20-state calculators take at most 8 categories");
	if (cfg.num_categories < 1 || cfg.num_categories > kMaxCategories)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "num_categories must be in 1..16");
	if (cfg.precision != B3G_PRECISION_F64 &&
	    cfg.precision != B3G_PRECISION_F32)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "unknown precision");
	if (cfg.reserved != 0)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "reserved must be 0");
	if (!samples)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "samples is null");
	if (cfg.num_leaves > (1u << 24) || cfg.num_patterns > (1u << 28))
		throw Error(B3G_ERR_INVALID_ARGUMENT, "problem too large");

	L_ = cfg.num_leaves;
	I_ = L_ - 1;
	P_ = cfg.num_patterns;
	S_ = cfg.num_states;
	C_ = cfg.num_categories;
	f32_ = cfg.precision == B3G_PRECISION_F32;
	scale_ln_ = cfg.scale_ln;
	device_ = cfg.device;
	ldp_ = static_cast<uint32_t>(align_up(P_, kPatternAlign));
	// patterns per block: 128 threads for up to 4 categories, one warp of
	// patterns per category above that (at most 16 x 32 = 512 threads)
	tile_ = C_ <= 1 ? 128 : C_ == 2 ? 64 : 32;

	int ndev = 0;
	check_cuda(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
	if (device_ < 0 || device_ >= ndev)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "no such CUDA device");
	DeviceGuard g(device_);
	int sms = 0;
	check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount,
					  device_),
		   "SM count");
	num_sms_ = static_cast<uint32_t>(sms);
	// run-synchronous FP32 walk: 64 patterns x C categories per tile while
	// a tile's columns fit one 512-thread block
	runs_tile_ = 64;
	while (runs_tile_ > 32 && runs_tile_ * C_ > 512)
		runs_tile_ >>= 1;
	if (const char *env = std::getenv("B3G_RUNS_TILE")) {
		const uint32_t t = static_cast<uint32_t>(std::atoi(env));
		if (t == 16 || t == 32 || t == 64 || t == 128)
			runs_tile_ = t;
	}
	if (const char *env = std::getenv("B3G_RUNS_BLOCK")) {
		const uint32_t b = static_cast<uint32_t>(std::atoi(env));
		if (b == 512 || b == 1024)
			runs_block_ = b;
	}
	use_runs_ = f32_ && S_ == 4 && runs_tile_ * C_ <= 512;
	// fused single-launch evaluation of short lists (B3G_DIRECT=0 turns
	// it off, e.g. to time the two-kernel path)
	// 20-state FP32 lists on the tensor cores (B3G_TC20=0: CUDA-core walk)
	use_tc20_ = f32_ && S_ == 20;
	if (const char *env = std::getenv("B3G_TC20"))
		use_tc20_ = use_tc20_ && std::atoi(env) != 0;
	// groups of 128 threads per tensor-core CTA (B3G_TC20_GROUPS = 1 or 2;
	// default: chosen per launch from the grid size)
	if (const char *env = std::getenv("B3G_TC20_CLUSTER")) {
		const int k = std::atoi(env);
		if (k >= 1 && k <= 8) {
			tc20_cluster_ = static_cast<uint32_t>(k);
			tc20_cluster_fixed_ = true;
		}
	}
	if (const char *env = std::getenv("B3G_TC20_GROUPS")) {
		const int gr = std::atoi(env);
		if (gr == 1 || gr == 2) {
			tc20_groups_ = static_cast<uint32_t>(gr);
			tc20_groups_fixed_ = true;
		}
	}
	use_direct_ = f32_ && S_ == 4 && (C_ == 1 || C_ == 2 || C_ == 4);
	if (const char *env = std::getenv("B3G_DIRECT"))
		use_direct_ = use_direct_ && std::atoi(env) != 0;

	selectors_.assign(I_, 0);
	stamp_.assign(2 * L_ - 1, 0);
	pos_.assign(2 * L_ - 1, 0);
	run_of_.assign(I_, 0);
	smem_of_.assign(2ull * I_, static_cast<uint8_t>(kNoSlot));
	// shared-memory slots of the run walk (B3G_RUNS_SLOTS=0: children of
	// listed entries read back from global memory, to time the difference)
	if (const char *env = std::getenv("B3G_RUNS_SLOTS"))
		use_slots_ = std::atoi(env) != 0;
	// per-run tables built by the run walk itself (B3G_RUNS_INLINE=0: a
	// separate transition kernel writes every table to global memory)
	if (const char *env = std::getenv("B3G_RUNS_INLINE"))
		use_inline_ = std::atoi(env) != 0;
	{
		int per_sm = 0, reserved = 0;
		check_cuda(cudaDeviceGetAttribute(
				   &per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
				   device_),
			   "shared memory per SM");
		check_cuda(cudaDeviceGetAttribute(
				   &reserved, cudaDevAttrReservedSharedMemoryPerBlock,
				   device_),
			   "reserved shared memory");
		smem_per_sm_ = static_cast<uint32_t>(per_sm);
		smem_reserved_ = static_cast<uint32_t>(reserved);
	}

	const size_t slots = 2ull * I_;
	const size_t rsz = f32_ ? sizeof(float) : sizeof(double);
	// one block sum per thread block of any walk: at most one block per
	// 16 patterns (the smallest run-walk tile)
	const size_t nblocks = ldp_ / 16;
	block_sums_cap_ = static_cast<uint32_t>(nblocks);

	try {
		check_cuda(cudaStreamCreateWithFlags(&stream_,
						     cudaStreamNonBlocking),
			   "cudaStreamCreate");
		check_cuda(cudaEventCreateWithFlags(&ev_stage_free_,
						    cudaEventDisableTiming),
			   "cudaEventCreate");
		check_cuda(cudaEventCreateWithFlags(&ev_model_free_,
						    cudaEventDisableTiming),
			   "cudaEventCreate");
		check_cuda(cudaEventCreate(&ev_span0_), "cudaEventCreate");
		check_cuda(cudaEventCreate(&ev_span1_), "cudaEventCreate");
		for (auto &slot : ring_) {
			check_cuda(cudaEventCreate(&slot.k0), "cudaEventCreate");
			check_cuda(cudaEventCreate(&slot.kmid), "cudaEventCreate");
			check_cuda(cudaEventCreate(&slot.k1), "cudaEventCreate");
		}

		dev_alloc(d_tips_, (size_t)L_ * ldp_, "tips");
		dev_alloc(d_partials_, slots * C_ * ldp_ * S_ * rsz, "partials");
		dev_alloc(d_scales_, slots * C_ * ldp_ * sizeof(int32_t), "scales");
		dev_alloc(d_weights_, ldp_ * sizeof(uint32_t), "weights");
		dev_alloc(d_site_, ldp_ * sizeof(double), "site lnl");
		dev_alloc(d_cat_, (size_t)C_ * ldp_ * sizeof(double), "cat lnl");
		dev_alloc(d_block_sums_, nblocks * sizeof(double), "block sums");
		dev_alloc(d_ticket_, sizeof(unsigned), "ticket");
		dev_alloc(d_lnl_, sizeof(double), "lnl");
		if (use_tc20_) {
			dev_alloc(d_tc_tab_, (size_t)I_ * 2 * C_ * 2 * 768 * sizeof(float),
				  "tensor-core tables");
			dev_alloc(d_root_val_, (size_t)C_ * ldp_ * sizeof(double), "root values");
			dev_alloc(d_root_exp_, (size_t)C_ * ldp_ * sizeof(int32_t), "root exponents");
			dev_alloc(d_status_, sizeof(unsigned), "status");
			check_cuda(cudaMemset(d_status_, 0, sizeof(unsigned)), "zero status");
			check_cuda(cudaHostAlloc((void **)&h_status_, sizeof(unsigned),
						 cudaHostAllocDefault),
				   "pinned status");
			*h_status_ = 0;
		}
		dev_alloc(d_model_, sizeof(ModelDev), "model");
		dev_alloc(d_ptab_, (size_t)I_ * 2 * C_ * (S_ + 1) * S_ * rsz,
			  "transition tables");

		off_pi_ = align_up((size_t)I_ * sizeof(NodeOp), 256);
		off_runs_ = align_up(off_pi_ + S_ * sizeof(double), 256);
		off_slots_ = align_up(off_runs_ + (size_t)(I_ + 1) * sizeof(uint32_t), 256);
		off_in_ = align_up(off_slots_ + (size_t)I_ * sizeof(uint32_t), 256);
		stage_bytes_ = off_in_ + (size_t)I_ * 2 * C_ * S_ * S_ * sizeof(double);
		dev_alloc(d_stage_, stage_bytes_, "stage");
		check_cuda(cudaHostAlloc((void **)&h_stage_, stage_bytes_,
					 cudaHostAllocDefault),
			   "pinned stage");
		check_cuda(cudaHostAlloc((void **)&h_model_, sizeof(ModelDev),
					 cudaHostAllocDefault),
			   "pinned model");
		// mapped: the fused short-list kernel writes the result here
		check_cuda(cudaHostAlloc((void **)&h_lnl_, sizeof(double),
					 cudaHostAllocMapped),
			   "pinned lnl");
		check_cuda(cudaHostGetDevicePointer((void **)&d_lnl_host_, h_lnl_, 0),
			   "mapped lnl");
		if (f32_ && S_ == 4) {
			check_cuda(cudaHostAlloc((void **)&h_bsums_,
						 block_sums_cap_ * sizeof(double),
						 cudaHostAllocMapped),
				   "pinned block sums");
			check_cuda(cudaHostGetDevicePointer((void **)&d_bsums_, h_bsums_, 0),
				   "mapped block sums");
		}

		// DNA: single bases -> 0..3, everything else -> unknown (4)
		// (cpu4.rs:117-124).  Protein: states 0..19 as given, anything
		// else -> unknown (20).  Padded patterns are unknown too.
		std::vector<uint8_t> tips((size_t)L_ * ldp_, (uint8_t)S_);
		for (uint32_t l = 0; l < L_; ++l)
			for (uint32_t p = 0; p < P_; ++p) {
				const uint8_t code = samples[(size_t)l * P_ + p];
				uint8_t s;
				if (S_ == 4)
					s = code == 1 ? 0 : code == 2 ? 1
						   : code == 4 ? 2
						   : code == 8 ? 3
							       : 4;
				else
					s = code < S_ ? code : (uint8_t)S_;
				tips[(size_t)l * ldp_ + p] = s;
			}
		check_cuda(cudaMemcpy(d_tips_, tips.data(), tips.size(),
				      cudaMemcpyHostToDevice),
			   "upload tips");
		std::vector<uint32_t> w(ldp_, 0);
		for (uint32_t p = 0; p < P_; ++p)
			w[p] = 1;
		check_cuda(cudaMemcpy(d_weights_, w.data(), ldp_ * sizeof(uint32_t),
				      cudaMemcpyHostToDevice),
			   "upload weights");
		// Buffer::zeroed partials (cpu4.rs:134-136)
		check_cuda(cudaMemset(d_partials_, 0, slots * C_ * ldp_ * S_ * rsz),
			   "zero partials");
		check_cuda(cudaMemset(d_scales_, 0,
				      slots * C_ * ldp_ * sizeof(int32_t)),
			   "zero scales");
		check_cuda(cudaMemset(d_ticket_, 0, sizeof(unsigned)), "ticket");

		std::memset(&model_host_, 0, sizeof(model_host_));
		model_host_.states = S_;
		for (uint32_t c = 0; c < C_; ++c)
			model_host_.cat_rates[c] = 1.0;
		upload_model();
		check_cuda(cudaStreamSynchronize(stream_), "construct sync");
	} catch (...) {
		release();
		throw;
	}
}

Calculator::~Calculator() { release(); }

void Calculator::release()
{
	if (device_ >= 0)
		cudaSetDevice(device_);
	if (stream_)
		cudaStreamSynchronize(stream_);
	cudaFree(d_tips_);
	cudaFree(d_partials_);
	cudaFree(d_scales_);
	cudaFree(d_weights_);
	cudaFree(d_site_);
	cudaFree(d_cat_);
	cudaFree(d_tc_tab_);
	cudaFree(d_root_val_);
	cudaFree(d_root_exp_);
	cudaFree(d_status_);
	if (h_status_)
		cudaFreeHost(h_status_);
	d_tc_tab_ = nullptr;
	d_root_val_ = nullptr;
	d_root_exp_ = nullptr;
	d_status_ = nullptr;
	h_status_ = nullptr;
	cudaFree(d_block_sums_);
	cudaFree(d_ticket_);
	cudaFree(d_lnl_);
	cudaFree(d_model_);
	cudaFree(d_ptab_);
	cudaFree(own_d_stage_ ? own_d_stage_ : d_stage_);
	cudaFreeHost(own_h_stage_ ? own_h_stage_ : h_stage_);
	own_d_stage_ = nullptr;
	own_h_stage_ = nullptr;
	cudaFreeHost(h_model_);
	cudaFreeHost(h_lnl_);
	cudaFreeHost(h_bsums_);
	h_bsums_ = d_bsums_ = nullptr;
	d_tips_ = nullptr;
	d_partials_ = nullptr;
	d_scales_ = nullptr;
	d_weights_ = nullptr;
	d_site_ = d_cat_ = d_block_sums_ = d_lnl_ = nullptr;
	d_ticket_ = nullptr;
	d_model_ = nullptr;
	d_ptab_ = nullptr;
	d_stage_ = nullptr;
	h_stage_ = nullptr;
	h_model_ = nullptr;
	h_lnl_ = nullptr;
	for (cudaEvent_t *e : {&ev_stage_free_, &ev_model_free_, &ev_span0_,
			       &ev_span1_})
		if (*e) {
			cudaEventDestroy(*e);
			*e = nullptr;
		}
	for (auto &slot : ring_)
		for (cudaEvent_t *e : {&slot.k0, &slot.kmid, &slot.k1})
			if (*e) {
				cudaEventDestroy(*e);
				*e = nullptr;
			}
	if (stream_) {
		cudaStreamDestroy(stream_);
		stream_ = nullptr;
	}
}

void Calculator::upload_model()
{
	check_cuda(cudaEventSynchronize(ev_model_free_), "model staging");
	std::memcpy(h_model_, &model_host_, sizeof(ModelDev));
	check_cuda(cudaMemcpyAsync(d_model_, h_model_, sizeof(ModelDev),
				   cudaMemcpyHostToDevice, stream_),
		   "upload model");
	check_cuda(cudaEventRecord(ev_model_free_, stream_), "event");
	stream_dirty_ = true;
}

// The dirty list must name distinct internals, children must be valid node
// ids, and an internal child that is itself listed must come first
// (children-first order of partials_lists, parameters/tree.rs:398-421).
void Calculator::validate_lists(const uint32_t *internals,
				const uint32_t *children, uint32_t n)
{
	if (!internals || !children)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null list");
	if (n < 1 || n > I_)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "dirty list length must be in 1..num_internals");
	const uint32_t nodes = 2 * L_ - 1;
	// two stamps per call: `listed` marks the dirty internals, `done` the
	// ones already visited in list order
	if (stamp_epoch_ > 0xfffffff0u) {
		std::fill(stamp_.begin(), stamp_.end(), 0u);
		stamp_epoch_ = 0;
	}
	const uint32_t listed = ++stamp_epoch_;
	const uint32_t done = ++stamp_epoch_;
	for (uint32_t i = 0; i < n; ++i) {
		const uint32_t v = internals[i];
		if (v < L_ || v >= nodes)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "dirty list entry is not an internal node");
		if (stamp_[v] == listed)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "dirty list names a node twice");
		stamp_[v] = listed;
	}
	for (uint32_t i = 0; i < n; ++i) {
		const uint32_t v = internals[i];
		const uint32_t l = children[2 * i], r = children[2 * i + 1];
		for (const uint32_t ch : {l, r}) {
			if (ch >= nodes || ch == v)
				throw Error(B3G_ERR_INVALID_ARGUMENT,
					    "child is not a node id");
			if (ch >= L_ && stamp_[ch] == listed)
				throw Error(B3G_ERR_INVALID_ARGUMENT,
					    "dirty list is not children-first");
		}
		if (l == r)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "both children are the same node");
		stamp_[v] = done;
	}
}

// Flips the selectors of the listed internals (Cpu4Calculator::
// set_selectors, cpu4.rs:93-98) and writes the schedule: output slot of each
// listed node and the slot or leaf of each child.
void Calculator::stage_ops(const uint32_t *internals, const uint32_t *children,
			   uint32_t n)
{
	for (uint32_t i = 0; i < n; ++i)
		set_edited(selectors_[internals[i] - L_]);
	NodeOp *ops = reinterpret_cast<NodeOp *>(h_stage_);
	auto slot_of = [&](uint32_t v) {
		const uint32_t k = v - L_;
		return k * 2 + (selectors_[k] & 1u);
	};
	// Runs of mutually independent entries: entry i opens a new run when
	// one of its children is listed inside the current run.  validate_lists
	// left stamp_[v] == stamp_epoch_ on every listed internal.
	// A run holds at most kRunCap / C entries, so that the run walk's
	// per-run transition tables fit shared memory.
	uint32_t run_start = 0;
	const uint32_t cap = std::max(8u, kRunCap / C_);
	tip_children_ = 0;
	for (uint32_t i = 0; i < n; ++i) {
		if (i - run_start >= cap)
			run_start = i;
		NodeOp op;
		op.out = slot_of(internals[i]);
		const uint32_t l = children[2 * i], r = children[2 * i + 1];
		op.left = l < L_ ? (kTipBit | l) : slot_of(l);
		op.right = r < L_ ? (kTipBit | r) : slot_of(r);
		tip_children_ += (l < L_) + (r < L_);
		for (const uint32_t ch : {l, r})
			if (ch >= L_ && stamp_[ch] == stamp_epoch_ &&
			    pos_[ch] >= run_start)
				run_start = i;
		pos_[internals[i]] = i;
		run_of_[i] = run_start;
		ops[i] = op;
	}
	// NodeOp::pad = entries left in the run, this one included
	for (uint32_t i = n; i-- > 0;)
		ops[i].pad = (i + 1 < n && run_of_[i + 1] == run_of_[i])
				     ? ops[i + 1].pad + 1
				     : 1;
	// run starts, then n
	uint32_t *runs = reinterpret_cast<uint32_t *>(h_stage_ + off_runs_);
	n_runs_ = 0;
	max_run_ = 0;
	for (uint32_t i = 0; i < n; ++i)
		if (run_of_[i] == i) {
			if (n_runs_)
				max_run_ = std::max(max_run_, i - runs[n_runs_ - 1]);
			runs[n_runs_++] = i;
		}
	runs[n_runs_] = n;
	if (n_runs_)
		max_run_ = std::max(max_run_, n - runs[n_runs_ - 1]);
}

// Shared-memory slots for the run walk's outputs (at most `capacity`),
// written as per-entry codes beside the schedule.  A listed child is read
// by exactly one entry, its parent, so an entry may write its output into
// its left (else right) child's slot; an entry without a slotted child
// takes a slot released in an earlier run; the slot of a second slotted
// child is released at the end of the run.  Outputs left without a slot,
// and the last entry's, are read from global memory (or, for the last,
// from registers).  Returns the number of slots used.
uint32_t Calculator::assign_slots(uint32_t n, uint32_t capacity)
{
	if (capacity == 0)
		return 0;
	const NodeOp *ops = reinterpret_cast<const NodeOp *>(h_stage_);
	uint32_t *codes = reinterpret_cast<uint32_t *>(h_stage_ + off_slots_);
	free_slots_.clear();
	pending_slots_.clear();
	for (uint32_t k = capacity; k-- > 0;)
		free_slots_.push_back(static_cast<uint8_t>(k));
	auto src = [&](uint32_t id) -> uint32_t {
		return (id & kTipBit) ? kNoSlot : smem_of_[id];
	};
	uint32_t used = 0;
	for (uint32_t i = 0; i < n; ++i) {
		if (run_of_[i] == i) {
			free_slots_.insert(free_slots_.end(), pending_slots_.begin(),
					   pending_slots_.end());
			pending_slots_.clear();
		}
		const uint32_t ls = src(ops[i].left), rs = src(ops[i].right);
		uint32_t os = kNoSlot;
		if (i + 1 < n) {
			if (ls != kNoSlot) {
				os = ls;
				if (rs != kNoSlot)
					pending_slots_.push_back(static_cast<uint8_t>(rs));
			} else if (rs != kNoSlot) {
				os = rs;
			} else if (!free_slots_.empty()) {
				os = free_slots_.back();
				free_slots_.pop_back();
			}
		}
		smem_of_[ops[i].out] = static_cast<uint8_t>(os);
		if (os != kNoSlot)
			used = std::max(used, os + 1);
		codes[i] = os | (ls << 8) | (rs << 16);
	}
	for (uint32_t i = 0; i < n; ++i)
		smem_of_[ops[i].out] = static_cast<uint8_t>(kNoSlot);
	return used;
}

void Calculator::launch(uint32_t n, bool matrices_mode, double clock_rate,
			bool want_cat)
{
	host_fold_blocks_ = 0;
	if (use_direct_ && !matrices_mode && !want_cat && n > 0 &&
	    n <= kDirectMax) {
		launch_direct(n, clock_rate);
		return;
	}
	// run walk configuration, decided before the upload because the slot
	// codes travel with the schedule
	const bool runs = S_ == 4 && use_runs_ && n <= 4096;
	PruneParams pp{};
	uint32_t block = 512;
	if (runs) {
		pp.n = n;
		pp.C = C_;
		pp.num_leaves = L_;
		pp.n_runs = n_runs_;
		pp.tile = pick_tile(n);
		pp.tips_smem = (4ull * tip_children_ >= L_ &&
				(size_t)L_ * pp.tile <= 32u * 1024u)
				       ? 1u
				       : 0u;
		pp.ptab_smem = (size_t)n * 2 * C_ * 5 * 16 <= kPtabSmemBytes ? 1u : 0u;
		const uint32_t cols = pp.tile * C_;
		// 1024-thread blocks only for the run walk proper (a 512-column
		// tile is the serial walk of a 512-thread block)
		block = (runs_block_ == 1024 && cols < 512) ? 1024u : 512u;
		const uint32_t budget = smem_budget(block);
		if (use_inline_ && block / cols >= 2 && max_run_ > 0) {
			// the walk builds each run's tables itself, one run ahead
			pp.tables_inline = 1;
			pp.ptab_smem = 0;
			pp.max_run = max_run_;
			pp.lengths_smem = (!matrices_mode && n <= 1024) ? 1u : 0u;
			if (prune4_runs_smem(pp) > budget) {
				pp.tables_inline = 0;
				pp.max_run = 0;
				pp.lengths_smem = 0;
				pp.ptab_smem = (size_t)n * 2 * C_ * 5 * 16 <= kPtabSmemBytes
						       ? 1u
						       : 0u;
			}
		}
		if (use_slots_ && block / cols >= 2) {
			// as many slots as fit beside the rest
			pp.n_slots = 1;
			const size_t one = prune4_runs_smem(pp);
			const size_t per = (size_t)cols * (sizeof(float4) + sizeof(int32_t));
			const size_t cap = one <= budget ? 1 + (budget - one) / per : 0;
			pp.n_slots = assign_slots(
				n, static_cast<uint32_t>(std::min<size_t>(cap, kNoSlot - 1)));
		}
	}
	const size_t in_bytes =
		matrices_mode ? (size_t)n * 2 * C_ * S_ * S_ * sizeof(double)
			      : (size_t)n * 2 * sizeof(double);
	last_upload_bytes_ = off_in_ + in_bytes;
	check_cuda(cudaMemcpyAsync(d_stage_, h_stage_, last_upload_bytes_,
				   cudaMemcpyHostToDevice, stream_),
		   "upload step");
	check_cuda(cudaEventRecord(ev_stage_free_, stream_), "event");
	upload_pending_ = true;
	TimingSlot &slot = ring_[ring_next_ % kRing];
	if (slot.pending)
		harvest(slot); // recorded kRing proposals ago: long complete
	slot.direct = false;
	record(slot.k0);

	if (S_ == 20) {
		launch20(n, matrices_mode, clock_rate, want_cat, slot);
		return;
	}
	PtabParams pt{};
	pt.lengths = matrices_mode
			     ? nullptr
			     : reinterpret_cast<const double *>(d_stage_ + off_in_);
	pt.matrices = matrices_mode
			      ? reinterpret_cast<const double *>(d_stage_ + off_in_)
			      : nullptr;
	pt.model = d_model_;
	pt.clock_rate = clock_rate;
	pt.n = n;
	pt.C = C_;
	pt.ptab = d_ptab_;
	if (pp.tables_inline) {
		pp.model = d_model_;
		pp.lengths = pt.lengths;
		pp.matrices = pt.matrices;
		pp.clock_rate = clock_rate;
		last_launches_ = 1;
	} else {
		check_cuda(launch_ptab4(pt, f32_, stream_), "transition kernel");
		last_launches_ = 2;
	}
	record(slot.kmid);

	pp.tips = d_tips_;
	pp.partials = d_partials_;
	pp.scales = d_scales_;
	pp.ops = reinterpret_cast<const NodeOp *>(d_stage_);
	pp.ptab = d_ptab_;
	pp.pi = reinterpret_cast<const double *>(d_stage_ + off_pi_);
	pp.weights = d_weights_;
	pp.site_lnl = d_site_;
	pp.cat_lnl = want_cat ? d_cat_ : nullptr;
	pp.block_sums = d_block_sums_;
	pp.ticket = d_ticket_;
	pp.lnl_out = d_lnl_;
	pp.n = n;
	pp.ldp = ldp_;
	pp.C = C_;
	pp.scale_ln = scale_ln_;
	pp.num_leaves = L_;
	// stage the tip tile when the list reads at least a quarter of the
	// leaves and the tile fits in 64 KiB of shared memory (the run walk
	// decided its own above)
	if (!runs)
		pp.tips_smem = (4ull * tip_children_ >= L_ &&
				(size_t)L_ * tile_ <= 64u * 1024u)
				       ? 1u
				       : 0u;
	pp.scale_threshold = std::exp(-static_cast<double>(scale_ln_));
	pp.scale_mult = std::exp(static_cast<double>(scale_ln_));
	pp.log_inv_c = std::log(1.0 / static_cast<double>(C_));
	// the run-synchronous walk stages the schedule in shared memory: keep
	// it for lists up to 4,096 entries
	if (runs) {
		pp.runs = reinterpret_cast<const uint32_t *>(d_stage_ + off_runs_);
		pp.slots = reinterpret_cast<const uint32_t *>(d_stage_ + off_slots_);
		const uint32_t tiles = ldp_ / pp.tile;
		const uint32_t ctas = std::min(tiles, num_sms_ * (1024 / block));
		if (ctas > block_sums_cap_)
			throw Error(B3G_ERR_STATE, "run walk grid exceeds the block sums");
		// the blocks' sums go straight to mapped host memory
		if (d_bsums_) {
			pp.sums_host = d_bsums_;
			arm_host_fold(ctas);
		} else {
			pp.lnl_host = d_lnl_host_;
			arm_poll();
		}
		check_cuda(launch_prune4_runs(pp, ctas, block, stream_), "pruning kernel");
	} else {
		poll_result_ = false;
		check_cuda(launch_prune4(pp, f32_, tile_, stream_), "pruning kernel");
	}
	++in_flight_;
	record(slot.k1);
	slot.pending = timing_;
	ring_next_ += timing_ ? 1 : 0;
	if (!runs)
		check_cuda(cudaMemcpyAsync(h_lnl_, d_lnl_, sizeof(double),
					   cudaMemcpyDeviceToHost, stream_),
			   "read lnl");
	have_result_ = true;
	outstanding_ = true;
	stream_dirty_ = true;
	cat_valid_ = want_cat;
}

// 20-state list: table kernel, then the column walk (prune20.cuh).
void Calculator::launch20(uint32_t n, bool matrices_mode, double clock_rate,
			  bool want_cat, TimingSlot &slot)
{
	poll_result_ = false; // result read back by a copy after the kernels
	++in_flight_;
	PtabParams pt{};
	pt.lengths = matrices_mode
			     ? nullptr
			     : reinterpret_cast<const double *>(d_stage_ + off_in_);
	pt.matrices = matrices_mode
			      ? reinterpret_cast<const double *>(d_stage_ + off_in_)
			      : nullptr;
	pt.model = d_model_;
	pt.clock_rate = clock_rate;
	pt.n = n;
	pt.C = C_;
	pt.ptab = d_ptab_;
	if (use_tc20_) {
		check_cuda(launch_ptab20tc(pt, d_tc_tab_, stream_), "transition kernel");
		last_launches_ = 3; // tables, pruning, root and sum
		record(slot.kmid);
		Tc20Params tp{};
		tp.tips = d_tips_;
		tp.partials = static_cast<float *>(d_partials_);
		tp.scales = d_scales_;
		tp.ops = reinterpret_cast<const NodeOp *>(d_stage_);
		tp.tab = static_cast<const float *>(d_ptab_);
		tp.tc_tab = d_tc_tab_;
		tp.pi = reinterpret_cast<const double *>(d_stage_ + off_pi_);
		tp.weights = d_weights_;
		tp.root_val = d_root_val_;
		tp.root_exp = d_root_exp_;
		tp.site_lnl = d_site_;
		tp.cat_lnl = want_cat ? d_cat_ : nullptr;
		tp.block_sums = d_block_sums_;
		tp.ticket = d_ticket_;
		tp.lnl_out = d_lnl_;
		tp.status = d_status_;
		tp.n = n;
		tp.ldp = ldp_;
		tp.C = C_;
		tp.L = L_;
		// the list, then the tile's tip codes, in shared memory when they
		// fit beside the operand areas at 4 / groups CTAs per SM
		// two groups (on independent entries of a run) unless the grid
		// holds six or more CTAs per SM, where one group per CTA and up to
		// four CTAs per SM hide the per-entry latency as well (measured:
		// two groups faster at 1 and 4.1 CTAs per SM, one at 10.2)
		const uint32_t groups =
			tc20_groups_ ? tc20_groups_
				     : ((ldp_ / 128u) * C_ < 6u * num_sms_ ? 2u : 1u);
		tp.groups = groups;
		// a work item (tile, category) spread over a cluster of CTAs
		// while the grid has fewer items than CTA slots (4 / groups per
		// SM), so that every SM holds groups on independent entries
		const uint32_t items = (ldp_ / 128u) * C_;
		uint32_t cluster = std::max(1u, std::min(8u, (4u / groups) * num_sms_ /
								      std::max(items, 1u)));
		if (tc20_cluster_fixed_)
			cluster = tc20_cluster_;
		tp.cluster = cluster;
		const size_t budget = smem_budget(256u * groups);
		const size_t ops_bytes = (size_t)n * sizeof(NodeOp);
		size_t used = prune20tc_smem(groups, false, n, false, L_);
		tp.ops_smem = used + ops_bytes <= budget ? 1u : 0u;
		used += tp.ops_smem ? ops_bytes : 0;
		tp.tips_smem = used + (size_t)L_ * 128u <= budget ? 1u : 0u;
		tp.log_inv_c = std::log(1.0 / static_cast<double>(C_));
		check_cuda(launch_prune20tc(tp, stream_), "tensor-core pruning kernel");
		record(slot.k1);
		slot.pending = timing_;
		ring_next_ += timing_ ? 1 : 0;
		check_cuda(cudaMemcpyAsync(h_lnl_, d_lnl_, sizeof(double),
					   cudaMemcpyDeviceToHost, stream_),
			   "read lnl");
		check_cuda(cudaMemcpyAsync(h_status_, d_status_, sizeof(unsigned),
					   cudaMemcpyDeviceToHost, stream_),
			   "read status");
		have_result_ = true;
		outstanding_ = true;
		stream_dirty_ = true;
		cat_valid_ = want_cat;
		return;
	}
	check_cuda(launch_ptab20(pt, f32_, stream_), "transition kernel");
	last_launches_ = 2;
	record(slot.kmid);
	PruneParams pp{};
	pp.tips = d_tips_;
	pp.partials = d_partials_;
	pp.scales = d_scales_;
	pp.ops = reinterpret_cast<const NodeOp *>(d_stage_);
	pp.ptab = d_ptab_;
	pp.pi = reinterpret_cast<const double *>(d_stage_ + off_pi_);
	pp.weights = d_weights_;
	pp.site_lnl = d_site_;
	pp.cat_lnl = want_cat ? d_cat_ : nullptr;
	pp.block_sums = d_block_sums_;
	pp.ticket = d_ticket_;
	pp.lnl_out = d_lnl_;
	pp.n = n;
	pp.ldp = ldp_;
	pp.C = C_;
	pp.scale_ln = scale_ln_;
	pp.num_leaves = L_;
	pp.scale_threshold = std::exp(-static_cast<double>(scale_ln_));
	pp.scale_mult = std::exp(static_cast<double>(scale_ln_));
	pp.log_inv_c = std::log(1.0 / static_cast<double>(C_));
	check_cuda(launch_prune20(pp, f32_, stream_), "pruning kernel");
	record(slot.k1);
	slot.pending = timing_;
	ring_next_ += timing_ ? 1 : 0;
	check_cuda(cudaMemcpyAsync(h_lnl_, d_lnl_, sizeof(double),
				   cudaMemcpyDeviceToHost, stream_),
		   "read lnl");
	have_result_ = true;
	outstanding_ = true;
	stream_dirty_ = true;
	cat_valid_ = want_cat;
}

// One launch for a short FP32 list: the staged schedule, the lengths and
// the root frequencies go into the kernel parameters (nothing is uploaded),
// the kernel builds its transition tables in shared memory and writes the
// result into the mapped pinned word that log_likelihood() reads.
void Calculator::launch_direct(uint32_t n, double clock_rate)
{
	DirectParams dp;
	dp.tips = d_tips_;
	dp.partials = d_partials_;
	dp.scales = d_scales_;
	dp.weights = d_weights_;
	dp.model = d_model_;
	dp.site_lnl = d_site_;
	dp.block_sums = d_block_sums_;
	dp.ticket = d_ticket_;
	dp.lnl_out = d_lnl_;
	dp.lnl_host = d_lnl_host_;
	dp.sums_host = d_bsums_;
	dp.n = n;
	dp.ldp = ldp_;
	dp.L = L_;
	dp.C = C_;
	dp.clock_rate = clock_rate;
	dp.log_inv_c = std::log(1.0 / static_cast<double>(C_));
	std::memcpy(dp.pi, h_stage_ + off_pi_, 4 * sizeof(double));
	for (int k = 0; k < 16; ++k) {
		dp.eig[k] = static_cast<float>(model_host_.V[k]);
		dp.eig[16 + k] = static_cast<float>(model_host_.Vinv[k]);
	}
	for (int k = 0; k < 4; ++k) {
		dp.eig[32 + k] = static_cast<float>(model_host_.lambda[k]);
		dp.rate[k] = clock_rate * model_host_.cat_rates[k];
	}
	dp.eig[36] = model_host_.shortcuts ? 1.0f : 0.0f;
	dp.eig[37] = dp.eig[38] = dp.eig[39] = 0.0f;
	std::memcpy(dp.ops, h_stage_, (size_t)n * sizeof(NodeOp));
	std::memcpy(dp.lengths, h_stage_ + off_in_, (size_t)n * 2 * sizeof(double));
	// where each child comes from in the walk
	for (uint32_t i = 0; i < n; ++i) {
		const uint32_t ids[2] = {dp.ops[i].left, dp.ops[i].right};
		for (int j = 0; j < 2; ++j) {
			const uint32_t id = ids[j];
			uint8_t src = kSrcClean;
			if (id & kTipBit) {
				src = kSrcTip;
			} else if (i >= 1 && id == dp.ops[i - 1].out) {
				src = kSrcPrev;
			} else if (i >= 2 && id == dp.ops[i - 2].out) {
				src = kSrcPrev2;
			} else {
				for (uint32_t k = 0; k + 2 < i; ++k)
					if (dp.ops[k].out == id) {
						src = kSrcEarlier;
						break;
					}
			}
			dp.src[i][j] = src;
		}
	}
	// bytes that reach the device with the launch
	last_upload_bytes_ = (uint64_t)n * (sizeof(NodeOp) + 2 * sizeof(double)) +
			     4 * sizeof(double);
	TimingSlot &slot = ring_[ring_next_ % kRing];
	if (slot.pending)
		harvest(slot);
	slot.direct = true;
	record(slot.k0);
	// 128-pattern tiles, 128 * C threads per block, 1024 threads per SM
	const uint32_t ctas = std::min(ldp_ / 128u, (8u / C_) * num_sms_);
	if (ctas > block_sums_cap_)
		throw Error(B3G_ERR_STATE, "short-list grid exceeds the block sums");
	if (d_bsums_)
		arm_host_fold(ctas);
	else
		arm_poll();
	check_cuda(launch_prune4_direct(dp, ctas, stream_), "fused pruning kernel");
	++in_flight_;
	last_launches_ = 1;
	record(slot.k1);
	slot.pending = timing_;
	ring_next_ += timing_ ? 1 : 0;
	have_result_ = true;
	outstanding_ = true;
	stream_dirty_ = true;
	cat_valid_ = false;
}

void Calculator::propose_matrices(const uint32_t *internals,
				  const uint32_t *children, uint32_t n,
				  const double *matrices, const double *freqs)
{
	DeviceGuard g(device_);
	validate_lists(internals, children, n);
	if (!matrices || !freqs)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null matrices");
	if (own_h_stage_)
		throw Error(B3G_ERR_STATE,
			    "a calculator in a batch takes edge-length proposals only");
	const size_t count = (size_t)n * 2 * C_ * S_ * S_;
	for (size_t k = 0; k < count; ++k)
		if (!std::isfinite(matrices[k]))
			throw Error(B3G_ERR_NUMERIC, "non-finite transition matrix");
	for (uint32_t s = 0; s < S_; ++s)
		if (!std::isfinite(freqs[s]))
			throw Error(B3G_ERR_NUMERIC, "non-finite frequency");
	wait_stage();
	stage_ops(internals, children, n);
	std::memcpy(h_stage_ + off_pi_, freqs, S_ * sizeof(double));
	std::memcpy(h_stage_ + off_in_, matrices, count * sizeof(double));
	launch(n, true, 1.0, true);
}

void Calculator::propose_lengths(const uint32_t *internals,
				 const uint32_t *children, uint32_t n,
				 const double *lengths, double clock_rate)
{
	DeviceGuard g(device_);
	if (!model_set_)
		throw Error(B3G_ERR_STATE,
			    "no substitution model set before propose_lengths");
	validate_lists(internals, children, n);
	if (!lengths)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null lengths");
	for (size_t k = 0; k < (size_t)n * 2; ++k)
		if (!std::isfinite(lengths[k]))
			throw Error(B3G_ERR_NUMERIC, "non-finite edge length");
	if (!std::isfinite(clock_rate))
		throw Error(B3G_ERR_NUMERIC, "non-finite clock rate");
	wait_stage();
	if (batch_done_)
		check_cuda(cudaEventSynchronize(batch_done_), "batch stage reuse");
	stage_ops(internals, children, n);
	std::memcpy(h_stage_ + off_pi_, model_host_.pi, S_ * sizeof(double));
	std::memcpy(h_stage_ + off_in_, lengths, (size_t)n * 2 * sizeof(double));
	staged_ = false;
	launch(n, false, clock_rate, false);
}

void Calculator::stage_lengths(const uint32_t *internals,
			       const uint32_t *children, uint32_t n,
			       const double *lengths, double clock_rate)
{
	DeviceGuard g(device_);
	if (!in_batch_)
		throw Error(B3G_ERR_STATE,
			    "stage_lengths needs the calculator to be in a batch");
	if (!model_set_)
		throw Error(B3G_ERR_STATE,
			    "no substitution model set before stage_lengths");
	if (n > 4096)
		throw Error(B3G_ERR_INVALID_ARGUMENT,
			    "batched lists hold at most 4,096 entries");
	validate_lists(internals, children, n);
	if (!lengths)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null lengths");
	for (size_t k = 0; k < (size_t)n * 2; ++k)
		if (!std::isfinite(lengths[k]))
			throw Error(B3G_ERR_NUMERIC, "non-finite edge length");
	if (!std::isfinite(clock_rate))
		throw Error(B3G_ERR_NUMERIC, "non-finite clock rate");
	// the batch's previous copy of this staging buffer must be done, and
	// so must this calculator's own last launch
	wait_stage();
	if (batch_done_)
		check_cuda(cudaEventSynchronize(batch_done_), "batch stage reuse");
	stage_ops(internals, children, n);
	std::memcpy(h_stage_ + off_pi_, model_host_.pi, S_ * sizeof(double));
	std::memcpy(h_stage_ + off_in_, lengths, (size_t)n * 2 * sizeof(double));
	staged_ = true;
	staged_n_ = n;
	staged_clock_ = clock_rate;
	staged_tile_ = pick_tile(n);
	staged_tips_smem_ = (4ull * tip_children_ >= L_ &&
			     (size_t)L_ * staged_tile_ <= 32u * 1024u)
				    ? 1u
				    : 0u;
	have_result_ = false; // results come from the batch
}

void Calculator::likelihoods(double *out)
{
	DeviceGuard g(device_);
	if (!out)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null output");
	if (!have_result_ || !cat_valid_)
		throw Error(B3G_ERR_STATE,
			    "likelihoods() needs a preceding propose()");
	check_cuda(cudaMemcpy2DAsync(out, P_ * sizeof(double), d_cat_,
				     ldp_ * sizeof(double), P_ * sizeof(double),
				     C_, cudaMemcpyDeviceToHost, stream_),
		   "read likelihoods");
	check_cuda(cudaStreamSynchronize(stream_), "sync");
	upload_pending_ = false;
	in_flight_ = 0;
}

namespace {
// a NaN payload the kernels never write
constexpr uint64_t kLnlSentinel = 0x7ff4b3a9c0de5e11ull;
} // namespace

void Calculator::arm_poll()
{
	poll_result_ = in_flight_ == 0;
	if (poll_result_)
		std::memcpy(h_lnl_, &kLnlSentinel, sizeof(double));
}

void Calculator::arm_host_fold(uint32_t blocks)
{
	host_fold_blocks_ = blocks;
	poll_result_ = in_flight_ == 0;
	if (poll_result_)
		for (uint32_t k = 0; k < blocks; ++k)
			std::memcpy(h_bsums_ + k, &kLnlSentinel, sizeof(double));
}

// Waits for every block's mapped sum to leave the sentinel (the same
// stream queries as wait_mapped); false: the stream finished with a sum
// missing, or polling was not armed.
bool Calculator::wait_host_sums()
{
	const volatile uint64_t *w = reinterpret_cast<const volatile uint64_t *>(h_bsums_);
	uint32_t k = 0;
	for (uint32_t poll = 1; k < host_fold_blocks_; ++poll) {
		if (w[k] != kLnlSentinel) {
			++k;
			continue;
		}
		if ((poll & 63u) == 0) {
			const cudaError_t e = cudaStreamQuery(stream_);
			if (e == cudaSuccess) {
				for (; k < host_fold_blocks_; ++k)
					if (w[k] == kLnlSentinel)
						return false;
				return true;
			}
			if (e != cudaErrorNotReady)
				check_cuda(e, "evaluation");
		}
	}
	return true;
}

double Calculator::fold_host_sums() const
{
	return fold_block_sums(h_bsums_, host_fold_blocks_);
}

// Waits for the mapped result word to leave the sentinel; every 64 polls
// the stream is queried, so a launch error surfaces and a stream that
// finished without writing the word ends the wait (false: synchronise).
bool Calculator::wait_mapped(double &value)
{
	const volatile uint64_t *w = reinterpret_cast<const volatile uint64_t *>(h_lnl_);
	for (uint32_t k = 1;; ++k) {
		uint64_t bits = *w;
		if (bits != kLnlSentinel) {
			std::memcpy(&value, &bits, sizeof(double));
			return true;
		}
		if ((k & 63u) == 0) {
			const cudaError_t e = cudaStreamQuery(stream_);
			if (e == cudaSuccess) {
				bits = *w;
				if (bits == kLnlSentinel)
					return false;
				std::memcpy(&value, &bits, sizeof(double));
				return true;
			}
			if (e != cudaErrorNotReady)
				check_cuda(e, "evaluation");
		}
	}
}

double Calculator::log_likelihood()
{
	DeviceGuard g(device_);
	if (!have_result_)
		throw Error(B3G_ERR_STATE, "no proposal evaluated yet");
	double value;
	if (host_fold_blocks_) {
		if (!(poll_result_ && wait_host_sums()))
			check_cuda(cudaStreamSynchronize(stream_), "sync");
		upload_pending_ = false;
		in_flight_ = 0;
		for (uint32_t k = 0; k < host_fold_blocks_; ++k) {
			uint64_t bits;
			std::memcpy(&bits, h_bsums_ + k, sizeof(bits));
			if (poll_result_ && bits == kLnlSentinel)
				throw Error(B3G_ERR_CUDA,
					    "the evaluation finished without writing its result");
		}
		value = fold_host_sums();
		// later reads return the folded value
		*h_lnl_ = value;
		host_fold_blocks_ = 0;
		poll_result_ = false;
		return value;
	}
	if (poll_result_ && wait_mapped(value)) {
		// the kernel ran, so the upload before it did too
		upload_pending_ = false;
		in_flight_ = 0;
		return value;
	}
	check_cuda(cudaStreamSynchronize(stream_), "sync");
	upload_pending_ = false;
	in_flight_ = 0;
	if (poll_result_) {
		uint64_t bits;
		std::memcpy(&bits, h_lnl_, sizeof(bits));
		if (bits == kLnlSentinel)
			throw Error(B3G_ERR_CUDA,
				    "the evaluation finished without writing its result");
	}
	if (h_status_ && *h_status_)
		throw Error(B3G_ERR_TIMEOUT,
			    "a tensor-core wait of the 20-state kernel gave up");
	return *h_lnl_;
}

void Calculator::site_log_likelihoods(double *out)
{
	DeviceGuard g(device_);
	if (!out)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null output");
	if (!have_result_)
		throw Error(B3G_ERR_STATE, "no proposal evaluated yet");
	check_cuda(cudaMemcpyAsync(out, d_site_, P_ * sizeof(double),
				   cudaMemcpyDeviceToHost, stream_),
		   "read site lnl");
	check_cuda(cudaStreamSynchronize(stream_), "sync");
	upload_pending_ = false;
	in_flight_ = 0;
}

// The staging buffer may be rewritten once the last upload from it has
// run: wait for that upload, unless the stream was synchronised since it
// was queued (the common case: the result was read before the next
// proposal).
void Calculator::wait_stage()
{
	if (upload_pending_) {
		check_cuda(cudaEventSynchronize(ev_stage_free_), "stage reuse");
		upload_pending_ = false;
	}
}

void Calculator::record(cudaEvent_t e)
{
	if (timing_)
		check_cuda(cudaEventRecord(e, stream_), "event");
}

void Calculator::harvest(TimingSlot &s)
{
	check_cuda(cudaEventSynchronize(s.k1), "timing sync");
	float t = 0.0f, p = 0.0f;
	if (s.direct) { // one fused kernel: all of it counts as pruning
		check_cuda(cudaEventElapsedTime(&p, s.k0, s.k1), "elapsed");
	} else {
		check_cuda(cudaEventElapsedTime(&t, s.k0, s.kmid), "elapsed");
		check_cuda(cudaEventElapsedTime(&p, s.kmid, s.k1), "elapsed");
	}
	acc_transition_ms_ += t;
	acc_prune_ms_ += p;
	++acc_count_;
	s.pending = false;
}

void Calculator::last_timing(float *transition_ms, float *prune_ms)
{
	DeviceGuard g(device_);
	if (!timing_)
		throw Error(B3G_ERR_STATE,
			    "timing is off (b3g_calculator_set_timing)");
	if (!have_result_ || ring_next_ == 0)
		throw Error(B3G_ERR_STATE, "no proposal evaluated yet");
	TimingSlot &s = ring_[(ring_next_ - 1) % kRing];
	check_cuda(cudaEventSynchronize(s.k1), "sync");
	if (s.direct) {
		*transition_ms = 0.0f;
		check_cuda(cudaEventElapsedTime(prune_ms, s.k0, s.k1), "elapsed");
		return;
	}
	check_cuda(cudaEventElapsedTime(transition_ms, s.k0, s.kmid), "elapsed");
	check_cuda(cudaEventElapsedTime(prune_ms, s.kmid, s.k1), "elapsed");
}

void Calculator::timing_totals(bool reset, double *transition_ms,
			       double *prune_ms, uint64_t *proposals)
{
	DeviceGuard g(device_);
	// harvest in recording order
	const uint64_t first = ring_next_ > kRing ? ring_next_ - kRing : 0;
	for (uint64_t i = first; i < ring_next_; ++i) {
		TimingSlot &s = ring_[i % kRing];
		if (s.pending)
			harvest(s);
	}
	*transition_ms = acc_transition_ms_;
	*prune_ms = acc_prune_ms_;
	*proposals = acc_count_;
	if (reset) {
		acc_transition_ms_ = acc_prune_ms_ = 0.0;
		acc_count_ = 0;
	}
}

void Calculator::span_begin()
{
	DeviceGuard g(device_);
	check_cuda(cudaEventRecord(ev_span0_, stream_), "event");
}

float Calculator::span_end()
{
	DeviceGuard g(device_);
	check_cuda(cudaEventRecord(ev_span1_, stream_), "event");
	check_cuda(cudaEventSynchronize(ev_span1_), "sync");
	float ms = 0.0f;
	check_cuda(cudaEventElapsedTime(&ms, ev_span0_, ev_span1_), "elapsed");
	return ms;
}

uint32_t Calculator::autotune(const uint32_t *internals,
			      const uint32_t *children, uint32_t n,
			      const double *lengths, double clock_rate)
{
	DeviceGuard g(device_);
	if (!f32_)
		return 0;
	const bool timing = timing_;
	timing_ = true; // the trials read the kernel timings
	struct Restore {
		bool &flag;
		bool value;
		~Restore() { flag = value; }
	} restore{timing_, timing};
	// best of three timed evaluations after one warm-up, each rejected
	auto trial = [&]() {
		float best = INFINITY;
		for (int r = 0; r < 4; ++r) {
			propose_lengths(internals, children, n, lengths, clock_rate);
			(void)log_likelihood();
			float t = 0.0f, p = 0.0f;
			last_timing(&t, &p);
			reject();
			if (r > 0)
				best = std::min(best, t + p);
		}
		return best;
	};
	if (S_ == 20) {
		if (!d_tc_tab_) // built without tensor-core buffers
			return 0;
		// tensor cores with one and with two thread groups per CTA
		// (unless B3G_TC20_GROUPS fixed it), then the CUDA-core walk
		use_tc20_ = true;
		float tc = INFINITY;
		uint32_t best_groups = tc20_groups_;
		for (const uint32_t gr : {1u, 2u}) {
			if (tc20_groups_fixed_ && gr != tc20_groups_)
				continue;
			tc20_groups_ = gr;
			const float t = trial();
			if (t < tc) {
				tc = t;
				best_groups = gr;
			}
		}
		tc20_groups_ = best_groups;
		use_tc20_ = false;
		const float cc = trial();
		use_tc20_ = tc <= cc;
		return use_tc20_ ? 1u : 0u;
	}
	// the direct launch of short lists and path-like lists do not use the
	// tuned tile
	if (!use_runs_ || (use_direct_ && n <= kDirectMax))
		return runs_tile_;
	// (patterns per tile, threads per block).  Two pattern columns of one
	// category per thread: a warp spans 32 / (tile / 2) categories, so
	// tiles of 16 and 32 patterns put four and two categories in a warp
	// (and give small alignments more blocks), 64 and 128 one.
	uint32_t best_tile = runs_tile_, best_block = runs_block_;
	float best_ms = INFINITY;
	const uint32_t cand[][2] = {{16, 512},  {32, 512},  {64, 512},
				    {128, 512}, {32, 1024}, {64, 1024}};
	for (const auto &tb : cand) {
		const uint32_t t = tb[0], b = tb[1];
		if (t * C_ > 512 || (b == 1024 && t * C_ >= 512))
			continue;
		runs_tile_ = t;
		runs_block_ = b;
		const float ms = trial();
		if (ms < best_ms) {
			best_ms = ms;
			best_tile = t;
			best_block = b;
		}
	}
	runs_tile_ = best_tile;
	runs_block_ = best_block;
	return best_tile;
}

void Calculator::accept()
{
	outstanding_ = false;
	// Cpu4Calculator::accept (cpu4.rs:78-83): EditBuf::accept
	for (auto &m : selectors_)
		m &= 1u;
}

void Calculator::reject()
{
	outstanding_ = false;
	// Cpu4Calculator::reject (cpu4.rs:85-89): EditBuf::reject
	for (auto &m : selectors_)
		m = static_cast<uint8_t>((m ^ (m >> 1)) & 1u);
}

void Calculator::set_weights(const uint32_t *w)
{
	DeviceGuard g(device_);
	if (!w)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null weights");
	std::vector<uint32_t> padded(ldp_, 0);
	std::memcpy(padded.data(), w, P_ * sizeof(uint32_t));
	check_cuda(cudaStreamSynchronize(stream_), "sync");
	upload_pending_ = false;
	in_flight_ = 0;
	check_cuda(cudaMemcpy(d_weights_, padded.data(), ldp_ * sizeof(uint32_t),
			      cudaMemcpyHostToDevice),
		   "upload weights");
}

void Calculator::set_eigen(const double *V, const double *Vinv,
			   const double *lambda, const double *Q,
			   const double *pi, int shortcuts)
{
	DeviceGuard g(device_);
	if (!V || !Vinv || !lambda || !Q || !pi)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null eigensystem");
	const uint32_t nn = S_ * S_;
	for (uint32_t k = 0; k < nn; ++k)
		if (!std::isfinite(V[k]) || !std::isfinite(Vinv[k]) ||
		    !std::isfinite(Q[k]))
			throw Error(B3G_ERR_NUMERIC, "non-finite eigensystem");
	for (uint32_t k = 0; k < S_; ++k)
		if (!std::isfinite(lambda[k]) || !std::isfinite(pi[k]))
			throw Error(B3G_ERR_NUMERIC, "non-finite eigensystem");
	std::memcpy(model_host_.V, V, nn * sizeof(double));
	std::memcpy(model_host_.Vinv, Vinv, nn * sizeof(double));
	std::memcpy(model_host_.Q, Q, nn * sizeof(double));
	std::memcpy(model_host_.lambda, lambda, S_ * sizeof(double));
	std::memcpy(model_host_.pi, pi, S_ * sizeof(double));
	model_host_.shortcuts = shortcuts ? 1u : 0u;
	upload_model();
	model_set_ = true;
}

void Calculator::set_reversible(const double *rates, const double *pi,
				int shortcuts)
{
	DeviceGuard g(device_);
	if (!rates || !pi)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null model");
	const uint32_t nr = S_ * (S_ - 1) / 2;
	double psum = 0.0;
	for (uint32_t k = 0; k < nr; ++k)
		if (!std::isfinite(rates[k]) || rates[k] < 0.0)
			throw Error(B3G_ERR_NUMERIC,
				    "exchangeabilities must be finite and >= 0");
	for (uint32_t k = 0; k < S_; ++k) {
		if (!std::isfinite(pi[k]) || !(pi[k] > 0.0))
			throw Error(B3G_ERR_NUMERIC,
				    "frequencies must be finite and > 0");
		psum += pi[k];
	}
	(void)psum;
	// decomposed on the host in FP64: a one-block Jacobi kernel measured
	// about 410 us per model on this GPU (its FP64 pipe issues at 1/64 of
	// the FP32 rate), the host takes a few microseconds
	const int sweeps = reversible_eigen((int)S_, rates, pi, model_host_.V,
					    model_host_.Vinv, model_host_.lambda,
					    model_host_.Q);
	if (sweeps < 0)
		throw Error(B3G_ERR_NUMERIC,
			    "eigen decomposition of Q did not converge");
	std::memcpy(model_host_.pi, pi, S_ * sizeof(double));
	model_host_.shortcuts = shortcuts ? 1u : 0u;
	upload_model();
	model_set_ = true;
}

void Calculator::set_category_rates(const double *rates)
{
	DeviceGuard g(device_);
	if (!rates)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null rates");
	for (uint32_t c = 0; c < C_; ++c)
		if (!std::isfinite(rates[c]) || rates[c] < 0.0)
			throw Error(B3G_ERR_NUMERIC, "bad category rate");
	// update only the category rates of the device model in place
	std::memcpy(model_host_.cat_rates, rates, C_ * sizeof(double));
	check_cuda(cudaEventSynchronize(ev_model_free_), "model staging");
	std::memcpy(h_model_->cat_rates, rates, C_ * sizeof(double));
	check_cuda(cudaMemcpyAsync(d_model_->cat_rates, h_model_->cat_rates,
				   C_ * sizeof(double), cudaMemcpyHostToDevice,
				   stream_),
		   "upload category rates");
	check_cuda(cudaEventRecord(ev_model_free_, stream_), "event");
	stream_dirty_ = true;
}

void Calculator::set_gamma(double alpha)
{
	if (!std::isfinite(alpha) || !(alpha > 0.0))
		throw Error(B3G_ERR_NUMERIC, "alpha must be finite and > 0");
	std::vector<double> r(C_);
	gamma_categories(alpha, static_cast<int>(C_), r.data());
	set_category_rates(r.data());
}

} // namespace b3g

// ===========================================================================
// C ABI

namespace {

thread_local std::string g_last_error;

template <typename F> b3g_status guarded(F &&f)
{
	try {
		f();
		g_last_error.clear();
		return B3G_OK;
	} catch (const b3g::Error &e) {
		g_last_error = e.what();
		return e.status;
	} catch (const std::bad_alloc &) {
		g_last_error = "host allocation failed";
		return B3G_ERR_OUT_OF_MEMORY;
	} catch (const std::exception &e) {
		g_last_error = e.what();
		return B3G_ERR_STATE;
	} catch (...) {
		g_last_error = "unknown error";
		return B3G_ERR_STATE;
	}
}

b3g::Calculator *calc_of(b3g_calculator *c)
{
	if (!c)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null calculator");
	return reinterpret_cast<b3g::Calculator *>(c);
}

} // namespace

namespace b3g {

// Records the outcome of an entry point defined in another translation unit
// in the per-thread message that b3g_last_error() returns.
void set_last_error(const char *message)
{
	g_last_error = message ? message : "";
}

} // namespace b3g

extern "C" {

B3G_API const char *b3g_last_error(void) { return g_last_error.c_str(); }

B3G_API const char *b3g_version(void) { return "b3g 0.1.0 sm_103a"; }

B3G_API b3g_status b3g_calculator_create(const b3g_config *config,
					 const uint8_t *samples,
					 b3g_calculator **out)
{
	return guarded([&] {
		if (!config || !out)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null argument");
		*out = nullptr;
		auto *c = new b3g::Calculator(*config, samples);
		*out = reinterpret_cast<b3g_calculator *>(c);
	});
}

B3G_API void b3g_calculator_destroy(b3g_calculator *calc)
{
	delete reinterpret_cast<b3g::Calculator *>(calc);
}

B3G_API uint32_t b3g_calculator_num_patterns(const b3g_calculator *calc)
{
	return calc ? reinterpret_cast<const b3g::Calculator *>(calc)->num_patterns()
		    : 0u;
}

B3G_API b3g_status b3g_calculator_propose(b3g_calculator *calc,
					  const uint32_t *internals,
					  const uint32_t *children, uint32_t n,
					  const double *matrices,
					  const double *frequencies)
{
	return guarded([&] {
		calc_of(calc)->propose_matrices(internals, children, n, matrices,
						frequencies);
	});
}

B3G_API b3g_status b3g_calculator_likelihoods(b3g_calculator *calc,
					      double *out)
{
	return guarded([&] { calc_of(calc)->likelihoods(out); });
}

B3G_API b3g_status b3g_calculator_accept(b3g_calculator *calc)
{
	return guarded([&] { calc_of(calc)->accept(); });
}

B3G_API b3g_status b3g_calculator_reject(b3g_calculator *calc)
{
	return guarded([&] { calc_of(calc)->reject(); });
}

B3G_API b3g_status b3g_calculator_set_weights(b3g_calculator *calc,
					      const uint32_t *weights)
{
	return guarded([&] { calc_of(calc)->set_weights(weights); });
}

B3G_API b3g_status b3g_calculator_set_eigen(b3g_calculator *calc,
					    const double *V,
					    const double *Vinv,
					    const double *lambda,
					    const double *Q,
					    const double *frequencies,
					    int shortcuts)
{
	return guarded([&] {
		calc_of(calc)->set_eigen(V, Vinv, lambda, Q, frequencies,
					 shortcuts);
	});
}

B3G_API b3g_status b3g_calculator_set_reversible(b3g_calculator *calc,
						 const double *rates,
						 const double *frequencies,
						 int shortcuts)
{
	return guarded([&] {
		calc_of(calc)->set_reversible(rates, frequencies, shortcuts);
	});
}

B3G_API b3g_status b3g_calculator_set_category_rates(b3g_calculator *calc,
						     const double *rates)
{
	return guarded([&] { calc_of(calc)->set_category_rates(rates); });
}

B3G_API b3g_status b3g_calculator_set_gamma(b3g_calculator *calc,
					    double alpha)
{
	return guarded([&] { calc_of(calc)->set_gamma(alpha); });
}

B3G_API b3g_status b3g_calculator_propose_lengths(b3g_calculator *calc,
						  const uint32_t *internals,
						  const uint32_t *children,
						  uint32_t n,
						  const double *lengths,
						  double clock_rate)
{
	return guarded([&] {
		calc_of(calc)->propose_lengths(internals, children, n, lengths,
					       clock_rate);
	});
}

B3G_API b3g_status b3g_calculator_log_likelihood(b3g_calculator *calc,
						 double *out)
{
	return guarded([&] {
		if (!out)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*out = calc_of(calc)->log_likelihood();
	});
}

B3G_API b3g_status b3g_calculator_site_log_likelihoods(b3g_calculator *calc,
						       double *out)
{
	return guarded([&] { calc_of(calc)->site_log_likelihoods(out); });
}

B3G_API b3g_status b3g_calculator_set_timing(b3g_calculator *calc, int on)
{
	return guarded([&] { calc_of(calc)->set_timing(on != 0); });
}

B3G_API b3g_status b3g_calculator_last_timing(b3g_calculator *calc,
					      float *transition_ms,
					      float *prune_ms)
{
	return guarded([&] {
		if (!transition_ms || !prune_ms)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		calc_of(calc)->last_timing(transition_ms, prune_ms);
	});
}

B3G_API b3g_status b3g_calculator_timing_totals(b3g_calculator *calc,
						int reset,
						double *transition_ms,
						double *prune_ms,
						uint64_t *proposals)
{
	return guarded([&] {
		if (!transition_ms || !prune_ms || !proposals)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		calc_of(calc)->timing_totals(reset != 0, transition_ms, prune_ms,
					     proposals);
	});
}

B3G_API b3g_status b3g_calculator_last_upload_bytes(b3g_calculator *calc,
						    uint64_t *bytes)
{
	return guarded([&] {
		if (!bytes)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*bytes = calc_of(calc)->last_upload_bytes();
	});
}

B3G_API b3g_status b3g_calculator_last_launches(b3g_calculator *calc,
						uint32_t *kernels)
{
	return guarded([&] {
		if (!kernels)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*kernels = calc_of(calc)->last_launches();
	});
}

B3G_API b3g_status b3g_calculator_span_begin(b3g_calculator *calc)
{
	return guarded([&] { calc_of(calc)->span_begin(); });
}

B3G_API b3g_status b3g_calculator_span_end(b3g_calculator *calc, float *ms)
{
	return guarded([&] {
		if (!ms)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*ms = calc_of(calc)->span_end();
	});
}

B3G_API b3g_status b3g_calculator_autotune(b3g_calculator *calc,
					   const uint32_t *internals,
					   const uint32_t *children, uint32_t n,
					   const double *lengths,
					   double clock_rate, uint32_t *choice)
{
	return guarded([&] {
		if (!choice)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*choice = calc_of(calc)->autotune(internals, children, n, lengths,
						  clock_rate);
	});
}

} // extern "C"
