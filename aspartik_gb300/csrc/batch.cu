// batch.cu -- many calculators (chains) evaluated by one launch, replayed
// as a CUDA graph.
//
// Every member keeps its own device store.  A step is: each member stages
// its dirty list and edge lengths (b3g_calculator_stage_lengths, host only)
// into its slice of one contiguous pinned block, then b3g_batch_run replays
// one graph: one copy of that block, the run walk for the members with long
// lists (one batched transition-table kernel, one persistent pruning kernel
// over their pattern tiles, handed out by an atomic work counter, costliest
// member first), one persistent short-list kernel per category count for the
// members with short lists (their tables built in shared memory, a serial
// walk per column), and the read-back of every member's log-likelihood.
#include "batch.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

namespace b3g {

void set_last_error(const char *message);

Batch::Batch(Calculator *const *members, uint32_t count)
{
	if (!members || count < 1 || count > 256)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "a batch holds 1..256 calculators");
	members_.assign(members, members + count);
	for (Calculator *c : members_) {
		if (!c)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "null member");
		if (!c->f32_ || !c->use_runs_)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "batch members must use the FP32 chosen form");
		if (c->in_batch_)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "a calculator is already in a batch");
		if (c->device_ != members_[0]->device_)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "batch members must share one device");
	}
	for (size_t i = 0; i < members_.size(); ++i)
		for (size_t j = i + 1; j < members_.size(); ++j)
			if (members_[i] == members_[j])
				throw Error(B3G_ERR_INVALID_ARGUMENT,
					    "a calculator appears twice");
	device_ = members_[0]->device_;
	check_cuda(cudaSetDevice(device_), "cudaSetDevice");
	const uint32_t M = count;
	// costliest first: internals x patterns x categories
	order_.resize(M);
	std::iota(order_.begin(), order_.end(), 0u);
	std::stable_sort(order_.begin(), order_.end(), [&](uint32_t a, uint32_t b) {
		const Calculator *x = members_[a], *y = members_[b];
		return (uint64_t)x->I_ * x->ldp_ * x->C_ > (uint64_t)y->I_ * y->ldp_ * y->C_;
	});
	try {
		check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking),
			   "stream");
		check_cuda(cudaStreamCreateWithFlags(&stream2_, cudaStreamNonBlocking),
			   "stream");
		check_cuda(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming), "event");
		check_cuda(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming), "event");
		check_cuda(cudaEventCreate(&ev0_), "event");
		check_cuda(cudaEventCreate(&ev1_), "event");
		check_cuda(cudaMalloc(&d_desc_, sizeof(MemberDesc) * M), "descriptors");
		check_cuda(cudaMalloc(&d_steps_, sizeof(MemberStep) * M), "steps");
		check_cuda(cudaHostAlloc((void **)&h_steps_, sizeof(MemberStep) * M,
					 cudaHostAllocDefault),
			   "pinned steps");
		check_cuda(cudaMalloc(&d_lnl_, sizeof(double) * M), "lnl");
		check_cuda(cudaHostAlloc((void **)&h_lnl_, sizeof(double) * M,
					 cudaHostAllocDefault),
			   "pinned lnl");
		check_cuda(cudaMalloc(&d_work_, 4 * sizeof(unsigned)), "work counters");
		// one sum per tile of a member, for tiles as small as 16 patterns
		// (whatever tile the member's autotuner picks later)
		size_t total_tiles = 0;
		for (Calculator *c : members_)
			total_tiles += c->ldp_ / 16;
		check_cuda(cudaMalloc(&d_tile_sums_, sizeof(double) * total_tiles),
			   "tile sums");
		check_cuda(cudaMalloc(&d_tickets_, sizeof(unsigned) * M), "tickets");
		check_cuda(cudaMemset(d_tickets_, 0, sizeof(unsigned) * M), "tickets");

		std::vector<MemberDesc> desc(M);
		size_t tile_off = 0;
		uint32_t max_ops = 0, max_tips = 0, max_cols = 0;
		bool narrow = true;
		for (uint32_t k = 0; k < M; ++k) {
			Calculator *c = members_[order_[k]];
			MemberDesc &d = desc[k];
			d.tips = c->d_tips_;
			d.partials = static_cast<float *>(c->d_partials_);
			d.scales = c->d_scales_;
			d.ptab = static_cast<float *>(c->d_ptab_);
			d.stage = nullptr; // set to the member's slice below
			d.model = c->d_model_;
			d.weights = c->d_weights_;
			d.site_lnl = c->d_site_;
			d.tile_sums = d_tile_sums_ + tile_off;
			d.ticket = d_tickets_ + k;
			d.off_pi = (uint32_t)c->off_pi_;
			d.off_runs = (uint32_t)c->off_runs_;
			d.off_in = (uint32_t)c->off_in_;
			d.ldp = c->ldp_;
			d.C = c->C_;
			d.L = c->L_;
			d.tile = c->runs_tile_;
			d.log_inv_c = std::log(1.0 / static_cast<double>(c->C_));
			tile_off += c->ldp_ / 16;
			max_ops = std::max<uint32_t>(
				max_ops, c->I_ * sizeof(NodeOp) +
						 ((c->I_ + 4) & ~3u) * sizeof(uint32_t));
			// a step may use tiles of up to 128 patterns (pick_tile); a
			// tile's columns never exceed one 512-thread block
			max_tips = std::max<uint32_t>(max_tips, c->L_ * 128u);
			max_cols = 512u;
			max_entries_ = std::max<uint32_t>(max_entries_, c->I_ * 2 * c->C_);
			if ((uint64_t)c->L_ * 2 * c->C_ * c->ldp_ >= (1ull << 31))
				narrow = false;
			if (c->C_ == 1 || c->C_ == 2 || c->C_ == 4)
				direct_c_[c->C_] = true;
		}
		// the members' staging slices: each member's layout up to the end
		// of its edge lengths (lengths-mode proposals only while batched)
		std::vector<size_t> slice(M);
		for (uint32_t k = 0; k < M; ++k) {
			const Calculator *c = members_[order_[k]];
			slice[k] = block_bytes_;
			block_bytes_ += (c->off_in_ + (size_t)c->I_ * 2 * sizeof(double) + 255) &
					~(size_t)255;
		}
		check_cuda(cudaHostAlloc((void **)&h_block_, block_bytes_, cudaHostAllocDefault),
			   "pinned staging block");
		check_cuda(cudaMalloc(&d_block_, block_bytes_), "staging block");
		for (uint32_t k = 0; k < M; ++k) {
			Calculator *c = members_[order_[k]];
			// the member's own last launch must be done with its buffer
			c->wait_stage();
			check_cuda(cudaStreamSynchronize(c->stream_), "member stream");
			c->own_h_stage_ = c->h_stage_;
			c->own_d_stage_ = c->d_stage_;
			c->h_stage_ = h_block_ + slice[k];
			c->d_stage_ = d_block_ + slice[k];
			desc[k].stage = c->d_stage_;
			c->in_batch_ = true;
		}
		check_cuda(cudaMemcpy(d_desc_, desc.data(), sizeof(MemberDesc) * M,
				      cudaMemcpyHostToDevice),
			   "upload descriptors");
		bp_.members = d_desc_;
		bp_.steps = d_steps_;
		bp_.lnl_out = d_lnl_;
		bp_.work_next = d_work_;
		bp_.num_members = M;
		bp_.smem_ops_bytes = (max_ops + 15u) & ~15u;
		bp_.smem_tips_bytes = std::min<uint32_t>(max_tips, 32u * 1024u);
		bp_.max_cols = max_cols;
		bp_.smem_ptab_bytes = kPtabSmemBytes;
		bp_.narrow = narrow ? 1u : 0u;
		ctas_ = 2 * members_[0]->num_sms_;
		evaluated_.assign(M, 0);

		// capture one step as a graph
		check_cuda(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal),
			   "begin capture");
		// external event-record nodes: the events are recorded each time
		// the graph runs and can be waited on outside it
		check_cuda(cudaEventRecordWithFlags(ev0_, stream_,
						    cudaEventRecordExternal),
			   "event");
		check_cuda(cudaMemcpyAsync(d_steps_, h_steps_, sizeof(MemberStep) * M,
					   cudaMemcpyHostToDevice, stream_),
			   "steps copy");
		check_cuda(cudaMemcpyAsync(d_block_, h_block_, block_bytes_,
					   cudaMemcpyHostToDevice, stream_),
			   "staging block copy");
		check_cuda(cudaMemsetAsync(d_work_, 0, 4 * sizeof(unsigned), stream_),
			   "work counters");
		// two branches: the run walk of long lists on this stream, the
		// short-list kernels on the second, joined before the read-back
		check_cuda(cudaEventRecord(ev_fork_, stream_), "fork");
		check_cuda(cudaStreamWaitEvent(stream2_, ev_fork_, 0), "fork");
		check_cuda(launch_ptab4_batch(bp_, max_entries_, stream_),
			   "batched transition kernel");
		check_cuda(launch_prune4_batch(bp_, ctas_, stream_),
			   "batched pruning kernel");
		for (uint32_t C : {4u, 2u, 1u})
			if (direct_c_[C])
				check_cuda(launch_prune4_direct_batch(
						   bp_, C, (8u / C) * members_[0]->num_sms_, stream2_),
					   "batched short-list kernel");
		check_cuda(cudaEventRecord(ev_join_, stream2_), "join");
		check_cuda(cudaStreamWaitEvent(stream_, ev_join_, 0), "join");
		check_cuda(cudaMemcpyAsync(h_lnl_, d_lnl_, sizeof(double) * M,
					   cudaMemcpyDeviceToHost, stream_),
			   "lnl copy");
		check_cuda(cudaEventRecordWithFlags(ev1_, stream_,
						    cudaEventRecordExternal),
			   "event");
		check_cuda(cudaStreamEndCapture(stream_, &graph_), "end capture");
		check_cuda(cudaGraphInstantiate(&exec_, graph_, 0), "instantiate");
	} catch (...) {
		release();
		throw;
	}
}

Batch::~Batch() { release(); }

void Batch::release()
{
	if (device_ >= 0)
		cudaSetDevice(device_);
	if (stream_)
		cudaStreamSynchronize(stream_);
	for (Calculator *c : members_) {
		if (c && c->own_h_stage_ &&
		    c->h_stage_ >= h_block_ && c->h_stage_ < h_block_ + block_bytes_) {
			// the member's own launches may still read the lent slice
			c->wait_stage();
			if (c->stream_)
				cudaStreamSynchronize(c->stream_);
			c->h_stage_ = c->own_h_stage_;
			c->d_stage_ = c->own_d_stage_;
			c->own_h_stage_ = nullptr;
			c->own_d_stage_ = nullptr;
			c->in_batch_ = false;
			c->staged_ = false;
		}
		if (c && c->batch_done_ == ev1_) {
			c->batch_done_ = nullptr;
			c->in_batch_ = false;
			c->staged_ = false;
		}
	}
	cudaFreeHost(h_block_);
	cudaFree(d_block_);
	h_block_ = nullptr;
	d_block_ = nullptr;
	if (exec_)
		cudaGraphExecDestroy(exec_);
	if (graph_)
		cudaGraphDestroy(graph_);
	cudaFree(d_desc_);
	cudaFree(d_steps_);
	cudaFreeHost(h_steps_);
	cudaFree(d_lnl_);
	cudaFreeHost(h_lnl_);
	cudaFree(d_work_);
	cudaFree(d_tile_sums_);
	cudaFree(d_tickets_);
	if (ev0_)
		cudaEventDestroy(ev0_);
	if (ev1_)
		cudaEventDestroy(ev1_);
	if (ev_fork_)
		cudaEventDestroy(ev_fork_);
	if (ev_join_)
		cudaEventDestroy(ev_join_);
	if (stream_)
		cudaStreamDestroy(stream_);
	if (stream2_)
		cudaStreamDestroy(stream2_);
	ev_fork_ = ev_join_ = nullptr;
	stream2_ = nullptr;
	exec_ = nullptr;
	graph_ = nullptr;
	d_desc_ = nullptr;
	d_steps_ = h_steps_ = nullptr;
	d_lnl_ = h_lnl_ = nullptr;
	d_work_ = nullptr;
	d_tile_sums_ = nullptr;
	d_tickets_ = nullptr;
	ev0_ = ev1_ = nullptr;
	stream_ = nullptr;
}

void Batch::run()
{
	check_cuda(cudaSetDevice(device_), "cudaSetDevice");
	// the previous replay reads h_steps_: it must be done
	if (ran_)
		check_cuda(cudaEventSynchronize(ev1_), "previous batch");
	const uint32_t M = (uint32_t)members_.size();
	for (uint32_t k = 0; k < M; ++k) {
		Calculator *c = members_[order_[k]];
		MemberStep &s = h_steps_[k];
		evaluated_[order_[k]] = c->staged_ ? 1 : 0;
		if (c->staged_) {
			// the member's own last launch must not still read its tables
			c->wait_stage();
			s.n = c->staged_n_;
			s.n_runs = c->n_runs_;
			s.tile = c->staged_tile_;
			s.tips_smem = c->staged_tips_smem_;
			s.clock_rate = c->staged_clock_;
			s.direct = (c->staged_n_ <= kDirectMax &&
				    (c->C_ == 1 || c->C_ == 2 || c->C_ == 4))
					   ? 1u
					   : 0u;
			c->staged_ = false;
		} else {
			s.n = 0;
			s.n_runs = 0;
			s.tile = c->runs_tile_;
			s.tips_smem = 0;
			s.direct = 0;
			s.clock_rate = 1.0;
		}
	}
	// members' own streams may still hold model uploads or eigen kernels
	for (Calculator *c : members_)
		if (c->stream_dirty_) {
			check_cuda(cudaStreamSynchronize(c->stream_), "member stream");
			c->stream_dirty_ = false;
		}
	check_cuda(cudaGraphLaunch(exec_, stream_), "graph launch");
	if (!ran_) // from now on members wait for the replay before restaging
		for (Calculator *c : members_)
			c->batch_done_ = ev1_;
	ran_ = true;
}

void Batch::log_likelihoods(double *out)
{
	if (!out)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null output");
	if (!ran_)
		throw Error(B3G_ERR_STATE, "the batch has not run");
	check_cuda(cudaSetDevice(device_), "cudaSetDevice");
	check_cuda(cudaEventSynchronize(ev1_), "batch");
	const uint32_t M = (uint32_t)members_.size();
	for (uint32_t k = 0; k < M; ++k) {
		const uint32_t m = order_[k];
		out[m] = evaluated_[m] ? h_lnl_[k] : NAN;
	}
}

float Batch::last_ms()
{
	if (!ran_)
		throw Error(B3G_ERR_STATE, "the batch has not run");
	check_cuda(cudaEventSynchronize(ev1_), "batch");
	float ms = 0.0f;
	check_cuda(cudaEventElapsedTime(&ms, ev0_, ev1_), "elapsed");
	return ms;
}

} // namespace b3g

// ===========================================================================

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
	}
}

b3g::Batch *batch_of(b3g_batch *b)
{
	if (!b)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null batch");
	return reinterpret_cast<b3g::Batch *>(b);
}

} // namespace

extern "C" {

B3G_API b3g_status b3g_batch_create(b3g_calculator *const *members,
				    uint32_t count, b3g_batch **out)
{
	return guarded([&] {
		if (!out)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*out = nullptr;
		auto *b = new b3g::Batch(
			reinterpret_cast<b3g::Calculator *const *>(members), count);
		*out = reinterpret_cast<b3g_batch *>(b);
	});
}

B3G_API void b3g_batch_destroy(b3g_batch *batch)
{
	delete reinterpret_cast<b3g::Batch *>(batch);
}

B3G_API b3g_status b3g_calculator_stage_lengths(b3g_calculator *calc,
						const uint32_t *internals,
						const uint32_t *children,
						uint32_t n,
						const double *lengths,
						double clock_rate)
{
	return guarded([&] {
		if (!calc)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null calculator");
		reinterpret_cast<b3g::Calculator *>(calc)->stage_lengths(
			internals, children, n, lengths, clock_rate);
	});
}

B3G_API b3g_status b3g_batch_run(b3g_batch *batch)
{
	return guarded([&] { batch_of(batch)->run(); });
}

B3G_API b3g_status b3g_batch_log_likelihoods(b3g_batch *batch, double *out)
{
	return guarded([&] { batch_of(batch)->log_likelihoods(out); });
}

B3G_API b3g_status b3g_batch_last_ms(b3g_batch *batch, float *ms)
{
	return guarded([&] {
		if (!ms)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*ms = batch_of(batch)->last_ms();
	});
}

} // extern "C"
