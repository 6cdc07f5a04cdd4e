// hetero.cu -- per-pattern class mixture over several calculators: the
// device sum and the host bookkeeping (see hetero.hpp).
#include "hetero.hpp"

#include <cmath>
#include <cstring>
#include <new>

namespace b3g {

void set_last_error(const char *message);

namespace {

// sum_p w_p lnL_{c(p)}(p): one thread per pattern, warp shuffles and the
// warps in order per block, then the last block folds the block sums in a
// fixed pairwise order (the result does not depend on block timing).
__global__ void __launch_bounds__(128) hetero_sum_kernel(HeteroParams prm)
{
	__shared__ double s_red[4];
	__shared__ unsigned s_last;
	const uint32_t t = threadIdx.x, p = blockIdx.x * 128 + t;
	double contrib = 0.0;
	if (p < prm.num_patterns) {
		const uint32_t w = prm.weights[p];
		if (w)
			contrib = prm.site[prm.classes[p]][p] * (double)w;
	}
	for (int off = 16; off > 0; off >>= 1)
		contrib += __shfl_down_sync(0xffffffffu, contrib, off);
	if ((t & 31u) == 0)
		s_red[t >> 5] = contrib;
	__syncthreads();
	if (t == 0) {
		prm.block_sums[blockIdx.x] = (s_red[0] + s_red[1]) + (s_red[2] + s_red[3]);
		__threadfence();
		s_last = atomicAdd(prm.ticket, 1u) == gridDim.x - 1u;
	}
	__syncthreads();
	if (!s_last)
		return;
	__threadfence();
	double sum = 0.0;
	for (uint32_t k = t; k < gridDim.x; k += 128)
		sum += __ldcg(prm.block_sums + k);
	for (int off = 16; off > 0; off >>= 1)
		sum += __shfl_down_sync(0xffffffffu, sum, off);
	__syncthreads();
	if ((t & 31u) == 0)
		s_red[t >> 5] = sum;
	__syncthreads();
	if (t == 0) {
		*prm.lnl_out = (s_red[0] + s_red[1]) + (s_red[2] + s_red[3]);
		*prm.ticket = 0u;
	}
}

struct OnDevice {
	int prev = -1;
	explicit OnDevice(int dev)
	{
		check_cuda(cudaGetDevice(&prev), "cudaGetDevice");
		if (prev != dev)
			check_cuda(cudaSetDevice(dev), "cudaSetDevice");
	}
	~OnDevice()
	{
		int cur = -1;
		if (cudaGetDevice(&cur) == cudaSuccess && cur != prev && prev >= 0)
			cudaSetDevice(prev);
	}
};

template <typename T> void alloc(T *&p, size_t bytes, const char *what)
{
	if (cudaMalloc((void **)&p, bytes) != cudaSuccess) {
		p = nullptr;
		throw Error(B3G_ERR_OUT_OF_MEMORY, std::string("device allocation: ") + what);
	}
}

} // namespace

cudaError_t launch_hetero_sum(const HeteroParams &p, cudaStream_t s)
{
	const uint32_t blocks = (p.num_patterns + 127u) / 128u;
	hetero_sum_kernel<<<blocks, 128, 0, s>>>(p);
	return cudaGetLastError();
}

Hetero::Hetero(Calculator *const *members, uint32_t count)
{
	if (!members || count < 1 || count > kHeteroMaxClasses)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "a mixture holds 1..16 calculators");
	members_.assign(members, members + count);
	for (Calculator *c : members_) {
		if (!c)
			throw Error(B3G_ERR_INVALID_ARGUMENT, "null member");
		if (c->P_ != members_[0]->P_ || c->device_ != members_[0]->device_)
			throw Error(B3G_ERR_INVALID_ARGUMENT,
				    "mixture members must share the patterns and the device");
		if (!c->have_result_ || c->outstanding_)
			throw Error(B3G_ERR_STATE,
				    "evaluate and accept every member before building the mixture");
	}
	for (size_t i = 0; i < members_.size(); ++i)
		for (size_t j = i + 1; j < members_.size(); ++j)
			if (members_[i] == members_[j])
				throw Error(B3G_ERR_INVALID_ARGUMENT, "a calculator appears twice");
	P_ = members_[0]->P_;
	ldp_ = members_[0]->ldp_;
	device_ = members_[0]->device_;
	OnDevice g(device_);
	try {
		check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
		check_cuda(cudaEventCreateWithFlags(&ev_member_, cudaEventDisableTiming), "event");
		alloc(d_accepted_, (size_t)count * ldp_ * sizeof(double), "class values");
		alloc(d_classes_, 2 * (size_t)ldp_ * sizeof(uint32_t), "classes");
		alloc(d_block_sums_, (ldp_ / 128 + 1) * sizeof(double), "block sums");
		alloc(d_ticket_, sizeof(unsigned), "ticket");
		alloc(d_lnl_, sizeof(double), "lnl");
		check_cuda(cudaHostAlloc((void **)&h_classes_, ldp_ * sizeof(uint32_t),
					 cudaHostAllocDefault),
			   "pinned classes");
		check_cuda(cudaHostAlloc((void **)&h_lnl_, sizeof(double), cudaHostAllocDefault),
			   "pinned lnl");
		check_cuda(cudaMemsetAsync(d_ticket_, 0, sizeof(unsigned), stream_), "zero");
		check_cuda(cudaMemsetAsync(d_classes_, 0, 2 * (size_t)ldp_ * sizeof(uint32_t),
					   stream_),
			   "zero classes");
		// every class starts from its member's accepted per-pattern values
		for (uint32_t k = 0; k < count; ++k) {
			Calculator *c = members_[k];
			check_cuda(cudaMemcpyAsync(d_accepted_ + (size_t)k * ldp_, c->d_site_,
						   ldp_ * sizeof(double),
						   cudaMemcpyDeviceToDevice, c->stream_),
				   "copy class values");
			check_cuda(cudaEventRecord(ev_member_, c->stream_), "event");
			check_cuda(cudaStreamWaitEvent(stream_, ev_member_, 0), "wait");
		}
		check_cuda(cudaStreamSynchronize(stream_), "sync");
	} catch (...) {
		release();
		throw;
	}
}

Hetero::~Hetero() { release(); }

void Hetero::release()
{
	if (stream_)
		cudaStreamSynchronize(stream_);
	cudaFree(d_accepted_);
	cudaFree(d_classes_);
	cudaFree(d_block_sums_);
	cudaFree(d_ticket_);
	cudaFree(d_lnl_);
	if (h_classes_)
		cudaFreeHost(h_classes_);
	if (h_lnl_)
		cudaFreeHost(h_lnl_);
	if (ev_member_)
		cudaEventDestroy(ev_member_);
	if (stream_)
		cudaStreamDestroy(stream_);
	d_accepted_ = nullptr;
	d_classes_ = nullptr;
	d_block_sums_ = nullptr;
	d_ticket_ = nullptr;
	d_lnl_ = nullptr;
	h_classes_ = nullptr;
	h_lnl_ = nullptr;
	ev_member_ = nullptr;
	stream_ = nullptr;
}

void Hetero::set_classes(const uint32_t *classes)
{
	OnDevice g(device_);
	if (!classes)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null classes");
	for (uint32_t p = 0; p < P_; ++p)
		if (classes[p] >= members_.size())
			throw Error(B3G_ERR_INVALID_ARGUMENT, "class index out of range");
	// the previous upload from the staging buffer must have finished
	check_cuda(cudaStreamSynchronize(stream_), "sync");
	std::memcpy(h_classes_, classes, P_ * sizeof(uint32_t));
	std::memset(h_classes_ + P_, 0, (ldp_ - P_) * sizeof(uint32_t));
	check_cuda(cudaMemcpyAsync(d_classes_ + ldp_, h_classes_, ldp_ * sizeof(uint32_t),
				   cudaMemcpyHostToDevice, stream_),
		   "upload classes");
	classes_proposed_ = true;
}

double Hetero::log_likelihood()
{
	OnDevice g(device_);
	HeteroParams hp{};
	for (uint32_t k = 0; k < members_.size(); ++k) {
		Calculator *c = members_[k];
		if (c->outstanding_) {
			// the class was evaluated this step: its new values, once
			// its stream has produced them
			hp.site[k] = c->d_site_;
			check_cuda(cudaEventRecord(ev_member_, c->stream_), "event");
			check_cuda(cudaStreamWaitEvent(stream_, ev_member_, 0), "wait");
		} else {
			hp.site[k] = d_accepted_ + (size_t)k * ldp_;
		}
	}
	hp.classes = d_classes_ + (classes_proposed_ ? ldp_ : 0);
	hp.weights = members_[0]->d_weights_;
	hp.block_sums = d_block_sums_;
	hp.ticket = d_ticket_;
	hp.lnl_out = d_lnl_;
	hp.num_patterns = ldp_;
	hp.num_classes = (uint32_t)members_.size();
	check_cuda(launch_hetero_sum(hp, stream_), "mixture sum");
	check_cuda(cudaMemcpyAsync(h_lnl_, d_lnl_, sizeof(double), cudaMemcpyDeviceToHost,
				   stream_),
		   "read lnl");
	check_cuda(cudaStreamSynchronize(stream_), "sync");
	return *h_lnl_;
}

void Hetero::accept()
{
	OnDevice g(device_);
	for (uint32_t k = 0; k < members_.size(); ++k) {
		Calculator *c = members_[k];
		if (!c->outstanding_)
			continue;
		// on the member's stream: before its next evaluation overwrites
		// its per-pattern output
		check_cuda(cudaMemcpyAsync(d_accepted_ + (size_t)k * ldp_, c->d_site_,
					   ldp_ * sizeof(double), cudaMemcpyDeviceToDevice,
					   c->stream_),
			   "keep class values");
		check_cuda(cudaEventRecord(ev_member_, c->stream_), "event");
		check_cuda(cudaStreamWaitEvent(stream_, ev_member_, 0), "wait");
		c->accept();
	}
	if (classes_proposed_) {
		check_cuda(cudaMemcpyAsync(d_classes_, d_classes_ + ldp_, ldp_ * sizeof(uint32_t),
					   cudaMemcpyDeviceToDevice, stream_),
			   "keep classes");
		classes_proposed_ = false;
	}
}

void Hetero::reject()
{
	for (Calculator *c : members_)
		if (c->outstanding_)
			c->reject();
	classes_proposed_ = false;
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

b3g::Hetero *hetero_of(b3g_hetero *h)
{
	if (!h)
		throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null mixture");
	return reinterpret_cast<b3g::Hetero *>(h);
}

} // namespace

extern "C" {

B3G_API b3g_status b3g_hetero_create(b3g_calculator *const *members, uint32_t count,
				     b3g_hetero **out)
{
	return guarded([&] {
		if (!out)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*out = nullptr;
		auto *h = new b3g::Hetero(reinterpret_cast<b3g::Calculator *const *>(members),
					  count);
		*out = reinterpret_cast<b3g_hetero *>(h);
	});
}

B3G_API void b3g_hetero_destroy(b3g_hetero *h)
{
	delete reinterpret_cast<b3g::Hetero *>(h);
}

B3G_API b3g_status b3g_hetero_set_classes(b3g_hetero *h, const uint32_t *classes)
{
	return guarded([&] { hetero_of(h)->set_classes(classes); });
}

B3G_API b3g_status b3g_hetero_log_likelihood(b3g_hetero *h, double *out)
{
	return guarded([&] {
		if (!out)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*out = hetero_of(h)->log_likelihood();
	});
}

B3G_API b3g_status b3g_hetero_accept(b3g_hetero *h)
{
	return guarded([&] { hetero_of(h)->accept(); });
}

B3G_API b3g_status b3g_hetero_reject(b3g_hetero *h)
{
	return guarded([&] { hetero_of(h)->reject(); });
}

} // extern "C"
