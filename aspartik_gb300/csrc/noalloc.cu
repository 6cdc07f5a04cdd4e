// noalloc.cu -- b3g_prune_noalloc: the pruning kernel on caller-owned device
// buffers, with its only working memory in a fixed array compiled into the
// library, so that the call allocates nothing.  The rules (size limit,
// first-call set-up, shared array, overlapping calls) are stated beside the
// declaration in include/b3g.h.
#include "../../include/b3g.h"
#include "b3g_device.cuh"

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

namespace b3g {
void set_last_error(const char *message);
}

namespace {

static_assert(sizeof(b3g_node_op) == sizeof(b3g::NodeOp),
	      "b3g_node_op and NodeOp must share one layout");
static_assert(B3G_TIP == b3g::kTipBit, "tip marker");

constexpr size_t kTicketBytes = 256; // counter, padded to keep sums aligned
constexpr size_t kScratchBytes =
	kTicketBytes + size_t(B3G_NOALLOC_MAX_BLOCKS) * sizeof(double);

// [0, 4): completion counter of the last-block fold; [256, ...): one block
// sum per thread block.  Zero-initialised when the module loads.
static __device__ __align__(256) unsigned char g_prune_scratch[kScratchBytes];

constexpr int kMaxDevices = 128;
std::mutex g_scratch_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_prune_scratch on `dev`, which must be current.  The
// host-side symbol is only a stand-in and is never passed to a kernel.
b3g_status scratch_address(int dev, void **out, std::string &err)
{
	std::lock_guard<std::mutex> lock(g_scratch_mu);
	if (!g_scratch_addr[dev]) {
		void *p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_prune_scratch);
		if (e != cudaSuccess || !p) {
			err = std::string("cudaGetSymbolAddress: ") +
			      cudaGetErrorString(e);
			return B3G_ERR_CUDA;
		}
		g_scratch_addr[dev] = p;
	}
	*out = g_scratch_addr[dev];
	return B3G_OK;
}

b3g_status fail(b3g_status s, const std::string &msg)
{
	b3g::set_last_error(msg.c_str());
	return s;
}

} // namespace

extern "C" B3G_API b3g_status b3g_prune_noalloc(const b3g_prune_buffers *b,
						 void *stream)
{
	if (!b)
		return fail(B3G_ERR_INVALID_ARGUMENT, "null buffers");
	if (!b->tips || !b->partials || !b->scales || !b->ops || !b->tables ||
	    !b->frequencies || !b->weights || !b->site_lnl || !b->lnl)
		return fail(B3G_ERR_INVALID_ARGUMENT, "null device pointer");
	if (b->reserved != 0)
		return fail(B3G_ERR_INVALID_ARGUMENT, "reserved must be 0");
	if (b->n < 1)
		return fail(B3G_ERR_INVALID_ARGUMENT, "n must be >= 1");
	if (b->ldp == 0 || b->ldp % b3g::kPatternAlign != 0)
		return fail(B3G_ERR_INVALID_ARGUMENT,
			    "ldp must be a positive multiple of 128");
	if (b->num_categories < 1 ||
	    b->num_categories > (uint32_t)b3g::kMaxCategories)
		return fail(B3G_ERR_INVALID_ARGUMENT,
			    "num_categories must be in 1..16");
	if (b->precision != B3G_PRECISION_F64 &&
	    b->precision != B3G_PRECISION_F32)
		return fail(B3G_ERR_INVALID_ARGUMENT, "unknown precision");
	const uint32_t C = b->num_categories;
	const uint32_t tile = C <= 1 ? 128u : C == 2 ? 64u : 32u;
	const uint32_t blocks = b->ldp / tile;
	if (blocks > B3G_NOALLOC_MAX_BLOCKS)
		return fail(B3G_ERR_INVALID_ARGUMENT,
			    "problem exceeds the allocation-free maximum of " +
				    std::to_string(B3G_NOALLOC_MAX_BLOCKS) +
				    " thread blocks (" + std::to_string(blocks) +
				    " needed)");

	int dev = -1;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess)
		return fail(B3G_ERR_CUDA,
			    std::string("cudaGetDevice: ") + cudaGetErrorString(e));
	if (dev < 0 || dev >= kMaxDevices)
		return fail(B3G_ERR_INVALID_ARGUMENT, "device ordinal too large");
	void *scratch = nullptr;
	std::string err;
	const b3g_status st = scratch_address(dev, &scratch, err);
	if (st != B3G_OK)
		return fail(st, err);

	cudaStream_t s = static_cast<cudaStream_t>(stream);
	unsigned *ticket = static_cast<unsigned *>(scratch);
	double *block_sums = reinterpret_cast<double *>(
		static_cast<unsigned char *>(scratch) + kTicketBytes);
	// the fold's counter must start at zero
	e = cudaMemsetAsync(ticket, 0, sizeof(unsigned), s);
	if (e != cudaSuccess)
		return fail(B3G_ERR_CUDA,
			    std::string("clear counter: ") + cudaGetErrorString(e));

	b3g::PruneParams pp{};
	pp.tips = b->tips;
	pp.partials = b->partials;
	pp.scales = b->scales;
	pp.ops = reinterpret_cast<const b3g::NodeOp *>(b->ops);
	pp.ptab = b->tables;
	pp.pi = b->frequencies;
	pp.weights = b->weights;
	pp.site_lnl = b->site_lnl;
	pp.cat_lnl = nullptr;
	pp.block_sums = block_sums;
	pp.ticket = ticket;
	pp.lnl_out = b->lnl;
	pp.n = b->n;
	pp.ldp = b->ldp;
	pp.C = C;
	pp.scale_ln = b->scale_ln;
	pp.scale_threshold = std::exp(-static_cast<double>(b->scale_ln));
	pp.scale_mult = std::exp(static_cast<double>(b->scale_ln));
	pp.log_inv_c = std::log(1.0 / static_cast<double>(C));
	// the slot ids index buffers of unknown size: 64-bit element indices
	pp.wide_index = b3g::noalloc_narrow_index(C, b->ldp) ? 0u : 1u;
	e = b3g::launch_prune4(pp, b->precision == B3G_PRECISION_F32, tile, s);
	if (e != cudaSuccess)
		return fail(B3G_ERR_CUDA,
			    std::string("pruning kernel: ") + cudaGetErrorString(e));
	b3g::set_last_error("");
	return B3G_OK;
}
