// dedup.cu -- site-pattern compression on the device.
//
// Restates deduplicate (crates/b3/src/likelihood/mod.rs:74-132): the unique
// columns of an alignment in first-occurrence order, how many sites each
// pattern stands for, and the pattern of every site; gaps (code 0) become
// 0b1111 for DNA (mod.rs:117-122).  The reference hashes columns with
// blake3 into a host map; here the work is integer and byte traffic over
// the alignment, laid out for the GPU:
//
//   1. one thread per site hashes its column (32-bit FNV-1a); adjacent
//      threads read adjacent bytes of every row, so each row is read
//      coalesced;
//   2. an open-addressing table of 64-bit keys (hash << 32 | site): one CAS
//      publishes a hash together with the site that represents it, so a
//      later site with the same hash compares its column byte by byte with
//      that representative (equal hashes of different columns probe on);
//      atomicMin keeps each slot's first site;
//   3. a site is a pattern's first occurrence when its slot's first site is
//      itself; an exclusive scan of those flags numbers the patterns in
//      first-occurrence order;
//   4. every site looks up its pattern, weights are counted with integer
//      atomics, and the pattern columns are gathered into the leaf-major
//      output.
// Every output depends only on the alignment, not on thread timing.
#include "../../include/b3g.h"
#include "calculator.hpp"

#include <cstring>
#include <new>
#include <string>

namespace b3g {

void set_last_error(const char *message);

namespace {

constexpr unsigned long long kEmptyKey = ~0ull;
constexpr uint32_t kScanBlock = 1024; // elements per scan block (256 x 4)

__global__ void hash_kernel(const uint8_t *__restrict__ msa, uint32_t L, uint32_t N,
			    uint32_t *__restrict__ hash)
{
	const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
	if (s >= N)
		return;
	uint32_t h = 2166136261u;
	for (uint32_t l = 0; l < L; ++l) {
		h ^= msa[(size_t)l * N + s];
		h *= 16777619u;
	}
	hash[s] = h;
}

__device__ bool same_column(const uint8_t *__restrict__ msa, uint32_t L, uint32_t N,
			    uint32_t a, uint32_t b)
{
	for (uint32_t l = 0; l < L; ++l)
		if (msa[(size_t)l * N + a] != msa[(size_t)l * N + b])
			return false;
	return true;
}

__global__ void insert_kernel(const uint8_t *__restrict__ msa, uint32_t L, uint32_t N,
			      const uint32_t *__restrict__ hash,
			      unsigned long long *keys, uint32_t *first, uint32_t mask,
			      uint32_t *__restrict__ slot_of_site, unsigned *status)
{
	const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
	if (s >= N)
		return;
	const uint32_t h = hash[s];
	const unsigned long long mine = ((unsigned long long)h << 32) | s;
	uint32_t slot = (h * 0x9E3779B1u) & mask;
	// the table holds at least 2N slots, so a free one exists; the loop
	// is bounded by the table size all the same
	for (uint32_t probe = 0; probe <= mask; ++probe) {
		unsigned long long cur = keys[slot];
		if (cur == kEmptyKey) {
			const unsigned long long prev = atomicCAS(keys + slot, kEmptyKey, mine);
			if (prev == kEmptyKey) {
				atomicMin(first + slot, s);
				slot_of_site[s] = slot;
				return;
			}
			cur = prev;
		}
		if ((uint32_t)(cur >> 32) == h &&
		    same_column(msa, L, N, (uint32_t)(cur & 0xFFFFFFFFu), s)) {
			atomicMin(first + slot, s);
			slot_of_site[s] = slot;
			return;
		}
		slot = (slot + 1) & mask;
	}
	atomicExch(status, 1u);
}

__global__ void first_flag_kernel(const uint32_t *__restrict__ first,
				  const uint32_t *__restrict__ slot_of_site, uint32_t N,
				  uint32_t *__restrict__ flag)
{
	const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
	if (s < N)
		flag[s] = first[slot_of_site[s]] == s ? 1u : 0u;
}

// Exclusive scan within blocks of kScanBlock elements (256 threads x 4);
// each block's total goes to sums[block].
__global__ void __launch_bounds__(256) scan_blocks_kernel(const uint32_t *__restrict__ in,
							  uint32_t n, uint32_t *__restrict__ out,
							  uint32_t *__restrict__ sums)
{
	__shared__ uint32_t s_warp[8];
	const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
	const uint32_t base = blockIdx.x * kScanBlock + 4 * t;
	uint32_t v[4], run = 0;
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		v[k] = base + k < n ? in[base + k] : 0u;
		run += v[k];
	}
	uint32_t incl = run; // inclusive scan of the per-thread totals
	for (int off = 1; off < 32; off <<= 1) {
		const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
		if (lane >= (uint32_t)off)
			incl += y;
	}
	if (lane == 31)
		s_warp[warp] = incl;
	__syncthreads();
	uint32_t warp_base = 0;
	for (uint32_t w = 0; w < warp; ++w)
		warp_base += s_warp[w];
	uint32_t acc = warp_base + incl - run;
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		if (base + k < n)
			out[base + k] = acc;
		acc += v[k];
	}
	if (t == 255)
		sums[blockIdx.x] = warp_base + incl;
}

// Exclusive scan of the block totals in place by one block (chunks of
// kScanBlock with a carry); total[0] = sum of all.
__global__ void __launch_bounds__(256) scan_sums_kernel(uint32_t *sums, uint32_t n,
							uint32_t *total)
{
	__shared__ uint32_t s_warp[8];
	__shared__ uint32_t s_carry;
	const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
	if (t == 0)
		s_carry = 0;
	__syncthreads();
	for (uint32_t chunk = 0; chunk < n; chunk += kScanBlock) {
		const uint32_t base = chunk + 4 * t;
		uint32_t v[4], run = 0;
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			v[k] = base + k < n ? sums[base + k] : 0u;
			run += v[k];
		}
		uint32_t incl = run;
		for (int off = 1; off < 32; off <<= 1) {
			const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
			if (lane >= (uint32_t)off)
				incl += y;
		}
		if (lane == 31)
			s_warp[warp] = incl;
		__syncthreads();
		uint32_t warp_base = 0, chunk_total = 0;
		for (uint32_t w = 0; w < 8; ++w) {
			if (w < warp)
				warp_base += s_warp[w];
			chunk_total += s_warp[w];
		}
		uint32_t acc = s_carry + warp_base + incl - run;
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			if (base + k < n)
				sums[base + k] = acc;
			acc += v[k];
		}
		__syncthreads();
		if (t == 0)
			s_carry += chunk_total;
		__syncthreads();
	}
	if (t == 0)
		*total = s_carry;
}

__global__ void add_block_base_kernel(uint32_t *__restrict__ idx, uint32_t n,
				      const uint32_t *__restrict__ sums)
{
	const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n)
		idx[i] += sums[i / kScanBlock];
}

__global__ void assign_kernel(const uint32_t *__restrict__ first,
			      const uint32_t *__restrict__ slot_of_site,
			      const uint32_t *__restrict__ idx, uint32_t N,
			      uint32_t *__restrict__ site_to_pattern, uint32_t *weights,
			      uint32_t *__restrict__ site_of_pattern)
{
	const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
	if (s >= N)
		return;
	const uint32_t f = first[slot_of_site[s]];
	const uint32_t p = idx[f];
	site_to_pattern[s] = p;
	atomicAdd(weights + p, 1u);
	if (f == s)
		site_of_pattern[p] = s;
}

// leaves[l][p] = msa[l][first site of p]; one thread per (pattern, leaf),
// patterns fastest so writes are coalesced.
__global__ void gather_kernel(const uint8_t *__restrict__ msa, uint32_t L, uint32_t N,
			      uint32_t P, const uint32_t *__restrict__ site_of_pattern,
			      int dna_gaps, uint8_t *__restrict__ leaves)
{
	const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
	if (p >= P)
		return;
	const uint32_t site = site_of_pattern[p];
	for (uint32_t l = blockIdx.y; l < L; l += gridDim.y) {
		const uint8_t v = msa[(size_t)l * N + site];
		leaves[(size_t)l * P + p] = (dna_gaps && v == 0) ? (uint8_t)0x0F : v;
	}
}

template <typename T> void dalloc(T *&p, size_t bytes, const char *what)
{
	if (cudaMalloc((void **)&p, bytes ? bytes : 1) != cudaSuccess) {
		p = nullptr;
		throw Error(B3G_ERR_OUT_OF_MEMORY, std::string("device allocation: ") + what);
	}
}

} // namespace

uint32_t deduplicate_device(const uint8_t *msa, uint32_t L, uint32_t N, int dna_gaps,
			    int device, uint8_t *leaves, uint32_t *weights,
			    uint32_t *site_to_pattern, float *device_ms)
{
	if (!msa || !leaves || !weights || !site_to_pattern)
		throw Error(B3G_ERR_INVALID_ARGUMENT, "null buffer");
	if (L < 1 || N < 1 || N > (1u << 28))
		throw Error(B3G_ERR_INVALID_ARGUMENT, "alignment size out of range");
	int prev = -1;
	check_cuda(cudaGetDevice(&prev), "cudaGetDevice");
	check_cuda(cudaSetDevice(device), "cudaSetDevice");
	uint32_t cap = 1;
	while (cap < 2 * N)
		cap <<= 1;
	const uint32_t nblk = (N + kScanBlock - 1) / kScanBlock;
	uint8_t *d_msa = nullptr, *d_leaves = nullptr;
	uint32_t *d_hash = nullptr, *d_first = nullptr, *d_slot = nullptr, *d_flag = nullptr,
		 *d_idx = nullptr, *d_sums = nullptr, *d_total = nullptr, *d_s2p = nullptr,
		 *d_w = nullptr, *d_sop = nullptr;
	unsigned long long *d_keys = nullptr;
	unsigned *d_status = nullptr;
	cudaStream_t st = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	uint32_t P = 0;
	auto cleanup = [&] {
		if (st)
			cudaStreamSynchronize(st);
		cudaFree(d_msa);
		cudaFree(d_leaves);
		cudaFree(d_hash);
		cudaFree(d_first);
		cudaFree(d_slot);
		cudaFree(d_flag);
		cudaFree(d_idx);
		cudaFree(d_sums);
		cudaFree(d_total);
		cudaFree(d_s2p);
		cudaFree(d_w);
		cudaFree(d_sop);
		cudaFree(d_keys);
		cudaFree(d_status);
		if (e0)
			cudaEventDestroy(e0);
		if (e1)
			cudaEventDestroy(e1);
		if (st)
			cudaStreamDestroy(st);
		if (prev >= 0)
			cudaSetDevice(prev);
	};
	try {
		const size_t bytes = (size_t)L * N;
		check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
		check_cuda(cudaEventCreate(&e0), "event");
		check_cuda(cudaEventCreate(&e1), "event");
		dalloc(d_msa, bytes, "alignment");
		dalloc(d_leaves, bytes, "patterns");
		dalloc(d_hash, N * sizeof(uint32_t), "hashes");
		dalloc(d_keys, (size_t)cap * sizeof(unsigned long long), "table");
		dalloc(d_first, (size_t)cap * sizeof(uint32_t), "first sites");
		dalloc(d_slot, N * sizeof(uint32_t), "slots");
		dalloc(d_flag, N * sizeof(uint32_t), "flags");
		dalloc(d_idx, N * sizeof(uint32_t), "indices");
		dalloc(d_sums, nblk * sizeof(uint32_t), "block sums");
		dalloc(d_total, sizeof(uint32_t), "total");
		dalloc(d_s2p, N * sizeof(uint32_t), "site patterns");
		dalloc(d_w, N * sizeof(uint32_t), "weights");
		dalloc(d_sop, N * sizeof(uint32_t), "pattern sites");
		dalloc(d_status, sizeof(unsigned), "status");
		check_cuda(cudaMemcpyAsync(d_msa, msa, bytes, cudaMemcpyHostToDevice, st),
			   "upload alignment");
		check_cuda(cudaEventRecord(e0, st), "event");
		check_cuda(cudaMemsetAsync(d_keys, 0xFF, (size_t)cap * sizeof(unsigned long long),
					   st),
			   "clear table");
		check_cuda(cudaMemsetAsync(d_first, 0xFF, (size_t)cap * sizeof(uint32_t), st),
			   "clear first sites");
		check_cuda(cudaMemsetAsync(d_w, 0, N * sizeof(uint32_t), st), "clear weights");
		check_cuda(cudaMemsetAsync(d_status, 0, sizeof(unsigned), st), "clear status");
		const uint32_t tb = 256, gb = (N + tb - 1) / tb;
		hash_kernel<<<gb, tb, 0, st>>>(d_msa, L, N, d_hash);
		insert_kernel<<<gb, tb, 0, st>>>(d_msa, L, N, d_hash, d_keys, d_first, cap - 1,
						 d_slot, d_status);
		first_flag_kernel<<<gb, tb, 0, st>>>(d_first, d_slot, N, d_flag);
		scan_blocks_kernel<<<nblk, 256, 0, st>>>(d_flag, N, d_idx, d_sums);
		scan_sums_kernel<<<1, 256, 0, st>>>(d_sums, nblk, d_total);
		add_block_base_kernel<<<gb, tb, 0, st>>>(d_idx, N, d_sums);
		assign_kernel<<<gb, tb, 0, st>>>(d_first, d_slot, d_idx, N, d_s2p, d_w, d_sop);
		check_cuda(cudaGetLastError(), "dedup kernels");
		check_cuda(cudaMemcpyAsync(&P, d_total, sizeof(uint32_t), cudaMemcpyDeviceToHost,
					   st),
			   "read pattern count");
		unsigned status = 0;
		check_cuda(cudaMemcpyAsync(&status, d_status, sizeof(unsigned),
					   cudaMemcpyDeviceToHost, st),
			   "read status");
		check_cuda(cudaStreamSynchronize(st), "sync");
		if (status)
			throw Error(B3G_ERR_STATE, "pattern table overflow");
		gather_kernel<<<dim3((P + tb - 1) / tb, L < 65535u ? L : 65535u), tb, 0, st>>>(
			d_msa, L, N, P, d_sop, dna_gaps, d_leaves);
		check_cuda(cudaGetLastError(), "gather kernel");
		check_cuda(cudaEventRecord(e1, st), "event");
		check_cuda(cudaMemcpyAsync(leaves, d_leaves, (size_t)L * P, cudaMemcpyDeviceToHost,
					   st),
			   "read patterns");
		check_cuda(cudaMemcpyAsync(weights, d_w, P * sizeof(uint32_t),
					   cudaMemcpyDeviceToHost, st),
			   "read weights");
		check_cuda(cudaMemcpyAsync(site_to_pattern, d_s2p, N * sizeof(uint32_t),
					   cudaMemcpyDeviceToHost, st),
			   "read site patterns");
		check_cuda(cudaStreamSynchronize(st), "sync");
		if (device_ms)
			check_cuda(cudaEventElapsedTime(device_ms, e0, e1), "elapsed");
	} catch (...) {
		cleanup();
		throw;
	}
	cleanup();
	return P;
}

} // namespace b3g

// ===========================================================================

extern "C" {

B3G_API b3g_status b3g_deduplicate(const uint8_t *msa, uint32_t num_sequences,
				   uint32_t num_sites, int dna_gaps, int32_t device,
				   uint8_t *leaves, uint32_t *weights,
				   uint32_t *site_to_pattern, uint32_t *num_patterns,
				   float *device_ms)
{
	try {
		if (!num_patterns)
			throw b3g::Error(B3G_ERR_INVALID_ARGUMENT, "null output");
		*num_patterns = b3g::deduplicate_device(msa, num_sequences, num_sites, dna_gaps,
							device, leaves, weights, site_to_pattern,
							device_ms);
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

} // extern "C"
