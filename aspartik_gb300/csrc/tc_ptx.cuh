// tc_ptx.cuh -- inline-PTX wrappers for the Blackwell tensor-core path
// (tcgen05 MMA with accumulators in tensor memory, mbarriers, descriptors).
//
// Operand layout used throughout: K-major, no swizzle.  A "core matrix" is
// 8 rows x 16 bytes stored contiguously (row r at +16 r); along K the core
// matrices of one MMA are LBO bytes apart, along M (or N) consecutive
// groups of 8 rows are SBO bytes apart.
#pragma once

#include <stdint.h>

namespace b3g {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
	return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (sm_100 family): start address, leading
// (K) and stride (M/N) byte offsets, all >> 4; version 1 at bits 46-47;
// base offset 0, relative LBO, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo,
					      uint32_t sbo)
{
	uint64_t d = 0;
	d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
	d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
	d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
	d |= (uint64_t)1 << 46;
	return d;
}

// Instruction descriptor of kind::tf32 with FP32 accumulation, both
// operands K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(uint32_t M, uint32_t N)
{
	return (1u << 4)            // D format: F32
	       | (2u << 7)          // A format: TF32
	       | (2u << 10)         // B format: TF32
	       | ((N >> 3) << 17)   // N / 8
	       | ((M >> 4) << 24);  // M / 16
}

// Tensor memory: allocation by one warp (all lanes), address written to
// shared memory.  ncols is a power of two >= 32.
__device__ __forceinline__ void tmem_alloc(uint32_t holder_saddr, uint32_t ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
		     ::"r"(holder_saddr), "r"(ncols)
		     : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
			     : "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr),
		     "r"(ncols)
		     : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]; issued by one thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc,
					 uint64_t bdesc, uint32_t idesc,
					 uint32_t accumulate)
{
	asm volatile("{\n\t.reg .pred p;\n\t"
		     "setp.ne.b32 p, %4, 0;\n\t"
		     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
		     ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
		     : "memory");
}

// Arrive once on the mbarrier when every MMA issued so far has completed.
__device__ __forceinline__ void mma_commit(uint32_t mbar_saddr)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
		     ::"r"(mbar_saddr)
		     : "memory");
}

__device__ __forceinline__ void fence_before_sync()
{
	asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync()
{
	asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes visible to the tensor core's reads.
__device__ __forceinline__ void fence_proxy_async_smem()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar_saddr, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar_saddr),
		     "r"(count)
		     : "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Wait for the phase with the given parity to complete, at most `limit`
// polls.  Returns false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar_saddr, uint32_t parity,
					  uint32_t limit)
{
	for (uint32_t k = 0; k < limit; ++k) {
		uint32_t ok;
		asm volatile("{\n\t.reg .pred p;\n\t"
			     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			     "selp.u32 %0, 1, 0, p;\n\t}"
			     : "=r"(ok)
			     : "r"(mbar_saddr), "r"(parity)
			     : "memory");
		if (ok)
			return true;
	}
	return false;
}

// Arm the mbarrier for one phase: one arrival that also expects `bytes`
// of asynchronous copies to complete on it.
__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar_saddr, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar_saddr),
		     "r"(bytes)
		     : "memory");
}

// Bulk copy (no tensor map) of `bytes` from global to this CTA's shared
// memory, completing on the mbarrier.  Both addresses 16-byte aligned,
// bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst_saddr, const void *src, uint32_t bytes,
					 uint32_t mbar_saddr)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
		     "[%0], [%1], %2, [%3];" ::"r"(dst_saddr),
		     "l"(src), "r"(bytes), "r"(mbar_saddr)
		     : "memory");
}

// Generic-proxy global writes ordered before later asynchronous-proxy
// (bulk copy) reads of them.
__device__ __forceinline__ void fence_proxy_async_global()
{
	asm volatile("fence.proxy.async.global;" ::: "memory");
}

// 32 lanes x 16 consecutive 32-bit columns: this thread's lane, columns
// taddr .. taddr + 15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
	uint32_t r[16];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
		     "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
		     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
		       "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
		       "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
		       "=r"(r[15])
		     : "r"(taddr));
#pragma unroll
	for (int i = 0; i < 16; i++)
		v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float v[4])
{
	uint32_t r[4];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
		     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
		     : "r"(taddr));
#pragma unroll
	for (int i = 0; i < 4; i++)
		v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld()
{
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Round to the nearest TF32 value (10 mantissa bits; low 13 bits zero).
__device__ __forceinline__ float round_tf32(float x)
{
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	return __uint_as_float(r);
}

// Split x into a TF32 head and a TF32 tail, both rounded to nearest so that
// what the tensor core reads is exactly what was stored and the rounding
// error of the tail is unbiased: x = hi + lo + O(2^-22 |x|).
__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo)
{
	hi = round_tf32(x);
	lo = round_tf32(x - hi);
}

} // namespace tc
} // namespace b3g
