// prune20tc.cuh -- 20-state pruning on the tensor cores (FP32 chosen form).
// Included by kernels4.cu inside its anonymous namespace after prune20.cuh
// (uses rescale_pow2_20, load20/store20 and block_fold).
//
// An internal child's contribution for a tile of 128 patterns and one
// category is a small GEMM: out[p][i] = sum_k x[p][k] P[i][k], M = 128
// patterns, N = 20 states (padded to 32), K = 20 (padded to 24).  It runs as
// tcgen05 MMAs of kind::tf32 with FP32 accumulation in tensor memory, in the
// 3xTF32 split form: x = x_hi + x_lo, P = P_hi + P_lo (TF32 heads and
// tails, each rounded to nearest) and out = x_hi P_hi + x_hi P_lo +
// x_lo P_hi, which keeps FP32-level accuracy without a bias.  The algorithmic flops are
// 2 S^2 per internal child and (pattern, category); the tensor core
// executes 3 x (32/20) x (24/20) times that.
//
// Work: one CTA per (pattern tile, category), 128 threads, thread p owns
// pattern p of the tile (tensor-memory lane p).  The CTA walks the whole
// children-first list; per entry the threads stage the internal children's
// partials (split) and the two tables' operand blocks in shared memory,
// thread 0 issues the MMAs and commits them to an mbarrier, and after the
// wait every thread reads its row of each product from tensor memory,
// multiplies the two children (a tip child is a table-row lookup),
// renormalises by a power of two and stores the partial.  The root's
// pi . x and exponent go to per-category buffers; finish20_kernel mixes the
// categories and folds the weighted sum.
//
// Shared-memory operand layout: K-major, no swizzle, core matrices of 8
// rows x 16 bytes; element (row, k) at (row / 8) * 768 + (k / 4) * 128 +
// (row % 8) * 16 + (k % 4) * 4 bytes: LBO = 128 (next 4 k), SBO = 768
// (next 8 rows).  A block: 128 rows x 24 k (12,288 B); B block: 32 rows x
// 24 k (3,072 B).

constexpr uint32_t kTcRows = 128;           // patterns per tile (M)
constexpr uint32_t kTcN = 32;               // states padded (N)
constexpr uint32_t kTcK = 24;               // states padded (K)
constexpr uint32_t kTcA = kTcRows * kTcK;   // floats per A block
constexpr uint32_t kTcB = kTcN * kTcK;      // floats per B block (768)
constexpr uint32_t kTcSmem = 4 * kTcA * 4 + 4 * kTcB * 4; // 61,440 B
constexpr uint32_t kTcWaitLimit = 1u << 22; // polls, far beyond an MMA

__host__ __device__ __forceinline__ uint32_t tc_off(uint32_t row, uint32_t k)
{
	return (row >> 3) * 192u + (k >> 2) * 32u + (row & 7u) * 4u + (k & 3u);
}

// One block per table (entry, side, category), 768 threads: P in FP64 (as
// ptab20_kernel), then the FP32 tip rows [21][20] (transposed, ones row)
// and the hi/lo operand blocks B[i][k] = P[i][k] in the layout above.
__global__ void __launch_bounds__(768) ptab20tc_kernel(PtabParams prm, float *tc_tab)
{
	constexpr int S = kS20;
	const uint32_t id = blockIdx.x;
	const uint32_t c = id % prm.C, es = id / prm.C;
	const ModelDev *m = prm.model;
	const uint32_t t = threadIdx.x;
	__shared__ double e[S];
	__shared__ double Ps[S * S];
	double d = 0.0;
	if (!prm.matrices)
		d = prm.lengths[es] * (prm.clock_rate * m->cat_rates[c]);
	if (t < S)
		e[t] = exp(m->lambda[t] * d);
	__syncthreads();
	float *tip = (float *)prm.ptab + (size_t)id * (S + 1) * S;
	if (t < S * S) {
		const uint32_t i = t / S, j = t - i * S;
		double P;
		if (prm.matrices) {
			P = prm.matrices[(size_t)id * S * S + t];
		} else if (m->shortcuts && d > 20.0) {
			P = m->pi[j];
		} else if (m->shortcuts && d < 1e-10) {
			P = i == j ? 1.0 : m->Q[i * S + j] * d;
		} else {
			double s = 0.0;
			for (int k = 0; k < S; k++)
				s = fma(m->V[i * S + k] * e[k], m->Vinv[k * S + j], s);
			P = s;
		}
		Ps[t] = P;
		tip[j * S + i] = (float)P;
	} else if (t < S * S + S) {
		tip[S * S + (t - S * S)] = 1.0f;
	}
	__syncthreads();
	// operand element t of the 32 x 24 block
	const uint32_t g = t / 192u, rem = t - g * 192u;
	const uint32_t kc = rem / 32u, r = (rem % 32u) / 4u, q = t % 4u;
	const uint32_t i = 8 * g + r, k = 4 * kc + q;
	const double v = (i < (uint32_t)S && k < (uint32_t)S) ? Ps[i * S + k] : 0.0;
	const float hi = tc::round_tf32((float)v);
	const float lo = tc::round_tf32((float)(v - (double)hi));
	float *blk = tc_tab + (size_t)id * 2 * kTcB;
	blk[t] = hi;
	blk[kTcB + t] = lo;
}

template <typename Idx>
__global__ void __launch_bounds__(128) prune20tc_kernel(Tc20Params prm)
{
	constexpr int S = kS20;
	extern __shared__ uint8_t tc_smem_raw[];
	float *sA = reinterpret_cast<float *>(((uintptr_t)tc_smem_raw + 1023) &
					      ~(uintptr_t)1023);
	float *sB = sA + 4 * kTcA; // [side][hi, lo][768]
	// then the list (when it fits) and the tile's tip codes
	NodeOp *sOps = reinterpret_cast<NodeOp *>(sB + 4 * kTcB);
	uint8_t *sTips = reinterpret_cast<uint8_t *>(sOps + (prm.ops_smem ? prm.n : 0));
	__shared__ __align__(8) uint64_t mbar;
	__shared__ uint32_t holder;
	const uint32_t t = threadIdx.x, warp = t >> 5;
	const uint32_t c = blockIdx.y, C = prm.C;
	const uint32_t p = blockIdx.x * kTcRows + t;
	const Idx stride = (Idx)C * prm.ldp;
	const Idx col = (Idx)c * prm.ldp + p;
	const uint32_t mb = tc::smem_u32(&mbar);
	for (uint32_t k = t; prm.ops_smem && k < prm.n; k += 128)
		sOps[k] = prm.ops[k];
	if (prm.tips_smem) {
		// 4-byte loads: the tile's 128 codes of every leaf
		uint32_t *s32 = reinterpret_cast<uint32_t *>(sTips);
		for (uint32_t k = t; k < prm.L * 32u; k += 128) {
			const uint32_t leaf = k >> 5, w4 = k & 31u;
			s32[k] = *reinterpret_cast<const uint32_t *>(
				prm.tips + (size_t)leaf * prm.ldp + blockIdx.x * kTcRows + 4 * w4);
		}
	}
	const NodeOp *ops = prm.ops_smem ? sOps : prm.ops;

	// K padding (k = 20..23) of the four A blocks stays zero
#pragma unroll
	for (uint32_t b = 0; b < 4; b++)
		*reinterpret_cast<float4 *>(sA + b * kTcA + tc_off(t, 20)) =
			make_float4(0.f, 0.f, 0.f, 0.f);
	if (t == 0)
		tc::mbar_init(mb, 1);
	if (warp == 0)
		tc::tmem_alloc(tc::smem_u32(&holder), 64);
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = holder;
	const uint32_t lane_base = (32u * warp) << 16;
	constexpr uint32_t idesc = tc::idesc_tf32(kTcRows, kTcN);
	// operand descriptors of K step 0: [child][hi, lo]
	uint64_t dA[2][2], dB[2][2];
#pragma unroll
	for (uint32_t j = 0; j < 2; j++)
#pragma unroll
		for (uint32_t h = 0; h < 2; h++) {
			dA[j][h] = tc::smem_desc(tc::smem_u32(sA + (2 * j + h) * kTcA), 128, 768);
			dB[j][h] = tc::smem_desc(tc::smem_u32(sB + (2 * j + h) * kTcB), 128, 768);
		}

	// Inputs of one entry, fetched into registers ahead of their use: for
	// an internal side the child's partial row, scale and this side's
	// operand blocks (three float4 per thread); for a tip side the table
	// row of the tip's code.
	struct Inputs {
		float x[2][S];
		float4 b[2][3];
		int32_t sc[2];
	};
	auto fetch = [&](uint32_t e, Inputs &in) {
		const NodeOp op = ops[e];
		const uint32_t ids[2] = {op.left, op.right};
#pragma unroll
		for (uint32_t j = 0; j < 2; j++) {
			const size_t tid_tab = (size_t)(2 * e + j) * C + c;
			if (ids[j] & kTipBit) {
				const uint32_t leaf = ids[j] & ~kTipBit;
				const uint8_t code =
					prm.tips_smem ? sTips[leaf * kTcRows + t]
						      : prm.tips[(size_t)leaf * prm.ldp + p];
				load20<true>(prm.tab + (tid_tab * (S + 1) + code) * S, in.x[j]);
				in.sc[j] = 0;
			} else {
				const Idx ix = (Idx)ids[j] * stride + col;
				load20<false>(prm.partials + (size_t)ix * S, in.x[j]);
				in.sc[j] = prm.scales[ix];
				const float4 *src = reinterpret_cast<const float4 *>(
					prm.tc_tab + tid_tab * 2 * kTcB);
#pragma unroll
				for (uint32_t q = 0; q < 3; q++)
					in.b[j][q] = __ldg(src + t + 128 * q);
			}
		}
	};

	float y[S];
#pragma unroll
	for (int i = 0; i < S; i++)
		y[i] = 0.f;
	int32_t cnt = 0;
	uint32_t phase = 0;
	bool failed = false;
	Inputs cur, nxt;
	if (prm.n)
		fetch(0, cur);
	for (uint32_t e = 0; e < prm.n; ++e) {
		const NodeOp op = ops[e];
		const uint32_t ids[2] = {op.left, op.right};
		const bool any = !(ids[0] & kTipBit) || !(ids[1] & kTipBit);
		// stage the internal sides: split partials, operand blocks
#pragma unroll
		for (uint32_t j = 0; j < 2; j++) {
			if (ids[j] & kTipBit)
				continue;
			float *ah = sA + (2 * j) * kTcA, *al = ah + kTcA;
#pragma unroll
			for (uint32_t q = 0; q < 5; q++) {
				float h[4], l[4];
#pragma unroll
				for (int u = 0; u < 4; u++)
					tc::split_tf32(cur.x[j][4 * q + u], h[u], l[u]);
				*reinterpret_cast<float4 *>(ah + tc_off(t, 4 * q)) =
					make_float4(h[0], h[1], h[2], h[3]);
				*reinterpret_cast<float4 *>(al + tc_off(t, 4 * q)) =
					make_float4(l[0], l[1], l[2], l[3]);
			}
			float4 *dst = reinterpret_cast<float4 *>(sB + j * 2 * kTcB);
#pragma unroll
			for (uint32_t q = 0; q < 3; q++)
				dst[t + 128 * q] = cur.b[j][q];
		}
		if (any) {
			tc::fence_proxy_async_smem();
			tc::fence_before_sync();
			__syncthreads();
			tc::fence_after_sync();
			if (t == 0) {
#pragma unroll
				for (uint32_t j = 0; j < 2; j++) {
					if (ids[j] & kTipBit)
						continue;
					// the start address sits in the low bits (>> 4):
					// the next K step (+256 B) adds 16
#pragma unroll
					for (uint32_t s = 0; s < 3; s++) {
						// x_hi P_hi, x_hi P_lo, x_lo P_hi
						tc::mma_tf32(tmem + 32 * j, dA[j][0] + 16 * s,
							     dB[j][0] + 16 * s, idesc, s != 0);
						tc::mma_tf32(tmem + 32 * j, dA[j][0] + 16 * s,
							     dB[j][1] + 16 * s, idesc, 1);
						tc::mma_tf32(tmem + 32 * j, dA[j][1] + 16 * s,
							     dB[j][0] + 16 * s, idesc, 1);
					}
				}
				tc::mma_commit(mb);
			}
		}
		// the next entry's inputs travel while the MMAs run, unless that
		// entry reads this one's output (fetched after the store below)
		const bool more = e + 1 < prm.n;
		bool next_dep = false;
		if (more) {
			const NodeOp nop = ops[e + 1];
			next_dep = nop.left == op.out || nop.right == op.out;
			if (!next_dep)
				fetch(e + 1, nxt);
		}
		float ab[2][S];
		if (any) {
			const bool ok = tc::mbar_wait(mb, phase, kTcWaitLimit);
			phase ^= 1u;
			if (__syncthreads_or(!ok)) {
				failed = true;
				break;
			}
			tc::fence_after_sync();
#pragma unroll
			for (uint32_t j = 0; j < 2; j++) {
				if (ids[j] & kTipBit)
					continue;
				const uint32_t ta = tmem + lane_base + 32 * j;
				tc::tmem_ld16(ta, ab[j]);
				tc::tmem_ld4(ta + 16, ab[j] + 16);
			}
			tc::tmem_wait_ld();
		}
#pragma unroll
		for (uint32_t j = 0; j < 2; j++)
			if (ids[j] & kTipBit)
#pragma unroll
				for (int i = 0; i < S; i++)
					ab[j][i] = cur.x[j][i];
#pragma unroll
		for (int i = 0; i < S; i++)
			y[i] = ab[0][i] * ab[1][i];
		cnt = cur.sc[0] + cur.sc[1] + rescale_pow2_20(y);
		const Idx ox = (Idx)op.out * stride + col;
		store20(prm.partials + (size_t)ox * S, y);
		prm.scales[ox] = cnt;
		// the next entry overwrites shared memory and tensor memory
		tc::fence_before_sync();
		__syncthreads();
		if (more) {
			if (next_dep) // this thread's own row, stored just above
				fetch(e + 1, nxt);
			cur = nxt;
		}
	}
	if (failed) {
		if (t == 0)
			atomicExch(prm.status, 1u);
	} else {
		double dot = 0.0;
#pragma unroll
		for (int i = 0; i < S; i++)
			dot = fma(prm.pi[i], (double)y[i], dot);
		prm.root_val[(size_t)c * prm.ldp + p] = dot;
		prm.root_exp[(size_t)c * prm.ldp + p] = cnt;
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	if (warp == 0)
		tc::tmem_dealloc(tmem, 64);
}

// Category mixing of the root (FP32 form: values with power-of-two
// exponents, as the single-calculator walks), weights, block sums and the
// deterministic fold by the last block.  128 patterns per block.
__global__ void __launch_bounds__(128) finish20_kernel(Tc20Params prm)
{
	__shared__ double s_red[32];
	__shared__ unsigned s_last;
	const uint32_t t = threadIdx.x, p = blockIdx.x * 128 + t;
	const uint32_t C = prm.C, ldp = prm.ldp;
	int32_t emax = INT32_MIN;
	for (uint32_t k = 0; k < C; k++)
		if (prm.root_val[(size_t)k * ldp + p] > 0.0)
			emax = max(emax, prm.root_exp[(size_t)k * ldp + p]);
	double site;
	if (emax == INT32_MIN) {
		site = -INFINITY;
	} else {
		double acc = 0.0;
		for (uint32_t k = 0; k < C; k++)
			acc += scalbn(prm.root_val[(size_t)k * ldp + p],
				      prm.root_exp[(size_t)k * ldp + p] - emax);
		site = log(acc) + (double)emax * 0.69314718055994530942 + prm.log_inv_c;
	}
	prm.site_lnl[p] = site;
	if (prm.cat_lnl)
		for (uint32_t k = 0; k < C; k++)
			prm.cat_lnl[(size_t)k * ldp + p] =
				log(prm.root_val[(size_t)k * ldp + p]) +
				(double)prm.root_exp[(size_t)k * ldp + p] * 0.69314718055994530942;
	const uint32_t w = prm.weights[p];
	double contrib = w ? site * (double)w : 0.0;
	for (int off = 16; off > 0; off >>= 1)
		contrib += __shfl_down_sync(0xffffffffu, contrib, off);
	if ((t & 31u) == 0)
		s_red[t >> 5] = contrib;
	__syncthreads();
	if (t == 0) {
		prm.block_sums[blockIdx.x] = s_red[0] + s_red[1] + s_red[2] + s_red[3];
		__threadfence();
		s_last = atomicAdd(prm.ticket, 1u) == gridDim.x - 1u;
	}
	__syncthreads();
	if (!s_last)
		return;
	__threadfence();
	const double total = block_fold(prm.block_sums, gridDim.x, s_red);
	if (t == 0) {
		*prm.lnl_out = total;
		*prm.ticket = 0u;
	}
}
