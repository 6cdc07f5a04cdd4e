// prune20tc.cuh -- 20-state pruning on the tensor cores (FP32 chosen form).
// Included by kernels4.cu inside its anonymous namespace after prune20.cuh
// (uses rescale_pow2_20 and block_fold).
//
// An internal child's contribution for a tile of 128 patterns and one
// category is a small GEMM: out[p][i] = sum_k x[p][k] P[i][k], M = 128
// patterns, N = 20 states (padded to 32), K = 20 (padded to 24).  It runs as
// tcgen05 MMAs of kind::tf32 with FP32 accumulation in tensor memory, in the
// 3xTF32 split form: x = x_hi + x_lo, P = P_hi + P_lo (TF32 heads and
// tails, each rounded to nearest) and out = x_hi P_hi + x_hi P_lo +
// x_lo P_hi, which keeps FP32-level accuracy without a bias: per K step one
// N = 64 MMA x_hi [P_hi; P_lo] and one N = 32 MMA adding x_lo P_hi to the
// first half, the halves summed in the epilogue.  The algorithmic flops are
// 2 S^2 per internal child and (pattern, category); the tensor core
// executes 3 x (32/20) x (24/20) times that.
//
// Work: one cluster of K CTAs per (pattern tile, category), each CTA with kG
// groups of 128 threads; thread t of a group owns pattern t of the tile
// (tensor-memory lane t).  The list is walked run by run (NodeOp::pad =
// entries left in the run, so the entries of a run are mutually
// independent): group gg = rank kG + g of the cluster takes entries gg,
// gg + K kG, ... of each run, and the cluster synchronises between runs
// (partials written by one CTA are read by another's bulk copies in the
// next run).  K > 1 spreads a work item over several SMs when the grid has
// fewer items than CTA slots (K = 1: one CTA, a barrier of its own).
// Per entry a group stages its internal children's partials (split) and the
// two tables' operand blocks in its own shared memory, thread 0 of the group
// issues the MMAs into the group's tensor-memory columns and commits them to
// the group's mbarrier, and after the wait every thread reads its row of
// each product from tensor memory, multiplies the two children (a tip child
// is a table-row lookup), renormalises by a power of two and stores the
// partial.  Several groups (and CTAs) per SM keep the tensor pipe and the
// memory system busy while one entry's round trip is in flight.  The root's
// pi . x and exponent go to per-category buffers; finish20_kernel mixes the
// categories and folds the weighted sum.
//
// Shared-memory operand layout: K-major, no swizzle, core matrices of 8
// rows x 16 bytes.  B block (32 rows x 24 k, 3,072 B): element (row, k) at
// (row / 8) * 768 + (k / 4) * 128 + (row % 8) * 16 + (k % 4) * 4 bytes,
// LBO = 128 (next 4 k), SBO = 768 (next 8 rows); its K padding k = 20..23
// is zero.  A block (128 rows x 20 k, 10,240 B): the same with SBO = 640,
// five K chunks per group of 8 rows; the MMA's sixth chunk (k = 20..23) of
// row group r is therefore read from row group r + 1's first chunk (for the
// last row group: the next block), finite values that meet B's zero padding.
// A group's area is its four A blocks [left hi, left lo, right hi, right lo]
// followed by its four B blocks, all zeroed at the start.

constexpr uint32_t kTcRows = 128;           // patterns per tile (M)
constexpr uint32_t kTcN = 32;               // states padded (N)
constexpr uint32_t kTcK = 24;               // states padded (K)
constexpr uint32_t kTcSboA = 640;           // bytes per 8 rows of an A block
constexpr uint32_t kTcA = kTcRows / 8 * kTcSboA / 4; // floats per A block (2,560)
constexpr uint32_t kTcB = kTcN * kTcK;      // floats per B block (768)
constexpr uint32_t kTcGroup = 4 * kTcA + 4 * kTcB; // floats per group (53,248 B)
constexpr uint32_t kTcWaitLimit = 1u << 22; // polls, far beyond an MMA

// offset (floats) of element (row, k < 20) in an A block
__host__ __device__ __forceinline__ uint32_t tc_off_a(uint32_t row, uint32_t k)
{
	return (row >> 3) * (kTcSboA / 4) + (k >> 2) * 32u + (row & 7u) * 4u + (k & 3u);
}

// Named barrier of one 128-thread group: id 1 for group 0, 2 for group 1
// (0 is __syncthreads).  Immediate ids keep the CTA's barrier count at 3.
__device__ __forceinline__ void group_sync(uint32_t g)
{
	if (g == 0)
		asm volatile("bar.sync 1, 128;" ::: "memory");
	else
		asm volatile("bar.sync 2, 128;" ::: "memory");
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

template <typename Idx, uint32_t kG>
__global__ void __launch_bounds__(128 * kG, 4 / kG) prune20tc_kernel(Tc20Params prm)
{
	static_assert(kG == 1 || kG == 2, "one or two groups per CTA");
	constexpr int S = kS20;
	constexpr uint32_t kRowBytes = kTcRows * S * 4;  // a side's 128 partial rows
	constexpr uint32_t kOpBytes = 2 * kTcB * 4;      // its hi and lo B blocks
	constexpr uint32_t kTipBytes = (S + 1) * S * 4;  // a tip side's table
	static_assert(kRowBytes == kTcA * 4 && kTipBytes <= kOpBytes, "copy areas");
	extern __shared__ uint8_t tc_smem_raw[];
	float *sBase = reinterpret_cast<float *>(((uintptr_t)tc_smem_raw + 1023) &
						 ~(uintptr_t)1023);
	// then the list (when it fits) and the tile's tip codes
	NodeOp *sOps = reinterpret_cast<NodeOp *>(sBase + kG * kTcGroup);
	uint8_t *sTips = reinterpret_cast<uint8_t *>(sOps + (prm.ops_smem ? prm.n : 0));
	__shared__ __align__(8) uint64_t mbar[kG]; // MMA completion, per group
	__shared__ __align__(8) uint64_t lbar[kG]; // input copies, per group
	__shared__ uint32_t holder;
	// cluster-wide stop flags (rank 0's are read), one per run parity
	__shared__ uint32_t s_stop[2];
	const uint32_t g = threadIdx.x >> 7, t = threadIdx.x & 127u;
	const uint32_t warp = threadIdx.x >> 5;
	float *sA = sBase + g * kTcGroup; // [side][hi, lo][2,560]
	float *sB = sA + 4 * kTcA;         // [side][hi, lo][768]
	// grid (K, tiles, C): the cluster's CTAs share blockIdx.y / z
	const uint32_t K = gridDim.x, rank = blockIdx.x;
	const uint32_t gg = rank * kG + g, G = K * kG; // group in the cluster
	const uint32_t tile = blockIdx.y;
	const uint32_t c = blockIdx.z, C = prm.C;
	const uint32_t p = tile * kTcRows + t;
	const Idx stride = (Idx)C * prm.ldp;
	const Idx col0 = (Idx)c * prm.ldp + tile * kTcRows;
	const Idx col = col0 + t;
	const uint32_t mb = tc::smem_u32(&mbar[g]);
	const uint32_t lb = tc::smem_u32(&lbar[g]);

	// zero the operand areas: the A blocks' sixth K chunks read
	// neighbouring rows, which must hold finite values from the start
	float4 *z4 = reinterpret_cast<float4 *>(sBase);
	for (uint32_t k = threadIdx.x; k < kG * kTcGroup / 4; k += blockDim.x)
		z4[k] = make_float4(0.f, 0.f, 0.f, 0.f);
	for (uint32_t k = threadIdx.x; prm.ops_smem && k < prm.n; k += blockDim.x)
		sOps[k] = prm.ops[k];
	if (prm.tips_smem) {
		// 4-byte loads: the tile's 128 codes of every leaf
		uint32_t *s32 = reinterpret_cast<uint32_t *>(sTips);
		for (uint32_t k = threadIdx.x; k < prm.L * 32u; k += blockDim.x) {
			const uint32_t leaf = k >> 5, w4 = k & 31u;
			s32[k] = *reinterpret_cast<const uint32_t *>(
				prm.tips + (size_t)leaf * prm.ldp + tile * kTcRows + 4 * w4);
		}
	}
	const NodeOp *ops = prm.ops_smem ? sOps : prm.ops;
	if (threadIdx.x == 0) {
		for (uint32_t k = 0; k < kG; k++) {
			tc::mbar_init(tc::smem_u32(&mbar[k]), 1);
			tc::mbar_init(tc::smem_u32(&lbar[k]), 1);
		}
		s_stop[0] = s_stop[1] = 0u;
	}
	if (warp == 0)
		tc::tmem_alloc(tc::smem_u32(&holder), 128 * kG);
	tc::fence_proxy_async_smem(); // the zeroed areas before the first copies
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	// this group's accumulators: columns [128 g, 128 g + 128), 64 per side:
	// [0, 32) x_hi P_hi + x_lo P_hi, [32, 64) x_hi P_lo
	const uint32_t tmem = holder + 128u * g;
	const uint32_t lane_base = (32u * (warp & 3u)) << 16;
	// the hi and lo B blocks are adjacent (SBO 768 throughout), so one
	// N = 64 MMA multiplies x_hi by both
	constexpr uint32_t idesc = tc::idesc_tf32(kTcRows, kTcN);
	constexpr uint32_t idesc2 = tc::idesc_tf32(kTcRows, 2 * kTcN);
	// operand descriptors of K step 0: A [child][hi, lo]; B [child], its hi
	// block (the N = 64 form reaches the lo block after it)
	uint64_t dA[2][2], dB[2];
#pragma unroll
	for (uint32_t j = 0; j < 2; j++) {
#pragma unroll
		for (uint32_t h = 0; h < 2; h++)
			dA[j][h] = tc::smem_desc(tc::smem_u32(sA + (2 * j + h) * kTcA), 128,
						 kTcSboA);
		dB[j] = tc::smem_desc(tc::smem_u32(sB + 2 * j * kTcB), 128, 768);
	}

	// Inputs of entry e, copied by thread 0 of the group: an internal
	// side's 128 partial rows (contiguous) into its A-lo block, where they
	// wait to be split, its 128 scale exponents and its operand blocks into
	// its B blocks; a tip side's table into its B blocks and, unless the
	// tile's codes sit in shared memory, its 128 tip codes.  Exponents and
	// codes land in the right A-hi block (scales at bytes [512 + 512 j,
	// 1024 + 512 j), codes at [1536 + 128 j, 1664 + 128 j)): it is free
	// from the MMAs' end, when the next entry's copies are issued, to the
	// split, which reads them into registers first (the output rows pass
	// through the left A-hi block meanwhile).  Its first 128 bytes stay
	// clear: the left A-lo block's padded K chunk reads them, and exponent
	// bits could be NaNs.  So no global load waits on the entry's path.
	uint8_t *sSide = reinterpret_cast<uint8_t *>(sA + 2 * kTcA);
	auto issue = [&](uint32_t e) {
		const NodeOp op = ops[e];
		const uint32_t ids[2] = {op.left, op.right};
		uint32_t bytes = 0;
#pragma unroll
		for (uint32_t j = 0; j < 2; j++)
			bytes += (ids[j] & kTipBit)
					 ? kTipBytes + (prm.tips_smem ? 0u : kTcRows)
					 : kRowBytes + kOpBytes + kTcRows * 4u;
		tc::mbar_expect_tx(lb, bytes);
#pragma unroll
		for (uint32_t j = 0; j < 2; j++) {
			const size_t tid_tab = (size_t)(2 * e + j) * C + c;
			const uint32_t bdst = tc::smem_u32(sB + j * 2 * kTcB);
			if (ids[j] & kTipBit) {
				tc::bulk_g2s(bdst, prm.tab + tid_tab * (S + 1) * S, kTipBytes, lb);
				if (!prm.tips_smem)
					tc::bulk_g2s(tc::smem_u32(sSide + 1536 + 128 * j),
						     prm.tips + (size_t)(ids[j] & ~kTipBit) * prm.ldp +
							     tile * kTcRows,
						     kTcRows, lb);
			} else {
				const Idx ix0 = (Idx)ids[j] * stride + col0;
				tc::bulk_g2s(tc::smem_u32(sA + (2 * j + 1) * kTcA),
					     prm.partials + (size_t)ix0 * S, kRowBytes, lb);
				tc::bulk_g2s(bdst, prm.tc_tab + tid_tab * 2 * kTcB, kOpBytes, lb);
				tc::bulk_g2s(tc::smem_u32(sSide + 512 + 512 * j), prm.scales + ix0,
					     kTcRows * 4u, lb);
			}
		}
	};
	auto run_len = [&](uint32_t e0) {
		const uint32_t r = ops[e0].pad;
		return r == 0 ? 1u : min(r, prm.n - e0);
	};

	// output rows pass through the left A-hi block (raw [128][20] layout)
	float *stage = sA;
	uint32_t lphase = 0, mphase = 0;
	bool failed = false, pending = false;
	uint32_t e0 = 0, r = run_len(0);
	if (K > 1)
		cg::this_cluster().sync(); // every CTA started, its flags zeroed
	if (gg < r) {
		if (t == 0)
			issue(gg);
		pending = true;
	}
	uint32_t run = 0;
	for (;;) {
		for (uint32_t e = e0 + gg; e < e0 + r; e += G) {
			const NodeOp op = ops[e];
			const uint32_t ids[2] = {op.left, op.right};
			const bool any = !(ids[0] & kTipBit) || !(ids[1] & kTipBit);
			// a wait that gives up only marks the thread failed: the group
			// keeps to its barriers and the run's closing barrier stops the
			// CTA (the values computed meanwhile are discarded)
			failed |= !tc::mbar_wait(lb, lphase, kTcWaitLimit);
			lphase ^= 1u;
			pending = false;
			// this thread's rows: a tip side's final value from its table,
			// an internal side's partial row from the copied block
			float v[2][S];
			int32_t sc[2];
#pragma unroll
			for (uint32_t j = 0; j < 2; j++) {
				const float *row;
				if (ids[j] & kTipBit) {
					const uint32_t leaf = ids[j] & ~kTipBit;
					const uint32_t code =
						prm.tips_smem ? sTips[leaf * kTcRows + t]
							      : sSide[1536 + 128 * j + t];
					row = sB + j * 2 * kTcB + min(code, (uint32_t)S) * S;
					sc[j] = 0;
				} else {
					row = sA + (2 * j + 1) * kTcA + t * S;
					sc[j] = reinterpret_cast<const int32_t *>(sSide + 512 + 512 * j)[t];
				}
				const float4 *r4 = reinterpret_cast<const float4 *>(row);
#pragma unroll
				for (int q = 0; q < 5; q++) {
					const float4 a = r4[q];
					v[j][4 * q] = a.x;
					v[j][4 * q + 1] = a.y;
					v[j][4 * q + 2] = a.z;
					v[j][4 * q + 3] = a.w;
				}
			}
			// every copied row read, the previous entry's output stored
			group_sync(g);
			const bool next = e + G < e0 + r;
			if (!any) {
				if (next) {
					if (t == 0)
						issue(e + G);
					pending = true;
				}
			} else {
				// stage the internal sides' split rows
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
							tc::split_tf32(v[j][4 * q + u], h[u], l[u]);
						*reinterpret_cast<float4 *>(ah + tc_off_a(t, 4 * q)) =
							make_float4(h[0], h[1], h[2], h[3]);
						*reinterpret_cast<float4 *>(al + tc_off_a(t, 4 * q)) =
							make_float4(l[0], l[1], l[2], l[3]);
					}
				}
				tc::fence_proxy_async_smem();
				tc::fence_before_sync();
				group_sync(g);
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
							// x_hi [P_hi; P_lo], then x_lo P_hi
							tc::mma_tf32(tmem + 64 * j, dA[j][0] + 16 * s,
								     dB[j] + 16 * s, idesc2, s != 0);
							tc::mma_tf32(tmem + 64 * j, dA[j][1] + 16 * s,
								     dB[j] + 16 * s, idesc, 1);
						}
					}
					tc::mma_commit(mb);
				}
				failed |= !tc::mbar_wait(mb, mphase, kTcWaitLimit);
				mphase ^= 1u;
				// operands consumed: the group's next entry's inputs
				// travel during this epilogue
				if (next) {
					if (t == 0)
						issue(e + G);
					pending = true;
				}
				tc::fence_after_sync();
#pragma unroll
				for (uint32_t j = 0; j < 2; j++) {
					if (ids[j] & kTipBit)
						continue;
					const uint32_t ta = tmem + lane_base + 64 * j;
					float lo[S];
					tc::tmem_ld16(ta, v[j]);
					tc::tmem_ld4(ta + 16, v[j] + 16);
					tc::tmem_ld16(ta + 32, lo);
					tc::tmem_ld4(ta + 48, lo + 16);
					tc::tmem_wait_ld();
#pragma unroll
					for (int i = 0; i < S; i++)
						v[j][i] += lo[i];
				}
			}
			float y[S];
#pragma unroll
			for (int i = 0; i < S; i++)
				y[i] = v[0][i] * v[1][i];
			const int32_t cnt = sc[0] + sc[1] + rescale_pow2_20(y);
			prm.scales[(Idx)op.out * stride + col] = cnt;
			if (e + 1 == prm.n) {
				double dot = 0.0;
#pragma unroll
				for (int i = 0; i < S; i++)
					dot = fma(prm.pi[i], (double)y[i], dot);
				prm.root_val[(size_t)c * prm.ldp + p] = dot;
				prm.root_exp[(size_t)c * prm.ldp + p] = cnt;
			}
			// the output rows through shared memory, then 16-byte stores
			// of consecutive addresses by consecutive threads
			float4 *srow = reinterpret_cast<float4 *>(stage + t * S);
#pragma unroll
			for (int q = 0; q < 5; q++)
				srow[q] = make_float4(y[4 * q], y[4 * q + 1], y[4 * q + 2], y[4 * q + 3]);
			group_sync(g);
			const float4 *s4 = reinterpret_cast<const float4 *>(stage);
			float4 *d4 = reinterpret_cast<float4 *>(
				prm.partials + (size_t)((Idx)op.out * stride + col0) * S);
#pragma unroll
			for (uint32_t q = 0; q < 5; q++)
				d4[t + 128 * q] = s4[t + 128 * q];
		}
		// the run's outputs are visible to every group of the cluster,
		// and to the bulk copies of the next run, before those read them
		tc::fence_proxy_async_global();
		tc::fence_before_sync();
		int stop = __syncthreads_or(failed);
		if (K > 1) {
			// a stop anywhere stops every CTA at this run: the flag of
			// this run's parity in rank 0 (the other parity's may
			// already be written by a CTA ahead, never this one)
			cg::cluster_group cl = cg::this_cluster();
			uint32_t *flag = cl.map_shared_rank(&s_stop[run & 1u], 0);
			if (threadIdx.x == 0 && stop)
				atomicOr(flag, 1u);
			cl.sync();
			stop = *(volatile uint32_t *)flag != 0u;
		}
		tc::fence_after_sync();
		if (stop) {
			failed = true;
			break;
		}
		++run;
		e0 += r;
		if (e0 >= prm.n)
			break;
		r = run_len(e0);
		if (gg < r) {
			if (t == 0) {
				// other CTAs' stores before this CTA's bulk copies
				tc::fence_proxy_async_global();
				issue(e0 + gg);
			}
			pending = true;
		}
	}
	if (failed) {
		// copies still in flight land before the CTA leaves
		if (pending && t == 0)
			tc::mbar_wait(lb, lphase, kTcWaitLimit);
		if (threadIdx.x == 0)
			atomicExch(prm.status, 1u);
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	if (warp == 0)
		tc::tmem_dealloc(holder, 128 * kG);
	// no CTA leaves while another may still read rank 0's flags
	if (K > 1)
		cg::this_cluster().sync();
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
