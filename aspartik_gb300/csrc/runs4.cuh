// runs4.cuh -- run-synchronous FP32 pruning walks, single calculator and
// batched.  Included by kernels4.cu inside its anonymous namespace (uses
// v4_apply, v4_mul, rescale_pow2, transition4 and the Neumaier helpers).
//
// The one-thread-per-column walk leaves the GPU with only patterns x
// categories threads, about 14 warps per SM on the largest workload, and it
// is latency-bound.  Here a block owns a tile of patterns and walks the
// schedule run by run (a run is a sequence of mutually independent entries,
// e.g. one level of the tree).  Inside a run its (entry, category, pattern)
// items are spread over all threads of the block, so a wide level keeps
// every thread busy; a __syncthreads() separates runs.
//
// Thread layout: column col = c * tile + pl (fixed per thread, patterns
// fastest, so a warp touches 32 consecutive patterns of one category) and
// group g; group g handles entries g, g + groups, ... of every run.

// Everything one tile walk needs; the single-calculator kernel fills it from
// PruneParams, the batched kernel from the member's descriptor.
struct TileArgs {
	const uint8_t *tips;
	float4 *part;
	int32_t *scales;
	const float4 *ptab;
	const double *pi;
	const uint32_t *weights;
	double *site_lnl;
	double *cat_lnl;
	uint32_t ldp, C, L, tile, n, n_runs, tips_smem;
	double log_inv_c;
};

// Tip codes come from the block's shared-memory tile (tip_row = tile) or
// from global memory (tips_p = tips + p, tip_row = ldp); the schedule from
// shared memory.
template <typename Idx>
__device__ __forceinline__ void run_item(const NodeOp *__restrict__ ops,
					 const uint8_t *__restrict__ tips_p,
					 uint32_t tip_row,
					 const float4 *__restrict__ ptab,
					 float4 *__restrict__ part,
					 int32_t *__restrict__ scales, uint32_t C,
					 Idx stride, Idx col_off, uint32_t c,
					 uint32_t i, float4 &y, int32_t &cnt)
{
	const NodeOp op = ops[i];
	const float4 *tl = ptab + ((size_t)(2 * i) * C + c) * 5;
	const float4 *tr = tl + 5 * C;
	float4 a, b;
	int32_t sa = 0, sb = 0;
	if (op.left & kTipBit) {
		a = tl[tips_p[(Idx)(op.left & ~kTipBit) * tip_row]];
	} else {
		const Idx ix = (Idx)op.left * stride + col_off;
		const float4 x = part[ix];
		sa = scales[ix];
		a = v4_apply(tl, x);
	}
	if (op.right & kTipBit) {
		b = tr[tips_p[(Idx)(op.right & ~kTipBit) * tip_row]];
	} else {
		const Idx ix = (Idx)op.right * stride + col_off;
		const float4 x = part[ix];
		sb = scales[ix];
		b = v4_apply(tr, x);
	}
	y = v4_mul(a, b);
	cnt = sa + sb + rescale_pow2(y);
	const Idx ox = (Idx)op.out * stride + col_off;
	part[ox] = y;
	scales[ox] = cnt;
}

__device__ __forceinline__ double root_dot4(const double *pi, const float4 &y)
{
	return (double)pi[0] * y.x + (double)pi[1] * y.y + (double)pi[2] * y.z +
	       (double)pi[3] * y.w;
}

// One pattern tile t: every run of the schedule, then the category mixing
// of the root.  Returns the tile's weighted site sum in thread 0.  Ends with
// the block synchronised.  s_dot/s_cnt hold tile * C entries, s_red 32.
template <typename Idx>
__device__ double tile_walk(const TileArgs &a, uint32_t t, double *s_dot,
			    int32_t *s_cnt, double *s_red,
			    const NodeOp *s_ops, const uint32_t *s_runs,
			    uint8_t *s_tips)
{
	const uint32_t tile = a.tile, C = a.C;
	const uint32_t cols = tile * C;
	const uint32_t groups = blockDim.x / cols;
	const uint32_t tid = threadIdx.x;
	const uint32_t col = tid % cols, g = tid / cols;
	const uint32_t c = col / tile, pl = col - c * tile;
	const bool worker = g < groups;
	const Idx stride = (Idx)C * a.ldp;
	const uint32_t p = t * tile + pl;
	const Idx col_off = (Idx)c * a.ldp + p;

	const uint8_t *tips_p;
	uint32_t tip_row;
	if (a.tips_smem) {
		// 4-byte loads: rows start at multiples of 32 patterns
		const uint32_t wpr = tile >> 2;
		const uint32_t total = a.L * wpr;
		uint32_t *s_t32 = (uint32_t *)s_tips;
		for (uint32_t k = tid; k < total; k += blockDim.x) {
			const uint32_t leaf = k / wpr, w4 = k - leaf * wpr;
			s_t32[k] = *(const uint32_t *)(a.tips + (size_t)leaf * a.ldp +
						       t * tile + w4 * 4);
		}
		tips_p = s_tips + pl;
		tip_row = tile;
	} else {
		tips_p = a.tips + p;
		tip_row = a.ldp;
	}
	__syncthreads();
	if (a.n_runs == a.n) {
		// A path (every run one entry, e.g. the ancestors of a node whose
		// height changed): each entry needs only the previous entry's
		// result and clean inputs, so one thread per column walks it alone
		// with no barrier, takes the previous result from registers and
		// prefetches the clean children two entries ahead into L1.
		if (g == 0) {
			float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
			int32_t cnt = 0;
			uint32_t prev_out = 0xFFFFFFFFu;
			// every input that does not come from this walk, requested
			// at once: one memory latency for the whole path
			for (uint32_t j = 0; j < a.n && j < 64; ++j) {
				const NodeOp o = s_ops[j];
				const uint32_t own = j ? s_ops[j - 1].out : 0xFFFFFFFFu;
				for (const uint32_t id : {o.left, o.right}) {
					const void *ptr;
					if (id & kTipBit) {
						if (a.tips_smem) // already on chip
							continue;
						ptr = tips_p + (Idx)(id & ~kTipBit) * tip_row;
					} else if (id != own)
						ptr = a.part + ((Idx)id * stride + col_off);
					else
						continue;
					asm volatile("prefetch.global.L1 [%0];" ::"l"(ptr));
				}
			}
			for (uint32_t i = 0; i < a.n; ++i) {
				const NodeOp op = s_ops[i];
				const float4 *tl = a.ptab + ((size_t)(2 * i) * C + c) * 5;
				const float4 *tr = tl + 5 * C;
				float4 ca, cb;
				int32_t sa = 0, sb = 0;
				if (op.left & kTipBit) {
					ca = tl[tips_p[(Idx)(op.left & ~kTipBit) * tip_row]];
				} else if (op.left == prev_out) {
					ca = v4_apply(tl, y);
					sa = cnt;
				} else {
					const Idx ix = (Idx)op.left * stride + col_off;
					sa = a.scales[ix];
					ca = v4_apply(tl, a.part[ix]);
				}
				if (op.right & kTipBit) {
					cb = tr[tips_p[(Idx)(op.right & ~kTipBit) * tip_row]];
				} else if (op.right == prev_out) {
					cb = v4_apply(tr, y);
					sb = cnt;
				} else {
					const Idx ix = (Idx)op.right * stride + col_off;
					sb = a.scales[ix];
					cb = v4_apply(tr, a.part[ix]);
				}
				y = v4_mul(ca, cb);
				cnt = sa + sb + rescale_pow2(y);
				const Idx ox = (Idx)op.out * stride + col_off;
				a.part[ox] = y;
				a.scales[ox] = cnt;
				prev_out = op.out;
			}
			s_dot[col] = root_dot4(a.pi, y);
			s_cnt[col] = cnt;
		}
		__syncthreads();
	}
	for (uint32_t r = 0; r < a.n_runs && a.n_runs != a.n; ++r) {
		const uint32_t start = s_runs[r], end = s_runs[r + 1];
		if (worker) {
			uint32_t i = start + g;
			// two independent entries per iteration: all their loads
			// are issued before either product
			for (; i + groups < end; i += 2 * groups) {
				float4 y0, y1;
				int32_t c0, c1;
				run_item<Idx>(s_ops, tips_p, tip_row, a.ptab, a.part,
					      a.scales, C, stride, col_off, c, i, y0, c0);
				run_item<Idx>(s_ops, tips_p, tip_row, a.ptab, a.part,
					      a.scales, C, stride, col_off, c,
					      i + groups, y1, c1);
				if (i + groups == a.n - 1) {
					s_dot[col] = root_dot4(a.pi, y1);
					s_cnt[col] = c1;
				}
			}
			if (i < end) {
				float4 y0;
				int32_t c0;
				run_item<Idx>(s_ops, tips_p, tip_row, a.ptab, a.part,
					      a.scales, C, stride, col_off, c, i, y0, c0);
				if (i == a.n - 1) {
					s_dot[col] = root_dot4(a.pi, y0);
					s_cnt[col] = c0;
				}
			}
		}
		__syncthreads();
	}
	// root: category mixing per pattern (threads 0 .. tile-1)
	double contrib = 0.0;
	if (tid < tile) {
		const uint32_t pp = t * tile + tid;
		int32_t emax = INT32_MIN;
		for (uint32_t k = 0; k < C; k++)
			if (s_dot[k * tile + tid] > 0.0)
				emax = max(emax, s_cnt[k * tile + tid]);
		double site;
		if (emax == INT32_MIN) {
			site = -INFINITY;
		} else {
			double acc = 0.0;
			for (uint32_t k = 0; k < C; k++)
				acc += scalbn(s_dot[k * tile + tid],
					      s_cnt[k * tile + tid] - emax);
			site = log(acc) + (double)emax * 0.69314718055994530942 +
			       a.log_inv_c;
		}
		a.site_lnl[pp] = site;
		if (a.cat_lnl)
			for (uint32_t k = 0; k < C; k++)
				a.cat_lnl[(size_t)k * a.ldp + pp] =
					log(s_dot[k * tile + tid]) +
					(double)s_cnt[k * tile + tid] *
						0.69314718055994530942;
		const uint32_t wgt = a.weights[pp];
		contrib = wgt ? site * (double)wgt : 0.0;
	}
	// tile sum in a fixed order (warp shuffles, then warps in order)
	for (int off = 16; off > 0; off >>= 1)
		contrib += __shfl_down_sync(0xffffffffu, contrib, off);
	if ((tid & 31u) == 0 && tid < tile)
		s_red[tid >> 5] = contrib;
	__syncthreads();
	double tsum = 0.0;
	if (tid == 0)
		for (uint32_t w2 = 0; w2 < (tile + 31u) / 32u; w2++)
			tsum += s_red[w2];
	__syncthreads();
	return tsum;
}

// Fold `count` compensated-free partial sums at `sums` with Neumaier
// compensation in a fixed-shape tree (threads of the block); the result is
// returned in thread 0.  Uses 2 * blockDim.x doubles at s_red.
__device__ double block_fold(const double *sums, uint32_t count, double *s_red)
{
	const uint32_t tid = threadIdx.x, nthr = blockDim.x;
	double sum = 0.0, comp = 0.0;
	for (uint32_t k = tid; k < count; k += nthr)
		neumaier_add(sum, comp, __ldcg(sums + k));
	double *s_sum = s_red;
	double *s_comp = s_red + nthr;
	s_sum[tid] = sum;
	s_comp[tid] = comp;
	__syncthreads();
	uint32_t span = 1;
	while (span < nthr)
		span <<= 1;
	for (uint32_t stride2 = span >> 1; stride2 > 0; stride2 >>= 1) {
		if (tid < stride2 && tid + stride2 < nthr) {
			double x = s_sum[tid], xc = s_comp[tid];
			neumaier_merge(x, xc, s_sum[tid + stride2], s_comp[tid + stride2]);
			s_sum[tid] = x;
			s_comp[tid] = xc;
		}
		__syncthreads();
	}
	double total = 0.0;
	if (tid == 0)
		total = isfinite(s_sum[0]) ? s_sum[0] + s_comp[0] : s_sum[0];
	__syncthreads();
	return total;
}

// shared memory: [dot: cols][cnt: cols/2][red: 2 * blockDim][ops][runs][tips]
template <typename Idx>
__global__ void __launch_bounds__(512, 2) prune4_runs_kernel(PruneParams prm)
{
	const uint32_t cols = prm.tile * prm.C;
	const uint32_t tid = threadIdx.x;
	extern __shared__ double smem[];
	double *s_dot = smem;
	int32_t *s_cnt = (int32_t *)(smem + cols);
	double *s_red = smem + cols + (cols + 1) / 2;
	NodeOp *s_ops = (NodeOp *)(s_red + 2 * blockDim.x);
	uint32_t *s_runs = (uint32_t *)(s_ops + prm.n);
	uint8_t *s_tips = (uint8_t *)(s_runs + ((prm.n_runs + 4) & ~3u));
	float4 *s_ptab = (float4 *)(((uintptr_t)s_tips +
				     (prm.tips_smem ? prm.num_leaves * prm.tile : 0u) + 15) &
				    ~(uintptr_t)15);
	__shared__ unsigned s_last;

	for (uint32_t k = tid; k < prm.n; k += blockDim.x)
		s_ops[k] = prm.ops[k];
	for (uint32_t k = tid; k <= prm.n_runs; k += blockDim.x)
		s_runs[k] = prm.runs[k];

	TileArgs a;
	a.tips = prm.tips;
	a.part = (float4 *)prm.partials;
	a.scales = prm.scales;
	a.ptab = (const float4 *)prm.ptab;
	a.pi = prm.pi;
	a.weights = prm.weights;
	a.site_lnl = prm.site_lnl;
	a.cat_lnl = prm.cat_lnl;
	a.ldp = prm.ldp;
	a.C = prm.C;
	a.L = prm.num_leaves;
	a.tile = prm.tile;
	a.n = prm.n;
	a.n_runs = prm.n_runs;
	a.tips_smem = prm.tips_smem;
	a.log_inv_c = prm.log_inv_c;
	if (prm.ptab_smem) {
		// every table row of the list, once per block (one load latency)
		const uint32_t rows = prm.n * 2 * prm.C * 5;
		for (uint32_t k = tid; k < rows; k += blockDim.x)
			s_ptab[k] = a.ptab[k];
		a.ptab = s_ptab;
	}

	double cta_sum = 0.0, cta_comp = 0.0; // thread 0: this block's tiles
	const uint32_t ntiles = prm.ldp / prm.tile;
	for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const double tsum =
			tile_walk<Idx>(a, t, s_dot, s_cnt, s_red, s_ops, s_runs, s_tips);
		if (tid == 0)
			neumaier_add(cta_sum, cta_comp, tsum);
	}
	if (tid == 0) {
		prm.block_sums[blockIdx.x] =
			isfinite(cta_sum) ? cta_sum + cta_comp : cta_sum;
		__threadfence();
		const unsigned tk = atomicAdd(prm.ticket, 1u);
		s_last = (tk == gridDim.x - 1u);
	}
	__syncthreads();
	if (!s_last)
		return;
	// the last block folds the block sums in a fixed-shape tree
	__threadfence();
	const double total = block_fold(prm.block_sums, gridDim.x, s_red);
	if (tid == 0) {
		*prm.lnl_out = total;
		*prm.ticket = 0u;
	}
}

// ---------------------------------------------------------------------------
// Batched evaluation: many calculators (chains) in one launch.

__global__ void __launch_bounds__(32) ptab4_batch_kernel(BatchParams bp)
{
	const uint32_t m = blockIdx.y;
	const MemberStep st = bp.steps[m];
	if (st.n == 0)
		return;
	const MemberDesc &md = bp.members[m];
	const uint32_t C = md.C;
	const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
	if (id >= st.n * 2u * C)
		return;
	const uint32_t c = id % C, es = id / C;
	const double *lengths = (const double *)(md.stage + md.off_in);
	const double d = lengths[es] * (st.clock_rate * md.model->cat_rates[c]);
	float P[16];
	transition4f(md.model, d, P);
	float *out = md.ptab + (size_t)id * 20;
	for (int k = 0; k < 4; k++)
		for (int j = 0; j < 4; j++)
			out[k * 4 + j] = P[j * 4 + k];
	for (int j = 0; j < 4; j++)
		out[16 + j] = 1.0f;
}

// Persistent blocks take (member, tile) work items from a counter; members
// are visited in the order of the descriptor array (the host puts the
// costliest first).  Each tile's weighted sum goes to the member's tile
// slot; the block that finishes a member's last tile folds that member's
// sums (fixed order, so the result does not depend on scheduling).
template <typename Idx>
__global__ void __launch_bounds__(512, 2) prune4_batch_kernel(BatchParams bp)
{
	constexpr uint32_t kMaxMembers = 256;
	__shared__ uint32_t s_prefix[kMaxMembers + 1];
	__shared__ uint32_t s_work;
	__shared__ unsigned s_last;
	extern __shared__ double smem[];
	const uint32_t tid = threadIdx.x;
	const uint32_t M = bp.num_members;
	double *s_dot = smem;
	int32_t *s_cnt = (int32_t *)(smem + bp.max_cols);
	double *s_red = smem + bp.max_cols + (bp.max_cols + 1) / 2;
	NodeOp *s_ops = (NodeOp *)(s_red + 2 * blockDim.x);
	uint8_t *s_tips = (uint8_t *)s_ops + bp.smem_ops_bytes;
	float4 *s_ptab = (float4 *)(((uintptr_t)s_tips + bp.smem_tips_bytes + 15) &
				    ~(uintptr_t)15);

	if (tid == 0) {
		uint32_t acc = 0;
		for (uint32_t m = 0; m < M; ++m) {
			s_prefix[m] = acc;
			if (bp.steps[m].n)
				acc += bp.members[m].ldp / bp.steps[m].tile;
		}
		s_prefix[M] = acc;
	}
	__syncthreads();
	const uint32_t total = s_prefix[M];
	uint32_t cur = 0xFFFFFFFFu;
	TileArgs a;
	uint32_t *s_runs = nullptr;
	for (;;) {
		if (tid == 0)
			s_work = atomicAdd(bp.work_next, 1u);
		__syncthreads();
		const uint32_t w = s_work;
		__syncthreads();
		if (w >= total)
			break;
		// the member whose tile range holds w
		uint32_t lo = 0, hi = M;
		while (hi - lo > 1) {
			const uint32_t mid = (lo + hi) >> 1;
			if (s_prefix[mid] <= w)
				lo = mid;
			else
				hi = mid;
		}
		while (lo + 1 < M && s_prefix[lo + 1] <= w)
			++lo;
		const uint32_t m = lo, t = w - s_prefix[m];
		const MemberDesc &md = bp.members[m];
		if (m != cur) {
			const MemberStep st = bp.steps[m];
			a.tips = md.tips;
			a.part = (float4 *)md.partials;
			a.scales = md.scales;
			a.ptab = (const float4 *)md.ptab;
			a.pi = (const double *)(md.stage + md.off_pi);
			a.weights = md.weights;
			a.site_lnl = md.site_lnl;
			a.cat_lnl = nullptr;
			a.ldp = md.ldp;
			a.C = md.C;
			a.L = md.L;
			a.tile = st.tile;
			a.n = st.n;
			a.n_runs = st.n_runs;
			a.tips_smem = st.tips_smem;
			a.log_inv_c = md.log_inv_c;
			const NodeOp *g_ops = (const NodeOp *)md.stage;
			const uint32_t *g_runs = (const uint32_t *)(md.stage + md.off_runs);
			s_runs = (uint32_t *)(s_ops + st.n);
			for (uint32_t k = tid; k < st.n; k += blockDim.x)
				s_ops[k] = g_ops[k];
			for (uint32_t k = tid; k <= st.n_runs; k += blockDim.x)
				s_runs[k] = g_runs[k];
			// a small list's tables in shared memory (see the single-
			// calculator kernel)
			const uint32_t rows = st.n * 2 * md.C * 5;
			if (rows * sizeof(float4) <= bp.smem_ptab_bytes) {
				for (uint32_t k = tid; k < rows; k += blockDim.x)
					s_ptab[k] = ((const float4 *)md.ptab)[k];
				a.ptab = s_ptab;
			}
			cur = m;
			__syncthreads();
		}
		const double tsum =
			tile_walk<Idx>(a, t, s_dot, s_cnt, s_red, s_ops, s_runs, s_tips);
		const uint32_t tiles = md.ldp / a.tile;
		if (tid == 0) {
			md.tile_sums[t] = tsum;
			__threadfence();
			const unsigned tk = atomicAdd(md.ticket, 1u);
			s_last = (tk == tiles - 1u);
		}
		__syncthreads();
		if (s_last) {
			__threadfence();
			const double lnl = block_fold(md.tile_sums, tiles, s_red);
			if (tid == 0) {
				bp.lnl_out[m] = lnl;
				*md.ticket = 0u;
			}
		}
		__syncthreads();
	}
}
