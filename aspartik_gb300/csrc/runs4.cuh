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
	// inline tables (RunSmem::tabs set): their sources
	const ModelDev *model;
	const double *lengths;
	const double *matrices;
};

// Shared-memory extras of the run walk (all null: none).  sp/ss: slot
// partials and counts (the entries' slot codes travel in NodeOp::pad of the
// schedule's shared-memory copy); tabs: two buffers of
// tab_stride float4 for the per-run tables; eig (V, V^-1, lambda in FP32),
// rate (clock rate x category rate) and len (edge lengths, or null: read
// from global memory) feed the table builder.
struct RunSmem {
	float4 *sp;
	int32_t *ss;
	float4 *tabs;
	uint32_t tab_stride;
	const float *eig;
	const double *rate;
	const double *len;
};

// Transition tables of entries [lo, hi) into buf, entry lo first, in
// ptab4_kernel's layout and with its arithmetic (the same FP32 eigensystem,
// the same product of the length and the rates in FP64), one matrix per
// thread.
__device__ __forceinline__ void build_run_tables(const TileArgs &a,
						 const RunSmem &rs,
						 uint32_t lo, uint32_t hi,
						 float4 *buf)
{
	const uint32_t C = a.C;
	const uint32_t count = (hi - lo) * 2 * C;
	// highest threads first: the last group walks the fewest entries
	for (uint32_t k = blockDim.x - 1u - threadIdx.x; k < count; k += blockDim.x) {
		const uint32_t id = lo * 2 * C + k;
		const uint32_t c = id % C, es = id / C;
		float P[16];
		if (a.matrices) {
			const double *src = a.matrices + (size_t)id * 16;
			for (int q = 0; q < 16; q++)
				P[q] = (float)src[q];
		} else {
			const double len = rs.len ? rs.len[es] : a.lengths[es];
			transition4f_eig(a.model, rs.eig, len * rs.rate[c], P);
		}
		float4 *out = buf + k * 5;
#pragma unroll
		for (int q = 0; q < 4; q++)
			out[q] = make_float4(P[q], P[4 + q], P[8 + q], P[12 + q]);
		out[4] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
	}
}

// Root: frequency-weighted sum of the partial vector, in FP32 (the FP64
// pipe runs at 1/64 of the FP32 rate on this part, and the root mixing of
// every pattern sits on the critical path of a short dirty list).
__device__ __forceinline__ float root_dot4(const float *pi, const float4 &y)
{
	return fmaf(pi[3], y.w, fmaf(pi[2], y.z, fmaf(pi[1], y.y, pi[0] * y.x)));
}

// Per-thread constants of a tile walk.  Tip codes come from the block's
// shared-memory tile (tip_row = tile) or from global memory (tips_p = tips
// + p, tip_row = ldp); the schedule and the slot codes from shared memory.
// A listed child whose output sits in a shared-memory slot (sp/ss: slot k
// of column col at k * cols + col) is read from there: the children of a
// whole-tree list are then never read back from L2 or DRAM.
template <typename Idx>
struct WalkCtx {
	const NodeOp *ops; // pad: the entry's slot codes
	float4 *sp;
	int32_t *ss;
	const uint8_t *tips_p;
	const float *pi;
	const float4 *tab; // tables of entry tab_i0 first
	uint32_t tab_i0;
	uint32_t tip_row, c, col, cols;
	uint32_t half; // the thread's second column: col + half (pattern + half)
	Idx stride, col_off;
};

// sum_k x_k * row_k for two vectors with the same four table rows (loaded
// once), in v4_apply's order.
__device__ __forceinline__ void v4_apply_pair(const float4 *pt, float4 &x0,
					      float4 &x1)
{
	const float4 r[4] = {pt[0], pt[1], pt[2], pt[3]};
	x0 = v4_apply(r, x0);
	x1 = v4_apply(r, x1);
}

// One child of entry i for the thread's two columns: a tip gives its
// table rows (the products themselves), a partial its vectors and
// cumulative counts (transformed by the caller).
template <typename Idx>
__device__ __forceinline__ void load_child2(const TileArgs &a,
					    const WalkCtx<Idx> &w, uint32_t id,
					    uint32_t slot, const float4 *tb,
					    float4 &x0, float4 &x1, int32_t &s0,
					    int32_t &s1)
{
	if (id & kTipBit) {
		const uint8_t *tp = w.tips_p + (Idx)(id & ~kTipBit) * w.tip_row;
		x0 = tb[tp[0]];
		x1 = tb[tp[w.half]];
		s0 = 0;
		s1 = 0;
	} else if (slot != kNoSlot) {
		const uint32_t k = slot * w.cols + w.col;
		x0 = w.sp[k];
		x1 = w.sp[k + w.half];
		s0 = w.ss[k];
		s1 = w.ss[k + w.half];
	} else {
		const Idx ix = (Idx)id * w.stride + w.col_off;
		x0 = a.part[ix];
		x1 = a.part[ix + w.half];
		s0 = a.scales[ix];
		s1 = a.scales[ix + w.half];
	}
}

// Entry i of the current run for the thread's two columns: both children
// (a tip's table row, a slot, or global memory), the products, the
// rescalings, the stores to global memory (read by later evaluations) and,
// when the entry has one, to its slot; the list's last entry (the root)
// leaves its frequency-weighted sums and counts in s_dot / s_cnt.  The
// entry's schedule word, slot codes and table rows are read once for both
// columns.  The host gives an entry one of its own children's slots or a
// slot released in an earlier run, so no other entry of the run reads the
// slot it writes.
template <typename Idx>
__device__ __forceinline__ void run_item2(const TileArgs &a,
					  const WalkCtx<Idx> &w, uint32_t i,
					  float *s_dot, int32_t *s_cnt)
{
	const NodeOp op = w.ops[i];
	const uint32_t sw = op.pad;
	const float4 *tl = w.tab + ((2 * (i - w.tab_i0)) * a.C + w.c) * 5;
	const float4 *tr = tl + 5 * a.C;
	float4 a0, a1, b0, b1;
	int32_t sa0, sa1, sb0, sb1;
	load_child2<Idx>(a, w, op.left, (sw >> 8) & 0xFFu, tl, a0, a1, sa0, sa1);
	load_child2<Idx>(a, w, op.right, (sw >> 16) & 0xFFu, tr, b0, b1, sb0,
			 sb1);
	if (!(op.left & kTipBit))
		v4_apply_pair(tl, a0, a1);
	if (!(op.right & kTipBit))
		v4_apply_pair(tr, b0, b1);
	float4 y0 = v4_mul(a0, b0), y1 = v4_mul(a1, b1);
	const int32_t n0 = sa0 + sb0 + rescale_pow2(y0);
	const int32_t n1 = sa1 + sb1 + rescale_pow2(y1);
	const Idx ox = (Idx)op.out * w.stride + w.col_off;
	a.part[ox] = y0;
	a.part[ox + w.half] = y1;
	a.scales[ox] = n0;
	a.scales[ox + w.half] = n1;
	const uint32_t os = sw & 0xFFu;
	if (os != kNoSlot) {
		const uint32_t k = os * w.cols + w.col;
		w.sp[k] = y0;
		w.sp[k + w.half] = y1;
		w.ss[k] = n0;
		w.ss[k + w.half] = n1;
	}
	if (i == a.n - 1) {
		s_dot[w.col] = root_dot4(w.pi, y0);
		s_dot[w.col + w.half] = root_dot4(w.pi, y1);
		s_cnt[w.col] = n0;
		s_cnt[w.col + w.half] = n1;
	}
}

__device__ double tile_root(const TileArgs &a, uint32_t t, const float *s_dot,
			    const int32_t *s_cnt, double *s_red);

// One pattern tile t: every run of the schedule, then the category mixing
// of the root.  Returns the tile's weighted site sum in thread 0.  Ends with
// the block synchronised.  s_dot/s_cnt hold tile * C entries, s_red 32;
// rs the run walk's shared-memory extras.  The run walk reads each entry's
// slot codes from NodeOp::pad of s_ops (0xFFFFFF: no slots).
template <typename Idx, bool kPrefetch = false>
__device__ double tile_walk(const TileArgs &a, uint32_t t, float *s_dot,
			    int32_t *s_cnt, double *s_red,
			    const NodeOp *s_ops, const uint32_t *s_runs,
			    uint8_t *s_tips, const RunSmem &rs = RunSmem{})
{
	const uint32_t tile = a.tile, C = a.C;
	const uint32_t cols = tile * C;
	const uint32_t groups = blockDim.x / cols;
	const uint32_t tid = threadIdx.x;
	const uint32_t col = tid % cols;
	const uint32_t c = col / tile, pl = col - c * tile;
	const Idx stride = (Idx)C * a.ldp;
	const uint32_t p = t * tile + pl;
	const Idx col_off = (Idx)c * a.ldp + p;

	__shared__ float s_pi[4];
	if (tid < 4)
		s_pi[tid] = (float)a.pi[tid];
	const bool serial = groups == 1;
	const uint8_t *tips_p, *tips_base;
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
		tips_base = s_tips;
		tip_row = tile;
	} else {
		tips_base = a.tips + t * tile;
		tip_row = a.ldp;
	}
	tips_p = tips_base + pl;
	const bool inl = !serial && rs.tabs != nullptr && a.n_runs != 0;
	if (inl)
		build_run_tables(a, rs, s_runs[0], s_runs[1], rs.tabs);
	__syncthreads();
	if (serial) {
		// One thread per column (tile * C == blockDim.x) walks the whole
		// list in order, with no barrier: a child that is the output of
		// one of the two previous entries comes from registers, any other
		// listed child from memory (written earlier by this thread).  The
		// walk is issue-bound (about 700 cycles an entry at 16 warps per
		// SM), so clean inputs are loaded plainly: staging them ahead in
		// shared memory was measured to gain nothing.
		float4 y0 = make_float4(0.f, 0.f, 0.f, 0.f), y1 = y0;
		int32_t c0 = 0, c1 = 0;
		uint32_t o0 = 0xFFFFFFFFu, o1 = 0xFFFFFFFFu;
		// A child that is neither a tip nor one of the two previous
		// outputs is read from global memory (a clean subtree, usually
		// not in L2).  With kPrefetch (the fused short-list kernel, whose
		// registers allow it) its load for entry i + 1 is issued before
		// entry i's product, so the latency overlaps the arithmetic: it is
		// never entry i's or i-1's output, and any earlier output it may
		// be was stored by this thread before the load.
		float4 pf[2];
		int32_t pfs[2];
		auto fetch = [&](const NodeOp &op, uint32_t f0, uint32_t f1) {
			const uint32_t ids[2] = {op.left, op.right};
#pragma unroll
			for (int j = 0; j < 2; ++j)
				if (!(ids[j] & kTipBit) && ids[j] != f0 && ids[j] != f1) {
					const Idx ix = (Idx)ids[j] * stride + col_off;
					pf[j] = a.part[ix];
					pfs[j] = a.scales[ix];
				}
		};
		auto input = [&](uint32_t id, const float4 *tb, int j, float4 &v,
				 int32_t &sc) {
			if (id & kTipBit) {
				v = tb[tips_p[(Idx)(id & ~kTipBit) * tip_row]];
				sc = 0;
			} else if (id == o0) {
				v = v4_apply(tb, y0);
				sc = c0;
			} else if (id == o1) {
				v = v4_apply(tb, y1);
				sc = c1;
			} else if (kPrefetch) {
				v = v4_apply(tb, pf[j]);
				sc = pfs[j];
			} else {
				const Idx ix = (Idx)id * stride + col_off;
				sc = a.scales[ix];
				v = v4_apply(tb, a.part[ix]);
			}
		};
		if (kPrefetch && a.n)
			fetch(s_ops[0], o0, o1);
		for (uint32_t i = 0; i < a.n; ++i) {
			const NodeOp op = s_ops[i];
			const float4 *tl = a.ptab + ((size_t)(2 * i) * C + c) * 5;
			const float4 *tr = tl + 5 * C;
			float4 ca, cb;
			int32_t sa, sb;
			input(op.left, tl, 0, ca, sa);
			input(op.right, tr, 1, cb, sb);
			if (kPrefetch && i + 1 < a.n) // forwards after this entry: op.out, o0
				fetch(s_ops[i + 1], op.out, o0);
			float4 y = v4_mul(ca, cb);
			const int32_t cnt = sa + sb + rescale_pow2(y);
			const Idx ox = (Idx)op.out * stride + col_off;
			a.part[ox] = y;
			a.scales[ox] = cnt;
			y1 = y0;
			c1 = c0;
			o1 = o0;
			y0 = y;
			c0 = cnt;
			o0 = op.out;
		}
		s_dot[col] = root_dot4(s_pi, y0);
		s_cnt[col] = c0;
		__syncthreads();
	}
	if (!serial) {
		// two columns per thread: patterns ph and ph + tile / 2 of one
		// category, so a warp still reads 32 consecutive patterns
		const uint32_t half = tile >> 1, tcols = cols >> 1;
		const uint32_t rgroups = blockDim.x / tcols;
		const uint32_t ct = tid % tcols, rg = tid / tcols;
		const uint32_t rc = ct / half, ph = ct - rc * half;
		WalkCtx<Idx> w;
		w.ops = s_ops;
		w.sp = rs.sp;
		w.ss = rs.ss;
		w.tab = a.ptab;
		w.tab_i0 = 0;
		w.tips_p = tips_base + ph;
		w.pi = s_pi;
		w.tip_row = tip_row;
		w.c = rc;
		w.col = rc * tile + ph;
		w.cols = cols;
		w.half = half;
		w.stride = stride;
		w.col_off = (Idx)rc * a.ldp + t * tile + ph;
		for (uint32_t r = 0; r < a.n_runs; ++r) {
			const uint32_t start = s_runs[r], end = s_runs[r + 1];
			if (inl) {
				// the next run's tables into the other buffer (last
				// read before the previous barrier)
				if (r + 1 < a.n_runs)
					build_run_tables(a, rs, end, s_runs[r + 2],
							 rs.tabs + ((r + 1) & 1u) * rs.tab_stride);
				w.tab = rs.tabs + (r & 1u) * rs.tab_stride;
				w.tab_i0 = start;
			}
			for (uint32_t i = start + rg; i < end; i += rgroups)
				run_item2<Idx>(a, w, i, s_dot, s_cnt);
			__syncthreads();
		}
	}
	return tile_root(a, t, s_dot, s_cnt, s_red);
}

// Root of tile t after its walk left pi . x and the exponent of every
// column in s_dot / s_cnt: category mixing per pattern (threads 0 ..
// tile-1), site values, and the tile's weighted sum in a fixed order,
// returned in thread 0.  Ends with the block synchronised.
__device__ double tile_root(const TileArgs &a, uint32_t t, const float *s_dot,
			    const int32_t *s_cnt, double *s_red)
{
	const uint32_t tile = a.tile, C = a.C;
	const uint32_t tid = threadIdx.x;
	double contrib = 0.0;
	if (tid < tile) {
		const uint32_t pp = t * tile + tid;
		int32_t emax = INT32_MIN;
		for (uint32_t k = 0; k < C; k++)
			if (s_dot[k * tile + tid] > 0.f)
				emax = max(emax, s_cnt[k * tile + tid]);
		double site;
		if (emax == INT32_MIN) {
			site = -INFINITY;
		} else {
			// categories mixed in FP32 at the largest exponent; only
			// the exact exponent term and the constant join in FP64
			float acc = 0.f;
			for (uint32_t k = 0; k < C; k++)
				acc += ldexpf(s_dot[k * tile + tid],
					      s_cnt[k * tile + tid] - emax);
			site = (double)logf(acc) +
			       fma((double)emax, 0.69314718055994530942,
				   a.log_inv_c);
		}
		a.site_lnl[pp] = site;
		if (a.cat_lnl)
			for (uint32_t k = 0; k < C; k++)
				a.cat_lnl[(size_t)k * a.ldp + pp] =
					log((double)s_dot[k * tile + tid]) +
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

// Sum `count` doubles at `sums` in a fixed order: lane l of warp 0 adds
// entries l, l + 32, ... in order, then a warp-shuffle tree.  The result is
// returned in thread 0; no barrier, so only warp 0 needs to call it (s_red
// is unused).  Pairwise FP64 over a few hundred block sums loses nothing at
// the FP32 form's accuracy, and keeps the serial tail of the launch to a
// few dependent FP64 adds (the pipe runs at 1/64 of the FP32 rate here).
__device__ double block_fold(const double *sums, uint32_t count, double *s_red)
{
	(void)s_red;
	const uint32_t tid = threadIdx.x;
	if (tid >= 32)
		return 0.0;
	double sum = 0.0;
	for (uint32_t k = tid; k < count; k += 32)
		sum += __ldcg(sums + k);
	for (int off = 16; off > 0; off >>= 1)
		sum += __shfl_down_sync(0xffffffffu, sum, off);
	return sum;
}

// shared memory (byte offsets as prune4_runs_smem computes them):
// [dot: cols][cnt: cols/2][red: 32][ops][runs][tips], 16-byte aligned
// [list tables], [run table buffers: 2 * max_run * 2C * 5 float4][rates: C
// doubles, rounded up to even][eigensystem: 40 floats][lengths: 2n
// doubles], 16-byte aligned [slot partials: n_slots * cols][slot counts:
// n_slots * cols]
template <typename Idx, int kThreads>
__global__ void __launch_bounds__(kThreads, 1024 / kThreads)
	prune4_runs_kernel(PruneParams prm)
{
	const uint32_t cols = prm.tile * prm.C;
	const uint32_t tid = threadIdx.x;
	extern __shared__ __align__(16) double smem[];
	double *s_dot = smem;
	int32_t *s_cnt = (int32_t *)(smem + cols);
	double *s_red = smem + cols + (cols + 1) / 2; // one per warp
	NodeOp *s_ops = (NodeOp *)(s_red + 32);
	uint32_t *s_runs = (uint32_t *)(s_ops + prm.n);
	uint8_t *s_tips = (uint8_t *)(s_runs + ((prm.n_runs + 4) & ~3u));
	float4 *s_ptab = (float4 *)(((uintptr_t)s_tips +
				     (prm.tips_smem ? prm.num_leaves * prm.tile : 0u) + 15) &
				    ~(uintptr_t)15);
	float4 *s_tabs = s_ptab + (prm.ptab_smem ? prm.n * 2 * prm.C * 5 : 0u);
	const uint32_t tab_stride = prm.max_run * 2 * prm.C * 5;
	double *s_rate = (double *)(s_tabs + (prm.tables_inline ? 2 * tab_stride : 0u));
	float *s_eig = (float *)(s_rate + (prm.tables_inline ? (prm.C + 1) & ~1u : 0u));
	double *s_len = (double *)(s_eig + (prm.tables_inline ? 40 : 0));
	float4 *s_sp = (float4 *)(((uintptr_t)(s_len + (prm.lengths_smem ? 2 * prm.n : 0u)) +
				   15) &
				  ~(uintptr_t)15);
	int32_t *s_ss = (int32_t *)(s_sp + (size_t)prm.n_slots * cols);
	__shared__ unsigned s_last;

	if (prm.tables_inline) {
		const ModelDev *m = prm.model;
		if (tid < 16)
			s_eig[tid] = (float)m->V[tid];
		else if (tid < 32)
			s_eig[tid] = (float)m->Vinv[tid - 16];
		else if (tid < 36)
			s_eig[tid] = (float)m->lambda[tid - 32];
		else if (tid == 36)
			s_eig[36] = m->shortcuts ? 1.0f : 0.0f;
		else if (tid < 40 + prm.C && tid >= 40)
			s_rate[tid - 40] = prm.clock_rate * m->cat_rates[tid - 40];
		if (prm.lengths_smem)
			for (uint32_t k = tid; k < 2 * prm.n; k += blockDim.x)
				s_len[k] = prm.lengths[k];
	}

	const bool slots = prm.n_slots != 0;
	for (uint32_t k = tid; k < prm.n; k += blockDim.x) {
		NodeOp op = prm.ops[k];
		op.pad = slots ? prm.slots[k] : 0xFFFFFFu;
		s_ops[k] = op;
	}
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
	a.model = prm.model;
	a.lengths = prm.lengths;
	a.matrices = prm.matrices;
	RunSmem rs{};
	if (slots) {
		rs.sp = s_sp;
		rs.ss = s_ss;
	}
	if (prm.tables_inline) {
		rs.tabs = s_tabs;
		rs.tab_stride = tab_stride;
		rs.eig = s_eig;
		rs.rate = s_rate;
		rs.len = prm.lengths_smem ? s_len : nullptr;
	}
	if (prm.ptab_smem) {
		// every table row of the list, once per block (one load latency)
		const uint32_t rows = prm.n * 2 * prm.C * 5;
		for (uint32_t k = tid; k < rows; k += blockDim.x)
			s_ptab[k] = a.ptab[k];
		a.ptab = s_ptab;
	}

	__syncthreads(); // the schedule and the table sources are staged
	double cta_sum = 0.0, cta_comp = 0.0; // thread 0: this block's tiles
	const uint32_t ntiles = prm.ldp / prm.tile;
	for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const double tsum = tile_walk<Idx>(a, t, (float *)s_dot, s_cnt,
						   s_red, s_ops, s_runs, s_tips, rs);
		if (tid == 0)
			neumaier_add(cta_sum, cta_comp, tsum);
	}
	if (prm.sums_host) { // the host folds the blocks' sums
		if (tid == 0)
			prm.sums_host[blockIdx.x] =
				isfinite(cta_sum) ? cta_sum + cta_comp : cta_sum;
		return;
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
	// without a host fold the last block folds the block sums in a
	// fixed-shape tree
	__threadfence();
	const double total = block_fold(prm.block_sums, gridDim.x, s_red);
	if (tid == 0) {
		*prm.lnl_out = total;
		if (prm.lnl_host)
			*prm.lnl_host = total;
		*prm.ticket = 0u;
	}
}

// ---------------------------------------------------------------------------
// Fused evaluation of a short list in one launch (FP32, four states, kC =
// 1, 2 or 4 categories, 128-pattern tiles: one thread per column, serial
// walk).  Every block converts the device eigensystem to FP32, builds the
// list's transition tables in shared memory with the same arithmetic as the
// transition kernels (so results match a two-kernel evaluation bit for
// bit), walks its tiles, and writes its sum to host-mapped memory, which
// the host folds (with sums_host null: the last block folds the sums and
// writes the root lnL to the device and to the host-mapped word).
//
// The walk is a chain: each entry needs the previous one's output, and its
// other child is a clean partial written long ago (mostly in DRAM) or a tip
// code.  Every clean input and tip code is known before the walk starts
// (the host marks each child's source in DirectParams::src), so they are
// loaded kDirectAhead entries ahead of their use, the first ones before the
// tables are built.  The two previous outputs stay in registers; an older
// output is read back when needed (written by the same thread earlier).
// Two entries ahead fit 64 registers, so two blocks share an SM and
// several chains' launches can overlap on the same SMs.  (One, two and four
// entries ahead measured within 2 % of each other on one chain and on
// eight: the walk is not bound by these loads.)
constexpr uint32_t kDirectAhead = 2;

template <typename Idx>
__device__ __forceinline__ void direct_fetch(const NodeOp *ops, const uint8_t (*src)[2],
					     uint32_t i, uint32_t ldp,
					     const float4 *part, const int32_t *scales,
					     const uint8_t *tips_p, Idx stride, Idx col_off,
					     float4 (&v)[2], int32_t (&s)[2])
{
	const NodeOp &op = ops[i];
	const uint32_t ids[2] = {op.left, op.right};
#pragma unroll
	for (int j = 0; j < 2; ++j) {
		const uint32_t sr = src[i][j];
		if (sr == kSrcTip) {
			s[j] = tips_p[(size_t)(ids[j] & ~kTipBit) * ldp];
		} else if (sr == kSrcClean) {
			const Idx ix = (Idx)ids[j] * stride + col_off;
			v[j] = part[ix];
			s[j] = scales[ix];
		}
	}
}

// The first kDirectAhead entries' clean inputs of tile t for this thread's
// column (c, pl).
template <typename Idx, uint32_t kC>
__device__ __forceinline__ void direct_prefetch(const NodeOp *ops, const uint8_t (*src)[2],
						uint32_t n, uint32_t ldp, const uint8_t *tips,
						const float4 *part, const int32_t *scales,
						uint32_t t, float4 (&pv)[kDirectAhead][2],
						int32_t (&ps)[kDirectAhead][2])
{
	constexpr uint32_t kTile = 128;
	const uint32_t c = threadIdx.x / kTile, pl = threadIdx.x - c * kTile;
	const Idx stride = (Idx)kC * ldp;
	const Idx col_off = (Idx)c * ldp + t * kTile + pl;
	const uint8_t *tips_p = tips + t * kTile + pl;
#pragma unroll
	for (uint32_t u = 0; u < kDirectAhead; ++u)
		if (u < n)
			direct_fetch<Idx>(ops, src, u, ldp, part, scales, tips_p, stride,
					  col_off, pv[u], ps[u]);
}

// The serial walk of tile t (one thread per column) after direct_prefetch:
// leaves pi . x and the exponent of the root in s_dot / s_cnt (not
// synchronised).
template <typename Idx, uint32_t kC>
__device__ __forceinline__ void direct_walk(const NodeOp *ops, const uint8_t (*src)[2],
					    uint32_t n, uint32_t ldp, const uint8_t *tips,
					    float4 *part, int32_t *scales, const float4 *s_tab,
					    const float *s_pi, uint32_t t, float *s_dot,
					    int32_t *s_cnt, float4 (&pv)[kDirectAhead][2],
					    int32_t (&ps)[kDirectAhead][2])
{
	constexpr uint32_t kTile = 128;
	const uint32_t tid = threadIdx.x;
	const uint32_t c = tid / kTile, pl = tid - c * kTile;
	const Idx stride = (Idx)kC * ldp;
	const Idx col_off = (Idx)c * ldp + t * kTile + pl;
	const uint8_t *tips_p = tips + t * kTile + pl;
	float4 y0 = make_float4(0.f, 0.f, 0.f, 0.f), y1 = y0;
	int32_t c0 = 0, c1 = 0;
	for (uint32_t i0 = 0; i0 < n; i0 += kDirectAhead) {
#pragma unroll
		for (uint32_t u = 0; u < kDirectAhead; ++u) {
			const uint32_t i = i0 + u;
			if (i < n) {
				const NodeOp op = ops[i];
				const float4 *tl = s_tab + ((size_t)(2 * i) * kC + c) * 5;
				const float4 *tr = tl + 5 * kC;
				float4 in[2];
				int32_t sc[2];
				const uint32_t ids[2] = {op.left, op.right};
#pragma unroll
				for (int j = 0; j < 2; ++j) {
					const float4 *tb = j ? tr : tl;
					const uint32_t sr = src[i][j];
					if (sr == kSrcTip) {
						in[j] = tb[ps[u][j]];
						sc[j] = 0;
					} else {
						// the internal child's vector, then one product
						// (one copy of the code for every source)
						float4 x;
						int32_t s;
						if (sr == kSrcClean) {
							x = pv[u][j];
							s = ps[u][j];
						} else if (sr == kSrcPrev) {
							x = y0;
							s = c0;
						} else if (sr == kSrcPrev2) {
							x = y1;
							s = c1;
						} else {
							const Idx ix = (Idx)ids[j] * stride + col_off;
							x = part[ix];
							s = scales[ix];
						}
						in[j] = v4_apply(tb, x);
						sc[j] = s;
					}
				}
				// the slot just consumed takes entry i + ahead
				if (i + kDirectAhead < n)
					direct_fetch<Idx>(ops, src, i + kDirectAhead, ldp, part,
							  scales, tips_p, stride, col_off, pv[u],
							  ps[u]);
				float4 y = v4_mul(in[0], in[1]);
				const int32_t cnt = sc[0] + sc[1] + rescale_pow2(y);
				const Idx ox = (Idx)op.out * stride + col_off;
				part[ox] = y;
				scales[ox] = cnt;
				y1 = y0;
				c1 = c0;
				y0 = y;
				c0 = cnt;
			}
		}
	}
	s_dot[tid] = root_dot4(s_pi, y0);
	s_cnt[tid] = c0;
}

// The list's transition tables (entry, side, category) in shared memory,
// laid out as ptab4_kernel's, from the FP32 eigensystem in s_eig and the
// scaled category rates in s_rate (same arithmetic as the transition
// kernels).
template <uint32_t kC>
__device__ __forceinline__ void direct_tables(const ModelDev *m, const float *s_eig,
					      const double *s_rate, const double *lengths,
					      uint32_t n, float4 *s_tab)
{
	const uint32_t tid = threadIdx.x;
	if (tid < n * 2 * kC) {
		const uint32_t cc = tid % kC, es = tid / kC;
		float P[16];
		transition4f_eig(m, s_eig, lengths[es] * s_rate[cc], P);
		float *out = reinterpret_cast<float *>(s_tab + tid * 5);
		for (int k = 0; k < 4; k++)
			for (int j = 0; j < 4; j++)
				out[k * 4 + j] = P[j * 4 + k];
		for (int j = 0; j < 4; j++)
			out[16 + j] = 1.0f;
	}
}

template <typename Idx, uint32_t kC>
__global__ void __launch_bounds__(128 * kC, 8 / kC)
prune4_direct_kernel(const __grid_constant__ DirectParams prm)
{
	constexpr uint32_t kTile = 128, kCols = kTile * kC;
	__shared__ float4 s_tab[kDirectMax * 2 * kC * 5];
	__shared__ float s_eig[37];
	__shared__ double s_rate[kC];
	__shared__ float s_pi[4];
	__shared__ float s_dot[kCols];
	__shared__ int32_t s_cnt[kCols];
	__shared__ double s_red[32];
	__shared__ unsigned s_last;
	const uint32_t tid = threadIdx.x;
	const uint32_t n = prm.n;
	const uint32_t ntiles = prm.ldp / kTile;
	float4 *part = (float4 *)prm.partials;

	// clean inputs of the first entries of the first tile, in flight while
	// the tables are built
	float4 pv[kDirectAhead][2];
	int32_t ps[kDirectAhead][2];
	if (blockIdx.x < ntiles)
		direct_prefetch<Idx, kC>(prm.ops, prm.src, n, prm.ldp, prm.tips, part,
					 prm.scales, blockIdx.x, pv, ps);
	// from the parameters: no global-memory round trip before the tables
	if (tid < 37)
		s_eig[tid] = prm.eig[tid];
	else if (tid < 37 + kC)
		s_rate[tid - 37] = prm.rate[tid - 37];
	else if (tid >= 64 && tid < 68)
		s_pi[tid - 64] = (float)prm.pi[tid - 64];
	__syncthreads();
	direct_tables<kC>(prm.model, s_eig, s_rate, prm.lengths, n, s_tab);
	__syncthreads();

	TileArgs a{};
	a.pi = prm.pi;
	a.weights = prm.weights;
	a.site_lnl = prm.site_lnl;
	a.cat_lnl = nullptr;
	a.C = kC;
	a.tile = kTile;
	a.log_inv_c = prm.log_inv_c;
	double cta_sum = 0.0, cta_comp = 0.0; // thread 0: this block's tiles
	for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
		if (t != blockIdx.x)
			direct_prefetch<Idx, kC>(prm.ops, prm.src, n, prm.ldp, prm.tips,
						 part, prm.scales, t, pv, ps);
		direct_walk<Idx, kC>(prm.ops, prm.src, n, prm.ldp, prm.tips, part,
				     prm.scales, s_tab, s_pi, t, s_dot, s_cnt, pv, ps);
		__syncthreads();
		const double tsum = tile_root(a, t, s_dot, s_cnt, s_red);
		if (tid == 0)
			neumaier_add(cta_sum, cta_comp, tsum);
	}
	if (prm.sums_host) { // the host folds the blocks' sums
		if (tid == 0)
			prm.sums_host[blockIdx.x] =
				isfinite(cta_sum) ? cta_sum + cta_comp : cta_sum;
		return;
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
	__threadfence();
	const double total = block_fold(prm.block_sums, gridDim.x, s_red);
	if (tid == 0) {
		*prm.lnl_out = total;
		*prm.lnl_host = total;
		*prm.ticket = 0u;
	}
}

// Batched short lists: persistent blocks take (member, 128-pattern tile)
// items of the members whose step is direct and has kC categories from
// their own counter (work_next[1], [2], [3] for 4, 2, 1 categories;
// costliest member first); a block that moves to another
// member copies its list, classifies every child's source, converts the
// member's eigensystem to FP32 and builds the list's tables (as the
// single-calculator kernel does, so values match it), then walks the tile
// serially with clean inputs loaded four entries ahead.  Each tile's
// weighted sum goes to the member's tile slot; the block finishing a
// member's last tile folds its sums (fixed order).
template <typename Idx, uint32_t kC>
__global__ void __launch_bounds__(128 * kC, 8 / kC)
prune4_direct_batch_kernel(BatchParams bp)
{
	constexpr uint32_t kTile = 128, kCols = kTile * kC;
	constexpr uint32_t kMaxMembers = 256;
	__shared__ float4 s_tab[kDirectMax * 2 * kC * 5];
	__shared__ NodeOp s_ops[kDirectMax];
	__shared__ uint8_t s_src[kDirectMax][2];
	__shared__ float s_eig[37];
	__shared__ double s_rate[kC];
	__shared__ float s_pi[4];
	__shared__ float s_dot[kCols];
	__shared__ int32_t s_cnt[kCols];
	__shared__ double s_red[32];
	__shared__ uint32_t s_prefix[kMaxMembers + 1];
	__shared__ uint32_t s_work;
	__shared__ unsigned s_last;
	const uint32_t tid = threadIdx.x;
	const uint32_t M = bp.num_members;
	if (tid == 0) {
		uint32_t acc = 0;
		for (uint32_t m = 0; m < M; ++m) {
			s_prefix[m] = acc;
			const MemberStep &st = bp.steps[m];
			if (st.n && st.direct && bp.members[m].C == kC)
				acc += bp.members[m].ldp / kTile;
		}
		s_prefix[M] = acc;
	}
	__syncthreads();
	const uint32_t total = s_prefix[M];
	uint32_t cur = 0xFFFFFFFFu, n = 0;
	const MemberDesc *md = nullptr;
	TileArgs a{};
	a.C = kC;
	a.tile = kTile;
	a.cat_lnl = nullptr;
	float4 pv[kDirectAhead][2];
	int32_t ps[kDirectAhead][2];
	// items come in chunks of consecutive tiles (mostly of one member), so
	// that a block rebuilds a member's tables less often
	constexpr uint32_t kChunk = 4;
	for (;;) {
		if (tid == 0)
			s_work = atomicAdd(bp.work_next + (kC == 4 ? 1 : kC == 2 ? 2 : 3), kChunk);
		__syncthreads();
		const uint32_t w0 = s_work;
		__syncthreads();
		if (w0 >= total)
			break;
	for (uint32_t w = w0; w < min(w0 + kChunk, total); ++w) {
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
		md = &bp.members[m];
		if (m != cur) {
			const MemberStep st = bp.steps[m];
			n = st.n;
			const NodeOp *g_ops = (const NodeOp *)md->stage;
			for (uint32_t k = tid; k < n; k += blockDim.x)
				s_ops[k] = g_ops[k];
			const ModelDev *mod = md->model;
			if (tid < 16) {
				s_eig[tid] = (float)mod->V[tid];
				s_eig[16 + tid] = (float)mod->Vinv[tid];
			} else if (tid < 20) {
				s_eig[32 + tid - 16] = (float)mod->lambda[tid - 16];
			} else if (tid == 20) {
				s_eig[36] = mod->shortcuts ? 1.0f : 0.0f;
			} else if (tid >= 32 && tid < 32 + kC) {
				s_rate[tid - 32] = st.clock_rate * mod->cat_rates[tid - 32];
			} else if (tid >= 64 && tid < 68) {
				s_pi[tid - 64] =
					(float)((const double *)(md->stage + md->off_pi))[tid - 64];
			}
			__syncthreads();
			// where each child comes from (as the host classifies it for
			// the single-calculator kernel)
			if (tid < n) {
				const NodeOp op = s_ops[tid];
				const uint32_t ids[2] = {op.left, op.right};
				for (int j = 0; j < 2; ++j) {
					const uint32_t id = ids[j];
					uint8_t sr = kSrcClean;
					if (id & kTipBit) {
						sr = kSrcTip;
					} else if (tid >= 1 && id == s_ops[tid - 1].out) {
						sr = kSrcPrev;
					} else if (tid >= 2 && id == s_ops[tid - 2].out) {
						sr = kSrcPrev2;
					} else {
						for (uint32_t k = 0; k + 2 < tid; ++k)
							if (s_ops[k].out == id) {
								sr = kSrcEarlier;
								break;
							}
					}
					s_src[tid][j] = sr;
				}
			}
			__syncthreads();
			a.pi = (const double *)(md->stage + md->off_pi);
			a.weights = md->weights;
			a.site_lnl = md->site_lnl;
			a.ldp = md->ldp;
			a.log_inv_c = md->log_inv_c;
			direct_prefetch<Idx, kC>(s_ops, s_src, n, md->ldp, md->tips,
						 (const float4 *)md->partials, md->scales, t, pv,
						 ps);
			direct_tables<kC>(mod, s_eig, s_rate,
					  (const double *)(md->stage + md->off_in), n, s_tab);
			cur = m;
			__syncthreads();
		} else {
			direct_prefetch<Idx, kC>(s_ops, s_src, n, md->ldp, md->tips,
						 (const float4 *)md->partials, md->scales, t, pv,
						 ps);
		}
		direct_walk<Idx, kC>(s_ops, s_src, n, md->ldp, md->tips,
				     (float4 *)md->partials, md->scales, s_tab, s_pi, t,
				     s_dot, s_cnt, pv, ps);
		__syncthreads();
		const double tsum = tile_root(a, t, s_dot, s_cnt, s_red);
		const uint32_t tiles = md->ldp / kTile;
		if (tid == 0) {
			md->tile_sums[t] = tsum;
			__threadfence();
			const unsigned tk = atomicAdd(md->ticket, 1u);
			s_last = (tk == tiles - 1u);
		}
		__syncthreads();
		if (s_last) {
			__threadfence();
			const double lnl = block_fold(md->tile_sums, tiles, s_red);
			if (tid == 0) {
				bp.lnl_out[m] = lnl;
				*md->ticket = 0u;
			}
		}
		__syncthreads();
	}
	}
}

// ---------------------------------------------------------------------------
// Batched evaluation: many calculators (chains) in one launch.

__global__ void __launch_bounds__(32) ptab4_batch_kernel(BatchParams bp)
{
	const uint32_t m = blockIdx.y;
	const MemberStep st = bp.steps[m];
	if (st.n == 0 || st.direct)
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
			if (bp.steps[m].n && !bp.steps[m].direct)
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
			for (uint32_t k = tid; k < st.n; k += blockDim.x) {
				NodeOp op = g_ops[k];
				op.pad = 0xFFFFFFu; // no slots
				s_ops[k] = op;
			}
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
			tile_walk<Idx>(a, t, (float *)s_dot, s_cnt, s_red, s_ops,
				       s_runs, s_tips);
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
