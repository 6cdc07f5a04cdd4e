// prune20.cuh -- 20-state (protein) pruning on the CUDA cores, both forms.
// Included by kernels4.cu inside its anonymous namespace (uses finish_root,
// the Neumaier helpers and the launch plumbing there).
//
// The arithmetic generalises the reference's CPU pruner (crates/b3/src/
// calculator/cpu4.rs:170-433) from 4 to S = 20 states: a tip child
// contributes the column P[.][code] (all ones for an unknown code), an
// internal child the matrix-vector product P x, and the node is the
// element-wise product of its two children.  Tables are the transposed
// P(t) = V diag(exp(lambda t)) V^-1 of every (entry, side, category) with a
// 21st row of ones, so both child kinds read whole 20-element rows.
//
// Layouts (S = 20, R = float or double):
//   partials  R  [2I][C][ldp][20]  80 B (FP32) per (slot, category, pattern)
//   scales    i32 [2I][C][ldp]
//   ptab      R  [n][2][C][21][20]

constexpr int kS20 = 20;

// One block per table (entry, side, category), one thread per element
// P[i][j], computed in FP64 (the same for both forms: the FP32 form only
// stores it in single precision) and written transposed.
template <typename R>
__global__ void __launch_bounds__(kS20 *kS20) ptab20_kernel(PtabParams prm)
{
	constexpr int S = kS20;
	const uint32_t id = blockIdx.x; // (entry * 2 + side) * C + category
	const uint32_t c = id % prm.C, es = id / prm.C;
	const ModelDev *m = prm.model;
	const uint32_t t = threadIdx.x, i = t / S, j = t - i * S;
	__shared__ double e[S];
	double d = 0.0;
	if (!prm.matrices)
		d = prm.lengths[es] * (prm.clock_rate * m->cat_rates[c]);
	if (t < S)
		e[t] = exp(m->lambda[t] * d);
	__syncthreads();
	double P;
	if (prm.matrices) {
		P = prm.matrices[(size_t)id * S * S + t];
	} else if (m->shortcuts && d > 20.0) {
		P = m->pi[j]; // transition_freqs (substitution.rs:245-252)
	} else if (m->shortcuts && d < 1e-10) {
		// transition_q (substitution.rs:258-268): I + Q d, unit diagonal
		P = i == j ? 1.0 : m->Q[i * S + j] * d;
	} else {
		double s = 0.0;
		for (int k = 0; k < S; k++)
			s = fma(m->V[i * S + k] * e[k], m->Vinv[k * S + j], s);
		P = s;
	}
	R *out = (R *)prm.ptab + (size_t)id * (S + 1) * S;
	out[j * S + i] = (R)P;
	if (t < S)
		out[S * S + t] = (R)1.0;
}

// 20 consecutive elements (16-byte aligned) into registers.  kRO: data
// that no thread writes during the launch (tables, tips) may take the
// read-only path; partials written earlier in the walk may not.
template <bool kRO>
__device__ __forceinline__ void load20(const float *src, float v[20])
{
	const float4 *s4 = reinterpret_cast<const float4 *>(src);
#pragma unroll
	for (int q = 0; q < 5; q++) {
		const float4 a = kRO ? __ldg(s4 + q) : s4[q];
		v[4 * q] = a.x;
		v[4 * q + 1] = a.y;
		v[4 * q + 2] = a.z;
		v[4 * q + 3] = a.w;
	}
}
template <bool kRO>
__device__ __forceinline__ void load20(const double *src,
				       double v[20])
{
	const double2 *s2 = reinterpret_cast<const double2 *>(src);
#pragma unroll
	for (int q = 0; q < 10; q++) {
		const double2 a = kRO ? __ldg(s2 + q) : s2[q];
		v[2 * q] = a.x;
		v[2 * q + 1] = a.y;
	}
}
__device__ __forceinline__ void store20(float *dst, const float v[20])
{
	float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll
	for (int q = 0; q < 5; q++)
		d4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}
__device__ __forceinline__ void store20(double *dst, const double v[20])
{
	double2 *d2 = reinterpret_cast<double2 *>(dst);
#pragma unroll
	for (int q = 0; q < 10; q++)
		d2[q] = make_double2(v[2 * q], v[2 * q + 1]);
}

// One child: tip row lookup or table-times-partial (k-outer, so every
// table row is one contiguous read shared by the warp's columns).
template <typename R, typename Idx>
__device__ __forceinline__ void child20(const PruneParams &prm, uint32_t id,
					const R *__restrict__ tab, Idx stride,
					Idx col, uint32_t p, R out[20],
					int32_t &sc, bool &tip)
{
	constexpr int S = kS20;
	if (id & kTipBit) {
		const uint8_t code = prm.tips[(size_t)(id & ~kTipBit) * prm.ldp + p];
		load20<true>(tab + (size_t)code * S, out);
		sc = 0;
		tip = true;
		return;
	}
	tip = false;
	const Idx ix = (Idx)id * stride + col;
	R x[S];
	load20<false>((const R *)prm.partials + (size_t)ix * S, x);
	sc = prm.scales[ix];
	R row[S];
	load20<true>(tab, row);
#pragma unroll
	for (int i = 0; i < S; i++)
		out[i] = x[0] * row[i];
#pragma unroll
	for (int k = 1; k < S; k++) {
		load20<true>(tab + k * S, row);
#pragma unroll
		for (int i = 0; i < S; i++)
			out[i] = fma(x[k], row[i], out[i]);
	}
}

// FP32 form: exact power-of-two normalisation of the largest entry into
// [1, 2); returns the exponent (see rescale_pow2).
__device__ __forceinline__ int32_t rescale_pow2_20(float y[20])
{
	float m = y[0];
#pragma unroll
	for (int i = 1; i < 20; i++)
		m = fmaxf(m, y[i]);
	if (!(m > 0.0f))
		return 0; // all zero: the pattern is impossible
	int32_t shift = 0;
	uint32_t ex = (__float_as_uint(m) >> 23) & 0xffu;
	if (ex == 0u) { // subnormal maximum: lift by 2^64 first (exact)
		const float lift = 18446744073709551616.0f;
#pragma unroll
		for (int i = 0; i < 20; i++)
			y[i] *= lift;
		shift = -64;
		m *= lift;
		ex = (__float_as_uint(m) >> 23) & 0xffu;
	}
	const int32_t e = (int32_t)ex - 127;
	const float f = __uint_as_float((uint32_t)(127 - e) << 23); // 2^-e
#pragma unroll
	for (int i = 0; i < 20; i++)
		y[i] *= f;
	return e + shift;
}

// FP64 form (cpu4.rs:403-433 with S entries): multiply by e^scale_ln when
// every entry is below e^-scale_ln.
__device__ __forceinline__ int32_t rescale_threshold_20(double y[20], double thr,
							double mult)
{
	bool all = true;
#pragma unroll
	for (int i = 0; i < 20; i++)
		all = all && y[i] < thr;
	if (!all)
		return 0;
#pragma unroll
	for (int i = 0; i < 20; i++)
		y[i] *= mult;
	return 1;
}

// One thread per (pattern, category) column walks the whole children-first
// list.  Block (32, C): 32 patterns of every category, so the root's
// category mixing stays in the block (finish_root).
template <typename R, bool kPow2, typename Idx>
__global__ void __launch_bounds__(256) prune20_kernel(PruneParams prm)
{
	constexpr int S = kS20;
	const uint32_t tp = blockDim.x, c = threadIdx.y;
	const uint32_t p = blockIdx.x * tp + threadIdx.x;
	extern __shared__ double smem[];
	const Idx stride = (Idx)prm.C * prm.ldp;
	const Idx col = (Idx)c * prm.ldp + p;
	const size_t tab_stride = (size_t)(S + 1) * S;
	R y[S];
#pragma unroll
	for (int i = 0; i < S; i++)
		y[i] = (R)0;
	int32_t cnt = 0;
	for (uint32_t e = 0; e < prm.n; ++e) {
		const NodeOp op = prm.ops[e];
		const R *tl = (const R *)prm.ptab + ((size_t)(2 * e) * prm.C + c) * tab_stride;
		const R *tr = tl + (size_t)prm.C * tab_stride;
		R a[S], b[S];
		int32_t sa, sb;
		bool ta, tb;
		child20<R, Idx>(prm, op.left, tl, stride, col, p, a, sa, ta);
		child20<R, Idx>(prm, op.right, tr, stride, col, p, b, sb, tb);
#pragma unroll
		for (int i = 0; i < S; i++)
			y[i] = a[i] * b[i];
		int32_t own;
		if constexpr (kPow2)
			own = rescale_pow2_20(y);
		else // tip-tip nodes are never rescaled (cpu4.rs:288-318)
			own = (ta && tb) ? 0
					 : rescale_threshold_20(y, prm.scale_threshold,
								prm.scale_mult);
		cnt = sa + sb + own;
		const Idx ox = (Idx)op.out * stride + col;
		store20((R *)prm.partials + (size_t)ox * S, y);
		prm.scales[ox] = cnt;
	}
	double root_dot = 0.0;
#pragma unroll
	for (int i = 0; i < S; i++)
		root_dot = fma(prm.pi[i], (double)y[i], root_dot);
	finish_root<kPow2>(prm, smem, tp, threadIdx.x, p, c, true, root_dot, cnt);
}
