// kernels4.cu -- sm_103a kernels of the 4-state (DNA) pruning likelihood.
//
//   ptab4_kernel   transition-matrix builder: P = V diag(exp(lambda d)) V^-1
//                  per (dirty node, child side, rate category), written
//                  transposed with a trailing row of ones so that both the
//                  internal-child product (sum_k x_k PT[k]) and the tip
//                  lookup (PT[code]) are one 4-vector access each.
//   prune4_kernel  Felsenstein pruning over the children-first dirty list.
//                  One thread owns one (pattern, category) column and walks
//                  the whole list, so no inter-block synchronisation exists;
//                  at the root the block mixes the categories, weights the
//                  patterns and the last block to finish folds the block
//                  sums with Neumaier compensation (no atomics on doubles,
//                  deterministic order).
//   prune4_runs_kernel / prune4_direct_kernel / prune4_batch_kernel
//                  FP32 walks of pattern tiles (runs4.cuh).
//
// The arithmetic restates the reference's CPU pruner
// (crates/b3/src/calculator/cpu4.rs:170-433): tip-tip nodes are products of
// P rows at the tip codes (unknown -> 1.0), internal children are 4x4
// matrix-vector products, and in the FP64 form a node whose four entries are
// all below e^-scale_ln is multiplied by e^scale_ln and counted.  Instead of
// the reference's per-pattern running sum, which is corrected by the flag of
// the other buffer, every slot stores the count of its whole subtree, so the
// root count is always exact, also when a proposal is evaluated twice.
#include "b3g_device.cuh"
#include "tc_ptx.cuh"

#include <cooperative_groups.h>

#include <math.h>

#include <atomic>

namespace b3g {
namespace {

namespace cg = cooperative_groups;

// ---------------------------------------------------------------------------
// 4-vectors: double4_32a (one 256-bit access) and float4 (one 128-bit access)

struct V4d {
	typedef double4_32a T;
	typedef double R;
};
struct V4f {
	typedef float4 T;
	typedef float R;
};

template <typename T, typename R>
__device__ __forceinline__ T v4_make(R x, R y, R z, R w)
{
	T r;
	r.x = x;
	r.y = y;
	r.z = z;
	r.w = w;
	return r;
}

template <typename T>
__device__ __forceinline__ T v4_mul(const T &a, const T &b)
{
	T r;
	r.x = a.x * b.x;
	r.y = a.y * b.y;
	r.z = a.z * b.z;
	r.w = a.w * b.w;
	return r;
}

// sum_k x_k * pt[k], accumulated in k order (the column order of
// cpu4.rs:386-391).
template <typename T>
__device__ __forceinline__ T v4_apply(const T *__restrict__ pt, const T &x)
{
	const T p0 = pt[0], p1 = pt[1], p2 = pt[2], p3 = pt[3];
	T r;
	r.x = x.x * p0.x;
	r.y = x.x * p0.y;
	r.z = x.x * p0.z;
	r.w = x.x * p0.w;
	r.x = fma(x.y, p1.x, r.x);
	r.y = fma(x.y, p1.y, r.y);
	r.z = fma(x.y, p1.z, r.z);
	r.w = fma(x.y, p1.w, r.w);
	r.x = fma(x.z, p2.x, r.x);
	r.y = fma(x.z, p2.y, r.y);
	r.z = fma(x.z, p2.z, r.z);
	r.w = fma(x.z, p2.w, r.w);
	r.x = fma(x.w, p3.x, r.x);
	r.y = fma(x.w, p3.y, r.y);
	r.z = fma(x.w, p3.z, r.z);
	r.w = fma(x.w, p3.w, r.w);
	return r;
}

// FP64 form (cpu4.rs:403-433): rescale by e^scale_ln when all four entries
// are below e^-scale_ln.  Returns the number of rescalings applied (0 or 1).
__device__ __forceinline__ int32_t rescale_threshold(double4_32a &y,
						     double thr, double mult)
{
	if (y.x < thr && y.y < thr && y.z < thr && y.w < thr) {
		y.x *= mult;
		y.y *= mult;
		y.z *= mult;
		y.w *= mult;
		return 1;
	}
	return 0;
}

// FP32 form: divide by the power of two that brings the largest entry into
// [1, 2).  The division is exact, so the exponent carries the scale without
// rounding.  Returns that exponent.
__device__ __forceinline__ int32_t rescale_pow2(float4 &y)
{
	float m = fmaxf(fmaxf(y.x, y.y), fmaxf(y.z, y.w));
	int32_t shift = 0;
	uint32_t ex = (__float_as_uint(m) >> 23) & 0xffu;
	if (ex == 0u) {
		if (!(m > 0.0f))
			return 0; // all zero: the pattern is impossible
		// subnormal maximum: lift by 2^64 first (exact)
		const float lift = 18446744073709551616.0f;
		y.x *= lift;
		y.y *= lift;
		y.z *= lift;
		y.w *= lift;
		shift = -64;
		m = fmaxf(fmaxf(y.x, y.y), fmaxf(y.z, y.w));
		ex = (__float_as_uint(m) >> 23) & 0xffu;
	}
	const int32_t e = (int32_t)ex - 127;
	const float f = __uint_as_float((uint32_t)(127 - e) << 23); // 2^-e
	y.x *= f;
	y.y *= f;
	y.z *= f;
	y.w *= f;
	return e + shift;
}

// ---------------------------------------------------------------------------
// transition matrices

__device__ void transition4(const ModelDev *__restrict__ m, double d,
			    double P[16])
{
	if (m->shortcuts && d > 20.0) {
		// transition_freqs (substitution.rs:245-252)
		for (int i = 0; i < 4; i++)
			for (int j = 0; j < 4; j++)
				P[i * 4 + j] = m->pi[j];
		return;
	}
	if (m->shortcuts && d < 1e-10) {
		// transition_q (substitution.rs:258-268): I + Q d, unit diagonal
		for (int i = 0; i < 4; i++)
			for (int j = 0; j < 4; j++)
				P[i * 4 + j] = i == j ? 1.0 : m->Q[i * 4 + j] * d;
		return;
	}
	double e[4];
	for (int k = 0; k < 4; k++)
		e[k] = exp(m->lambda[k] * d);
	for (int i = 0; i < 4; i++) {
		double t0 = m->V[i * 4 + 0] * e[0], t1 = m->V[i * 4 + 1] * e[1];
		double t2 = m->V[i * 4 + 2] * e[2], t3 = m->V[i * 4 + 3] * e[3];
		for (int j = 0; j < 4; j++) {
			double s = t0 * m->Vinv[0 * 4 + j];
			s = fma(t1, m->Vinv[1 * 4 + j], s);
			s = fma(t2, m->Vinv[2 * 4 + j], s);
			s = fma(t3, m->Vinv[3 * 4 + j], s);
			P[i * 4 + j] = s;
		}
	}
}

// FP32 chosen form: P(t) in single precision from the FP64 eigensystem
// (the decomposition of Q is the only FP64 work of this step; on GB300 FP64
// issues at 1/64 of the FP32 rate).  The shortcut tests stay in FP64.
// eig: V (16), Vinv (16) and lambda (4) of a four-state model, in FP32,
// then the model's shortcuts flag (nonzero: on) at eig[36], so that the
// common path reads nothing from the model in global memory.
__device__ void transition4f_eig(const ModelDev *__restrict__ m,
				 const float *__restrict__ eig, double d,
				 float P[16])
{
	const bool shortcuts = eig[36] != 0.0f;
	if (shortcuts && d > 20.0) {
		for (int i = 0; i < 4; i++)
			for (int j = 0; j < 4; j++)
				P[i * 4 + j] = (float)m->pi[j];
		return;
	}
	if (shortcuts && d < 1e-10) {
		for (int i = 0; i < 4; i++)
			for (int j = 0; j < 4; j++)
				P[i * 4 + j] = i == j ? 1.0f : (float)(m->Q[i * 4 + j] * d);
		return;
	}
	const float df = (float)d;
	float e[4];
	for (int k = 0; k < 4; k++)
		e[k] = expf(eig[32 + k] * df);
	for (int i = 0; i < 4; i++) {
		const float t0 = eig[i * 4 + 0] * e[0];
		const float t1 = eig[i * 4 + 1] * e[1];
		const float t2 = eig[i * 4 + 2] * e[2];
		const float t3 = eig[i * 4 + 3] * e[3];
		for (int j = 0; j < 4; j++) {
			float s = t0 * eig[16 + 0 * 4 + j];
			s = fmaf(t1, eig[16 + 1 * 4 + j], s);
			s = fmaf(t2, eig[16 + 2 * 4 + j], s);
			s = fmaf(t3, eig[16 + 3 * 4 + j], s);
			P[i * 4 + j] = s;
		}
	}
}

__device__ void transition4f(const ModelDev *__restrict__ m, double d,
			     float P[16])
{
	float eig[37];
	for (int k = 0; k < 16; k++) {
		eig[k] = (float)m->V[k];
		eig[16 + k] = (float)m->Vinv[k];
	}
	for (int k = 0; k < 4; k++)
		eig[32 + k] = (float)m->lambda[k];
	eig[36] = m->shortcuts ? 1.0f : 0.0f;
	transition4f_eig(m, eig, d, P);
}

template <typename R>
__global__ void __launch_bounds__(32) ptab4_kernel(PtabParams prm)
{
	const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
	if (id >= prm.n * 2u * prm.C)
		return;
	const uint32_t c = id % prm.C;
	const uint32_t es = id / prm.C; // dirty index * 2 + side
	R *out = (R *)prm.ptab + (size_t)id * 20;
	if constexpr (sizeof(R) == 4) {
		float P[16];
		if (prm.matrices) {
			const double *src = prm.matrices + (size_t)id * 16;
			for (int k = 0; k < 16; k++)
				P[k] = (float)src[k];
		} else {
			const double d = prm.lengths[es] *
					 (prm.clock_rate * prm.model->cat_rates[c]);
			transition4f(prm.model, d, P);
		}
		for (int k = 0; k < 4; k++)
			for (int j = 0; j < 4; j++)
				out[k * 4 + j] = P[j * 4 + k];
	} else {
		double P[16];
		if (prm.matrices) {
			const double *src = prm.matrices + (size_t)id * 16;
			for (int k = 0; k < 16; k++)
				P[k] = src[k];
		} else {
			const double d = prm.lengths[es] *
					 (prm.clock_rate * prm.model->cat_rates[c]);
			transition4(prm.model, d, P);
		}
		for (int k = 0; k < 4; k++)
			for (int j = 0; j < 4; j++)
				out[k * 4 + j] = (R)P[j * 4 + k];
	}
	for (int j = 0; j < 4; j++)
		out[16 + j] = (R)1.0;
}

// ---------------------------------------------------------------------------
// pruning

__device__ __forceinline__ void neumaier_add(double &sum, double &comp,
					     double x)
{
	const double t = sum + x;
	// an impossible pattern (-inf) makes the sum -inf; the compensation
	// of infinities would be NaN, so it only tracks finite sums
	if (isfinite(t)) {
		if (fabs(sum) >= fabs(x))
			comp += (sum - t) + x;
		else
			comp += (x - t) + sum;
	}
	sum = t;
}

// Per-thread constants of the pruning walk.  Partial and scale elements of
// slot `s` for this thread's (pattern, category) column sit at
// s * stride + col; table rows of entry i start at (2i) * 5C + 5c.
template <typename T, typename Idx> struct Walk {
	T *partials;
	int32_t *scales;
	const T *ptab_c;        // ptab + 5c
	const uint8_t *tips_p;  // tips + p (global) or the block's tile + pl
	Idx stride;             // C * ldp
	Idx col;                // c * ldp + p
	uint32_t tip_row;       // ldp (global) or patterns per block (tile)
	uint32_t row5c;         // 5C
};

// Inputs of one child of a node: a tip code, or a partial with the
// cumulative rescale count of its subtree.
template <typename T> struct ChildIn {
	T x;
	int32_t s;
	uint32_t code;
};

template <typename T, typename Idx>
__device__ __forceinline__ void load_child(const Walk<T, Idx> &w, uint32_t id,
					   ChildIn<T> &in)
{
	if (id & kTipBit) {
		in.code = w.tips_p[(Idx)(id & ~kTipBit) * w.tip_row];
		in.s = 0;
	} else {
		const Idx ix = (Idx)id * w.stride + w.col;
		in.x = w.partials[ix];
		in.s = w.scales[ix];
		in.code = 0;
	}
}

// P(t) applied to the child: the transposed table row of the tip code, or
// the 4x4 product with the child's partial.
template <typename T>
__device__ __forceinline__ T apply_child(uint32_t id, const T *__restrict__ pt,
					 const ChildIn<T> &in)
{
	return (id & kTipBit) ? pt[in.code] : v4_apply(pt, in.x);
}

// U consecutive schedule entries that are mutually independent: every load
// of the batch is issued before any product, so a thread keeps 2U child
// partials in flight instead of 2.
template <typename VT, bool kPow2, int U, typename Idx>
__device__ __forceinline__ void prune_batch(const PruneParams &prm,
					    const Walk<typename VT::T, Idx> &w,
					    uint32_t i0, typename VT::T &y_out,
					    int32_t &cnt_out)
{
	typedef typename VT::T T;
	NodeOp op[U];
	ChildIn<T> l[U], r[U];
#pragma unroll
	for (int u = 0; u < U; ++u) {
		op[u] = prm.ops[i0 + u];
		load_child(w, op[u].left, l[u]);
		load_child(w, op[u].right, r[u]);
	}
#pragma unroll
	for (int u = 0; u < U; ++u) {
		const T *tl = w.ptab_c + (2 * (i0 + u)) * w.row5c;
		const T *tr = tl + w.row5c;
		T y = v4_mul(apply_child(op[u].left, tl, l[u]),
			     apply_child(op[u].right, tr, r[u]));
		int32_t own;
		if constexpr (kPow2) {
			own = rescale_pow2(y);
		} else {
			// tip-tip nodes are never rescaled (cpu4.rs:288-318)
			own = ((op[u].left & op[u].right) & kTipBit)
				      ? 0
				      : rescale_threshold(y, prm.scale_threshold,
							  prm.scale_mult);
		}
		const int32_t cnt = l[u].s + r[u].s + own;
		const Idx ox = (Idx)op[u].out * w.stride + w.col;
		w.partials[ox] = y;
		w.scales[ox] = cnt;
		y_out = y;
		cnt_out = cnt;
	}
}

// Neumaier merge of two compensated partial sums.
__device__ __forceinline__ void neumaier_merge(double &sum, double &comp,
					       double sum2, double comp2)
{
	neumaier_add(sum, comp, sum2);
	if (isfinite(sum))
		comp += comp2;
}

// Root of the schedule: category mixing, pattern weights, block sum and the
// fold of all block sums by the last block to finish.  One `lead` thread per
// (pattern, category) column reports its root dot product pi . x and count;
// `pl` is the column's pattern inside the block.  Shared memory: 2 * nthr +
// 32 doubles, nthr = threads per block.
template <bool kPow2>
__device__ __forceinline__ void finish_root(const PruneParams &prm, double *smem,
					    uint32_t tp, uint32_t pl, uint32_t p,
					    uint32_t c, bool lead, double root_dot,
					    int32_t cnt)
{
	const uint32_t C = prm.C, ldp = prm.ldp;
	const uint32_t nthr = blockDim.x * blockDim.y;
	double *s_val = smem;                         // [tp * C]
	int32_t *s_exp = (int32_t *)(smem + nthr);    // [tp * C]
	double *s_warp = smem + 2 * nthr;             // [32]
	__shared__ unsigned s_last;

	if (lead) {
		if constexpr (kPow2) {
			s_val[c * tp + pl] = root_dot;
			s_exp[c * tp + pl] = cnt;
			if (prm.cat_lnl)
				prm.cat_lnl[(size_t)c * ldp + p] =
					log(root_dot) +
					(double)cnt * 0.69314718055994530942;
		} else {
			// cpu4.rs:277-284 and :63-68; the count times scale_ln
			// is an unsigned 32-bit product as in the reference
			const double lcat = log(root_dot) -
					    (double)((uint32_t)cnt * prm.scale_ln);
			s_val[c * tp + pl] = lcat;
			if (prm.cat_lnl)
				prm.cat_lnl[(size_t)c * ldp + p] = lcat;
		}
	}
	__syncthreads();

	double contrib = 0.0;
	if (c == 0 && lead) {
		double site;
		if constexpr (kPow2) {
			// sum_c s_c 2^E_c = 2^Emax sum_c s_c 2^(E_c - Emax)
			int32_t emax = INT32_MIN;
			for (uint32_t k = 0; k < C; k++)
				if (s_val[k * tp + pl] > 0.0)
					emax = max(emax, s_exp[k * tp + pl]);
			if (emax == INT32_MIN) {
				site = -INFINITY;
			} else {
				double acc = 0.0;
				for (uint32_t k = 0; k < C; k++)
					acc += scalbn(s_val[k * tp + pl],
						      s_exp[k * tp + pl] - emax);
				site = log(acc) +
				       (double)emax * 0.69314718055994530942 +
				       prm.log_inv_c;
			}
		} else {
			// log_sum_exp (likelihood/mod.rs:141-151) + ln(1/C)
			// (gamma.rs:155-165); exact identity for C = 1
			double mx = -INFINITY;
			for (uint32_t k = 0; k < C; k++)
				mx = fmax(mx, s_val[k * tp + pl]);
			if (mx == -INFINITY) {
				site = -INFINITY;
			} else {
				double se = 0.0;
				for (uint32_t k = 0; k < C; k++)
					se += exp(s_val[k * tp + pl] - mx);
				site = mx + log(se) + prm.log_inv_c;
			}
		}
		prm.site_lnl[p] = site;
		const uint32_t w = prm.weights[p];
		contrib = w ? site * (double)w : 0.0;
	}

	// block sum over the category-0 warps, in a fixed order
	const uint32_t tid = threadIdx.y * blockDim.x + threadIdx.x;
	const uint32_t lane = tid & 31u, warp = tid >> 5;
	for (int off = 16; off > 0; off >>= 1)
		contrib += __shfl_down_sync(0xffffffffu, contrib, off);
	if (c == 0 && lane == 0)
		s_warp[warp] = contrib;
	__syncthreads();
	if (tid == 0) {
		double bsum = 0.0;
		for (uint32_t w = 0; w < blockDim.x / 32u; w++)
			bsum += s_warp[w];
		prm.block_sums[blockIdx.x] = bsum;
		__threadfence();
		const unsigned t = atomicAdd(prm.ticket, 1u);
		s_last = (t == gridDim.x - 1u);
	}
	__syncthreads();
	if (!s_last)
		return;
	// The last block folds every block sum: each thread a fixed strided
	// subset with Neumaier compensation, then a fixed-shape tree in shared
	// memory, so the result does not depend on block completion order.
	__threadfence();
	double sum = 0.0, comp = 0.0;
	for (uint32_t bix = tid; bix < gridDim.x; bix += nthr)
		neumaier_add(sum, comp, __ldcg(prm.block_sums + bix));
	double *s_sum = smem;
	double *s_comp = smem + nthr;
	__syncthreads();
	s_sum[tid] = sum;
	s_comp[tid] = comp;
	__syncthreads();
	uint32_t span = 1;
	while (span < nthr)
		span <<= 1;
	for (uint32_t stride = span >> 1; stride > 0; stride >>= 1) {
		if (tid < stride && tid + stride < nthr) {
			double a = s_sum[tid], ac = s_comp[tid];
			neumaier_merge(a, ac, s_sum[tid + stride],
				       s_comp[tid + stride]);
			s_sum[tid] = a;
			s_comp[tid] = ac;
		}
		__syncthreads();
	}
	if (tid == 0) {
		const double total = s_sum[0];
		*prm.lnl_out = isfinite(total) ? total + s_comp[0] : total;
		*prm.ticket = 0u;
	}
}

template <typename VT, bool kPow2, typename Idx>
__global__ void __launch_bounds__(512) prune4_kernel(PruneParams prm)
{
	typedef typename VT::T T;
	typedef typename VT::R R;
	const uint32_t tp = blockDim.x;
	const uint32_t c = threadIdx.y;
	const uint32_t p0 = blockIdx.x * tp;
	const uint32_t p = p0 + threadIdx.x;
	const uint32_t nthr = blockDim.x * blockDim.y;
	extern __shared__ double smem[];

	Walk<T, Idx> w;
	w.partials = (T *)prm.partials;
	w.scales = prm.scales;
	w.ptab_c = (const T *)prm.ptab + 5 * c;
	w.stride = (Idx)prm.C * prm.ldp;
	w.col = (Idx)c * prm.ldp + p;
	w.row5c = 5 * prm.C;
	if (prm.tips_smem) {
		// the tip codes of this block's patterns for every leaf, staged
		// once with 4-byte loads (rows are 16-byte aligned: ldp and p0 are
		// multiples of 32)
		uint32_t *s_t32 = (uint32_t *)(smem + 2 * nthr + 32);
		const uint32_t wpr = tp >> 2;
		const uint32_t total = prm.num_leaves * wpr;
		const uint32_t tid = threadIdx.y * blockDim.x + threadIdx.x;
		for (uint32_t k = tid; k < total; k += nthr) {
			const uint32_t leaf = k / wpr, col = k - leaf * wpr;
			s_t32[k] = *(const uint32_t *)(prm.tips +
						       (size_t)leaf * prm.ldp +
						       p0 + col * 4);
		}
		__syncthreads();
		w.tips_p = (const uint8_t *)s_t32 + threadIdx.x;
		w.tip_row = tp;
	} else {
		w.tips_p = prm.tips + p;
		w.tip_row = prm.ldp;
	}

	// The schedule is split on the host into runs of mutually independent
	// entries; NodeOp::pad of an entry is the number of entries left in its
	// run (itself included).
	T y = v4_make<T, R>(0, 0, 0, 0);
	int32_t cnt = 0;
	for (uint32_t i = 0; i < prm.n;) {
		// a run never reaches past the end of the list, whatever the
		// entry says
		const uint32_t avail = min(prm.ops[i].pad, prm.n - i);
		// FP64 partials take twice the registers: batches of at most 2
		constexpr uint32_t kMaxU = sizeof(R) == 4 ? 4u : 2u;
		if (kMaxU >= 4 && avail >= 4) {
			prune_batch<VT, kPow2, 4, Idx>(prm, w, i, y, cnt);
			i += 4;
		} else if (avail >= 2) {
			prune_batch<VT, kPow2, 2, Idx>(prm, w, i, y, cnt);
			i += 2;
		} else {
			prune_batch<VT, kPow2, 1, Idx>(prm, w, i, y, cnt);
			i += 1;
		}
	}

	const double root_dot = (double)prm.pi[0] * (double)y.x +
				(double)prm.pi[1] * (double)y.y +
				(double)prm.pi[2] * (double)y.z +
				(double)prm.pi[3] * (double)y.w;
	finish_root<kPow2>(prm, smem, tp, threadIdx.x, p, c, true, root_dot, cnt);
}

// ---------------------------------------------------------------------------
// Plain FP64 form: the same walk with every child read straight from
// global memory (tip codes included) and 64-bit indices formed per access.
// On this part the FP64 arithmetic dominates; the shared-memory tip tile and
// hoisted indexing of prune4_kernel, which help the FP32 walk, measured 19 %
// slower here (1.63 against 1.36 ms per whole 256-taxon tree).
struct PlainChild {
	double4_32a x;
	int32_t s;
	uint32_t code;
};

__device__ __forceinline__ void plain_load(const PruneParams &prm,
					   const double4_32a *__restrict__ partials,
					   uint32_t id, uint32_t p, uint32_t c,
					   PlainChild &in)
{
	if (id & kTipBit) {
		in.code = prm.tips[(size_t)(id & ~kTipBit) * prm.ldp + p];
		in.s = 0;
	} else {
		const size_t ix = ((size_t)id * prm.C + c) * prm.ldp + p;
		in.x = partials[ix];
		in.s = prm.scales[ix];
		in.code = 0;
	}
}

// U consecutive mutually independent entries: every load is issued before
// any product.
template <int U>
__device__ __forceinline__ void plain_batch(const PruneParams &prm,
					    double4_32a *__restrict__ partials,
					    const double4_32a *__restrict__ ptab,
					    uint32_t i0, uint32_t p, uint32_t c,
					    double4_32a &y_out, int32_t &cnt_out)
{
	NodeOp op[U];
	PlainChild l[U], r[U];
#pragma unroll
	for (int u = 0; u < U; ++u) {
		op[u] = prm.ops[i0 + u];
		plain_load(prm, partials, op[u].left, p, c, l[u]);
		plain_load(prm, partials, op[u].right, p, c, r[u]);
	}
#pragma unroll
	for (int u = 0; u < U; ++u) {
		const uint32_t i = i0 + u;
		const double4_32a *tl = ptab + ((size_t)(2 * i) * prm.C + c) * 5;
		const double4_32a *tr = ptab + ((size_t)(2 * i + 1) * prm.C + c) * 5;
		const double4_32a a = (op[u].left & kTipBit) ? tl[l[u].code] : v4_apply(tl, l[u].x);
		const double4_32a b = (op[u].right & kTipBit) ? tr[r[u].code] : v4_apply(tr, r[u].x);
		double4_32a y = v4_mul(a, b);
		// tip-tip nodes are never rescaled (cpu4.rs:288-318)
		const int32_t own = ((op[u].left & op[u].right) & kTipBit)
					    ? 0
					    : rescale_threshold(y, prm.scale_threshold,
								prm.scale_mult);
		const int32_t cnt = l[u].s + r[u].s + own;
		const size_t ox = ((size_t)op[u].out * prm.C + c) * prm.ldp + p;
		partials[ox] = y;
		prm.scales[ox] = cnt;
		y_out = y;
		cnt_out = cnt;
	}
}

__global__ void __launch_bounds__(512) prune4_plain_kernel(PruneParams prm)
{
	const uint32_t tp = blockDim.x, c = threadIdx.y;
	const uint32_t p = blockIdx.x * tp + threadIdx.x;
	double4_32a *__restrict__ partials = (double4_32a *)prm.partials;
	const double4_32a *__restrict__ ptab = (const double4_32a *)prm.ptab;
	extern __shared__ double smem[];
	double4_32a y = v4_make<double4_32a, double>(0, 0, 0, 0);
	int32_t cnt = 0;
	for (uint32_t i = 0; i < prm.n;) {
		if (prm.ops[i].pad >= 2 && i + 1 < prm.n) {
			plain_batch<2>(prm, partials, ptab, i, p, c, y, cnt);
			i += 2;
		} else {
			plain_batch<1>(prm, partials, ptab, i, p, c, y, cnt);
			i += 1;
		}
	}
	const double root_dot = prm.pi[0] * y.x + prm.pi[1] * y.y + prm.pi[2] * y.z +
				prm.pi[3] * y.w;
	finish_root<false>(prm, smem, tp, threadIdx.x, p, c, true, root_dot, cnt);
}

// ---------------------------------------------------------------------------
#include "runs4.cuh"

// ---------------------------------------------------------------------------
#include "prune20.cuh"
#include "prune20tc.cuh"

} // namespace

cudaError_t launch_ptab4(const PtabParams &p, bool f32, cudaStream_t s)
{
	const uint32_t total = p.n * 2u * p.C;
	if (total == 0)
		return cudaSuccess;
	// one warp per block spreads the (mostly FP64/exp) work over many SMs
	const uint32_t blocks = (total + 31u) / 32u;
	if (f32)
		ptab4_kernel<float><<<blocks, 32, 0, s>>>(p);
	else
		ptab4_kernel<double><<<blocks, 32, 0, s>>>(p);
	return cudaGetLastError();
}

template <typename VT, bool kPow2>
static cudaError_t launch_prune4_t(const PruneParams &p, uint32_t tile,
				   cudaStream_t s)
{
	const dim3 grid(p.ldp / tile);
	const dim3 block(tile, p.C);
	size_t smem = sizeof(double) * (2 * (size_t)p.C * tile + 32);
	if (p.tips_smem)
		smem += (size_t)p.num_leaves * tile;
	// 32-bit element indices when every slot index fits
	const bool narrow =
		!p.wide_index && narrow_index((uint64_t)p.num_leaves * 2, p.C, p.ldp);
	auto kern = narrow ? prune4_kernel<VT, kPow2, uint32_t>
			   : prune4_kernel<VT, kPow2, size_t>;
	if (smem > 48 * 1024) {
		const cudaError_t e = cudaFuncSetAttribute(
			kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess)
			return e;
	}
	kern<<<grid, block, smem, s>>>(p);
	return cudaGetLastError();
}

cudaError_t launch_prune4(const PruneParams &p, bool f32, uint32_t tile,
			  cudaStream_t s)
{
	if (f32)
		return launch_prune4_t<V4f, true>(p, tile, s);
	const dim3 grid(p.ldp / tile), block(tile, p.C);
	const size_t smem = sizeof(double) * (2 * (size_t)p.C * tile + 32);
	prune4_plain_kernel<<<grid, block, smem, s>>>(p);
	return cudaGetLastError();
}

size_t prune4_runs_smem(const PruneParams &p)
{
	const uint32_t cols = p.tile * p.C;
	size_t off = sizeof(double) * (cols + (cols + 1) / 2 + 32) +
		     sizeof(NodeOp) * p.n + sizeof(uint32_t) * ((p.n_runs + 4) & ~3u);
	if (p.tips_smem)
		off += (size_t)p.num_leaves * p.tile;
	off = (off + 15) & ~(size_t)15;
	if (p.ptab_smem)
		off += (size_t)p.n * 2 * p.C * 5 * sizeof(float4);
	if (p.tables_inline) {
		off += 2 * (size_t)p.max_run * 2 * p.C * 5 * sizeof(float4);
		off += sizeof(double) * ((p.C + 1) & ~1u) + 40 * sizeof(float);
		if (p.lengths_smem)
			off += 2 * sizeof(double) * p.n;
	}
	if (p.n_slots) {
		off = (off + 15) & ~(size_t)15;
		off += (size_t)p.n_slots * cols * (sizeof(float4) + sizeof(int32_t));
	}
	return off;
}

cudaError_t launch_prune4_runs(const PruneParams &p, uint32_t ctas,
			       uint32_t block, cudaStream_t s)
{
	const uint32_t cols = p.tile * p.C;
	if ((block != 512 && block != 1024) || cols > 512 || p.n_slots >= kNoSlot ||
	    (block == 1024 && cols * 2 > block) ||
	    (p.n_slots && (block / cols < 2 || !p.slots)) ||
	    (p.tables_inline &&
	     (block / cols < 2 || !p.model || p.C > 16 || p.max_run == 0 ||
	      (!p.lengths && !p.matrices) || (p.lengths_smem && !p.lengths))))
		return cudaErrorInvalidValue;
	const uint32_t threads = cols * (block / cols);
	const size_t smem = prune4_runs_smem(p);
	const bool narrow = (uint64_t)p.num_leaves * 2 * p.C * p.ldp < (1ull << 31);
	auto kern = block == 1024
			    ? (narrow ? prune4_runs_kernel<uint32_t, 1024>
				      : prune4_runs_kernel<size_t, 1024>)
			    : (narrow ? prune4_runs_kernel<uint32_t, 512>
				      : prune4_runs_kernel<size_t, 512>);
	if (smem > 48 * 1024) {
		// once per (kernel variant, device): allow the device's whole
		// opt-in shared memory (a permission, not a reservation), so no
		// call lowers another's limit and later launches pay nothing
		static std::atomic<bool> opted[4][64];
		int dev = 0;
		cudaError_t e = cudaGetDevice(&dev);
		if (e != cudaSuccess)
			return e;
		const int v = (block == 1024 ? 2 : 0) + (narrow ? 0 : 1);
		if (dev < 0 || dev >= 64 || !opted[v][dev].load(std::memory_order_acquire)) {
			int most = 0;
			e = cudaDeviceGetAttribute(
				&most, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
			if (e != cudaSuccess)
				return e;
			cudaFuncAttributes fa{};
			e = cudaFuncGetAttributes(&fa, kern);
			if (e != cudaSuccess)
				return e;
			most -= (int)fa.sharedSizeBytes; // static + dynamic <= opt-in
			if ((int)smem > most)
				return cudaErrorInvalidValue;
			e = cudaFuncSetAttribute(
				kern, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
			if (e != cudaSuccess)
				return e;
			if (dev >= 0 && dev < 64)
				opted[v][dev].store(true, std::memory_order_release);
		}
	}
	kern<<<ctas, threads, smem, s>>>(p);
	return cudaGetLastError();
}

cudaError_t launch_ptab4_batch(const BatchParams &p, uint32_t max_entries,
			       cudaStream_t s)
{
	const dim3 grid((max_entries + 31u) / 32u, p.num_members);
	ptab4_batch_kernel<<<grid, 32, 0, s>>>(p);
	return cudaGetLastError();
}

cudaError_t launch_prune4_batch(const BatchParams &p, uint32_t ctas,
				cudaStream_t s)
{
	const size_t smem = sizeof(double) * (p.max_cols + (p.max_cols + 1) / 2 +
					      2 * 512) +
			    p.smem_ops_bytes + p.smem_tips_bytes + 16 + p.smem_ptab_bytes;
	auto kern = p.narrow ? prune4_batch_kernel<uint32_t>
			     : prune4_batch_kernel<size_t>;
	if (smem > 48 * 1024) {
		const cudaError_t e = cudaFuncSetAttribute(
			kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess)
			return e;
	}
	kern<<<ctas, 512, smem, s>>>(p);
	return cudaGetLastError();
}

cudaError_t launch_prune4_direct_batch(const BatchParams &p, uint32_t C,
				       uint32_t ctas, cudaStream_t s)
{
	const uint32_t threads = 128 * C;
	if (C == 4) {
		if (p.narrow)
			prune4_direct_batch_kernel<uint32_t, 4><<<ctas, threads, 0, s>>>(p);
		else
			prune4_direct_batch_kernel<size_t, 4><<<ctas, threads, 0, s>>>(p);
	} else if (C == 2) {
		if (p.narrow)
			prune4_direct_batch_kernel<uint32_t, 2><<<ctas, threads, 0, s>>>(p);
		else
			prune4_direct_batch_kernel<size_t, 2><<<ctas, threads, 0, s>>>(p);
	} else if (C == 1) {
		if (p.narrow)
			prune4_direct_batch_kernel<uint32_t, 1><<<ctas, threads, 0, s>>>(p);
		else
			prune4_direct_batch_kernel<size_t, 1><<<ctas, threads, 0, s>>>(p);
	} else {
		return cudaErrorInvalidValue;
	}
	return cudaGetLastError();
}

cudaError_t launch_ptab20(const PtabParams &p, bool f32, cudaStream_t s)
{
	const uint32_t tables = p.n * 2u * p.C;
	if (f32)
		ptab20_kernel<float><<<tables, kS20 * kS20, 0, s>>>(p);
	else
		ptab20_kernel<double><<<tables, kS20 * kS20, 0, s>>>(p);
	return cudaGetLastError();
}

template <typename R, bool kPow2>
static cudaError_t launch_prune20_t(const PruneParams &p, cudaStream_t s)
{
	const dim3 block(32, p.C), grid(p.ldp / 32);
	const size_t smem = sizeof(double) * (2 * (size_t)block.x * block.y + 32);
	const bool narrow = (uint64_t)p.num_leaves * 2 * p.C * p.ldp < (1ull << 31);
	if (narrow)
		prune20_kernel<R, kPow2, uint32_t><<<grid, block, smem, s>>>(p);
	else
		prune20_kernel<R, kPow2, size_t><<<grid, block, smem, s>>>(p);
	return cudaGetLastError();
}

cudaError_t launch_prune20(const PruneParams &p, bool f32, cudaStream_t s)
{
	if (p.C == 0 || p.C > 8 || p.ldp % 32u)
		return cudaErrorInvalidValue;
	return f32 ? launch_prune20_t<float, true>(p, s)
		   : launch_prune20_t<double, false>(p, s);
}

cudaError_t launch_ptab20tc(const PtabParams &p, float *tc_tab, cudaStream_t s)
{
	ptab20tc_kernel<<<p.n * 2u * p.C, 768, 0, s>>>(p, tc_tab);
	return cudaGetLastError();
}

size_t prune20tc_smem(uint32_t groups, bool ops_smem, uint32_t n, bool tips_smem,
		      uint32_t L)
{
	return 1024 + (size_t)groups * kTcGroup * sizeof(float) +
	       (ops_smem ? (size_t)n * sizeof(NodeOp) : 0) +
	       (tips_smem ? (size_t)L * kTcRows : 0);
}

template <uint32_t kG>
static cudaError_t launch_prune20tc_g(const Tc20Params &p, bool narrow, int smem,
				      cudaStream_t s)
{
	auto kern = narrow ? prune20tc_kernel<uint32_t, kG> : prune20tc_kernel<size_t, kG>;
	cudaError_t e = cudaFuncSetAttribute(
		kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
	if (e != cudaSuccess)
		return e;
	// grid (K, tiles, C), clusters of the K CTAs of one work item
	cudaLaunchConfig_t cfg{};
	cfg.gridDim = dim3(p.cluster, p.ldp / kTcRows, p.C);
	cfg.blockDim = dim3(128 * kG);
	cfg.dynamicSmemBytes = (size_t)smem;
	cfg.stream = s;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeClusterDimension;
	attr[0].val.clusterDim.x = p.cluster;
	attr[0].val.clusterDim.y = 1;
	attr[0].val.clusterDim.z = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	e = cudaLaunchKernelEx(&cfg, kern, p);
	if (e != cudaSuccess)
		return e;
	return cudaGetLastError();
}

cudaError_t launch_prune20tc(const Tc20Params &p, cudaStream_t s)
{
	if (p.C == 0 || p.C > 8 || p.ldp % kTcRows || p.n == 0 ||
	    (p.groups != 1 && p.groups != 2) || p.cluster < 1 || p.cluster > 8)
		return cudaErrorInvalidValue;
	const bool narrow = (uint64_t)p.L * 2 * p.C * p.ldp < (1ull << 31);
	const int smem = (int)prune20tc_smem(p.groups, p.ops_smem != 0, p.n,
					     p.tips_smem != 0, p.L);
	cudaError_t e = p.groups == 2 ? launch_prune20tc_g<2>(p, narrow, smem, s)
				      : launch_prune20tc_g<1>(p, narrow, smem, s);
	if (e != cudaSuccess)
		return e;
	finish20_kernel<<<p.ldp / kTcRows, 128, 0, s>>>(p);
	return cudaGetLastError();
}

cudaError_t launch_prune4_direct(const DirectParams &p, uint32_t ctas,
				 cudaStream_t s)
{
	if (p.n == 0 || p.n > kDirectMax || p.ldp % 128u ||
	    (p.C != 1 && p.C != 2 && p.C != 4))
		return cudaErrorInvalidValue;
	const bool narrow = (uint64_t)p.L * 2 * p.C * p.ldp < (1ull << 31);
	const uint32_t threads = 128 * p.C;
	if (p.C == 4) {
		if (narrow)
			prune4_direct_kernel<uint32_t, 4><<<ctas, threads, 0, s>>>(p);
		else
			prune4_direct_kernel<size_t, 4><<<ctas, threads, 0, s>>>(p);
	} else if (p.C == 2) {
		if (narrow)
			prune4_direct_kernel<uint32_t, 2><<<ctas, threads, 0, s>>>(p);
		else
			prune4_direct_kernel<size_t, 2><<<ctas, threads, 0, s>>>(p);
	} else {
		if (narrow)
			prune4_direct_kernel<uint32_t, 1><<<ctas, threads, 0, s>>>(p);
		else
			prune4_direct_kernel<size_t, 1><<<ctas, threads, 0, s>>>(p);
	}
	return cudaGetLastError();
}


} // namespace b3g
