/*
 * b3oracle.c -- CPU oracle for the b3 pruning likelihood.  TEST
 * INFRASTRUCTURE ONLY (see b3oracle.h for what it restates and for its parity
 * status: parity unpinned against reference-produced values, pinned against
 * closed forms, matrix exponentials and brute-force enumeration).
 *
 * Every function names the reference file:line it restates.
 */
#define _GNU_SOURCE
#include "b3oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ===================================================================== */
/* EditBuf (sk/src/editbuf.rs:8-105): bit 0 selects the buffer, bit 1 says */
/* whether the slot was edited in the current epoch.                       */
/* ===================================================================== */

static inline unsigned eb_offset(const uint8_t *eb, size_t i)
{
	return eb[i] & 1u; /* editbuf.rs:25-29 */
}

static inline void eb_set_edited(uint8_t *eb, size_t i)
{
	/* editbuf.rs:71-81: an unedited slot flips its buffer and becomes
	 * edited; an edited slot keeps both bits. */
	if (!(eb[i] & 2u))
		eb[i] = (uint8_t)(((eb[i] & 1u) ^ 1u) | 2u);
}

static void eb_accept(uint8_t *eb, size_t n)
{
	for (size_t i = 0; i < n; i++) /* editbuf.rs:48-53 */
		eb[i] &= 1u;
}

static void eb_reject(uint8_t *eb, size_t n)
{
	for (size_t i = 0; i < n; i++) { /* editbuf.rs:55-65 */
		unsigned m = eb[i];
		eb[i] = (uint8_t)((m ^ (m >> 1)) & 1u);
	}
}

/* ===================================================================== */
/* A persistent worker pool that splits [0, n) into contiguous slices, as  */
/* fork_union's for_slices does for cpu4.rs:403.                           */
/* ===================================================================== */

typedef void (*slice_fn)(void *ctx, size_t start, size_t count);

typedef struct {
	pthread_t *threads;
	size_t num_threads; /* including the calling thread */
	pthread_mutex_t mu;
	pthread_cond_t go, done;
	uint64_t generation;
	size_t pending;
	int stop;
	slice_fn fn;
	void *ctx;
	size_t n;
} pool_t;

typedef struct {
	pool_t *pool;
	size_t index;
} worker_arg;

static void slice_bounds(size_t n, size_t parts, size_t index, size_t *start,
			 size_t *count)
{
	size_t base = n / parts, extra = n % parts;
	*start = index * base + (index < extra ? index : extra);
	*count = base + (index < extra ? 1 : 0);
}

static void *worker_main(void *p)
{
	worker_arg *wa = (worker_arg *)p;
	pool_t *pool = wa->pool;
	size_t index = wa->index;
	free(wa);
	uint64_t seen = 0;
	for (;;) {
		pthread_mutex_lock(&pool->mu);
		while (pool->generation == seen && !pool->stop)
			pthread_cond_wait(&pool->go, &pool->mu);
		if (pool->stop) {
			pthread_mutex_unlock(&pool->mu);
			return NULL;
		}
		seen = pool->generation;
		slice_fn fn = pool->fn;
		void *ctx = pool->ctx;
		size_t n = pool->n;
		pthread_mutex_unlock(&pool->mu);

		size_t start, count;
		slice_bounds(n, pool->num_threads, index, &start, &count);
		if (count)
			fn(ctx, start, count);

		pthread_mutex_lock(&pool->mu);
		if (--pool->pending == 0)
			pthread_cond_signal(&pool->done);
		pthread_mutex_unlock(&pool->mu);
	}
}

static void pool_init(pool_t *pool, size_t num_threads)
{
	memset(pool, 0, sizeof(*pool));
	pool->num_threads = num_threads ? num_threads : 1;
	pthread_mutex_init(&pool->mu, NULL);
	pthread_cond_init(&pool->go, NULL);
	pthread_cond_init(&pool->done, NULL);
	if (pool->num_threads > 1) {
		pool->threads = calloc(pool->num_threads - 1, sizeof(pthread_t));
		for (size_t i = 1; i < pool->num_threads; i++) {
			worker_arg *wa = malloc(sizeof(*wa));
			wa->pool = pool;
			wa->index = i;
			pthread_create(&pool->threads[i - 1], NULL, worker_main, wa);
		}
	}
}

static void pool_run(pool_t *pool, size_t n, slice_fn fn, void *ctx)
{
	if (pool->num_threads > 1) {
		pthread_mutex_lock(&pool->mu);
		pool->fn = fn;
		pool->ctx = ctx;
		pool->n = n;
		pool->pending = pool->num_threads - 1;
		pool->generation++;
		pthread_cond_broadcast(&pool->go);
		pthread_mutex_unlock(&pool->mu);
	}
	size_t start, count;
	slice_bounds(n, pool->num_threads, 0, &start, &count);
	if (count)
		fn(ctx, start, count);
	if (pool->num_threads > 1) {
		pthread_mutex_lock(&pool->mu);
		while (pool->pending)
			pthread_cond_wait(&pool->done, &pool->mu);
		pthread_mutex_unlock(&pool->mu);
	}
}

static void pool_destroy(pool_t *pool)
{
	if (pool->num_threads > 1) {
		pthread_mutex_lock(&pool->mu);
		pool->stop = 1;
		pthread_cond_broadcast(&pool->go);
		pthread_mutex_unlock(&pool->mu);
		for (size_t i = 1; i < pool->num_threads; i++)
			pthread_join(pool->threads[i - 1], NULL);
		free(pool->threads);
	}
	pthread_mutex_destroy(&pool->mu);
	pthread_cond_destroy(&pool->go);
	pthread_cond_destroy(&pool->done);
}

/* ===================================================================== */
/* Cpu4Calculator (calculator/cpu4.rs:12-166)                              */
/* ===================================================================== */

struct orc_cpu4 {
	size_t num_leaves, num_internals, num_patterns;
	uint8_t *selectors;       /* EditBuf over internals (cpu4.rs:16) */
	uint8_t *samples;         /* remapped to 0..4 (cpu4.rs:117-124) */
	double *partials;         /* [(v-L)*2 + sel][P][4] (cpu4.rs:134-136) */
	double *likelihoods;      /* [P] */
	uint8_t *scales;          /* [(v-L)*2 + sel][P] */
	uint32_t *scale_sums, *scale_sums_backup;
	uint32_t scale_ln;
	double scale_threshold, scale_mult;
	pool_t pool;
};

orc_cpu4 *orc_cpu4_new(size_t num_patterns, const uint8_t *samples,
		       size_t num_samples, uint32_t scale_ln,
		       size_t num_threads)
{
	if (num_patterns == 0 || num_samples % num_patterns)
		return NULL;
	orc_cpu4 *c = calloc(1, sizeof(*c));
	c->num_patterns = num_patterns;
	c->num_leaves = num_samples / num_patterns;
	if (c->num_leaves < 2) {
		free(c);
		return NULL;
	}
	c->num_internals = c->num_leaves - 1;
	c->samples = malloc(num_samples);
	for (size_t i = 0; i < num_samples; i++) {
		/* cpu4.rs:117-124: single bases map to 0..3, anything
		 * ambiguous (including the gap code 0b1111) to 4. */
		switch (samples[i]) {
		case 1: c->samples[i] = 0; break;
		case 2: c->samples[i] = 1; break;
		case 4: c->samples[i] = 2; break;
		case 8: c->samples[i] = 3; break;
		default: c->samples[i] = 4; break;
		}
	}
	if (num_threads == 0) { /* cpu4.rs:126-131 */
		long cores = sysconf(_SC_NPROCESSORS_ONLN);
		size_t want = (num_patterns + 999) / 1000;
		num_threads = (size_t)cores < want ? (size_t)cores : want;
		if (num_threads == 0)
			num_threads = 1;
	}
	size_t slots = c->num_internals * 2;
	c->selectors = calloc(c->num_internals, 1);
	c->partials = aligned_alloc(32, ((slots * num_patterns * 4 * sizeof(double)) + 31) / 32 * 32);
	memset(c->partials, 0, slots * num_patterns * 4 * sizeof(double));
	c->likelihoods = malloc(num_patterns * sizeof(double));
	for (size_t i = 0; i < num_patterns; i++)
		c->likelihoods[i] = NAN;
	c->scales = calloc(slots * num_patterns, 1);
	c->scale_sums = calloc(num_patterns, sizeof(uint32_t));
	c->scale_sums_backup = calloc(num_patterns, sizeof(uint32_t));
	c->scale_ln = scale_ln;
	c->scale_mult = exp((double)scale_ln);       /* cpu4.rs:141-143 */
	c->scale_threshold = exp(-(double)scale_ln);
	pool_init(&c->pool, num_threads);
	return c;
}

void orc_cpu4_free(orc_cpu4 *c)
{
	if (!c)
		return;
	pool_destroy(&c->pool);
	free(c->selectors);
	free(c->samples);
	free(c->partials);
	free(c->likelihoods);
	free(c->scales);
	free(c->scale_sums);
	free(c->scale_sums_backup);
	free(c);
}

typedef struct {
	orc_cpu4 *c;
	const uint32_t *internals, *children;
	size_t n;
	const double (*tms)[4][5]; /* [2n] padded rows (cpu4.rs:53-61) */
} propose_ctx;

/* scale (cpu4.rs:403-433) */
static inline void scale_one(double prod[4], uint8_t *scale_new,
			     const uint8_t *scale_old, uint32_t *scale_sum,
			     double threshold, double mult)
{
	int old = *scale_old;
	if (prod[0] < threshold && prod[1] < threshold &&
	    prod[2] < threshold && prod[3] < threshold) {
		for (int j = 0; j < 4; j++)
			prod[j] *= mult;
		if (!old)
			*scale_sum += 1;
		*scale_new = 1;
	} else {
		if (old)
			*scale_sum -= 1;
		*scale_new = 0;
	}
}

static void propose_slice(void *p, size_t start, size_t count)
{
	propose_ctx *ctx = (propose_ctx *)p;
	orc_cpu4 *c = ctx->c;
	const size_t P = c->num_patterns, L = c->num_leaves;

	for (size_t i = 0; i < ctx->n; i++) { /* cpu4.rs:210-275 */
		size_t v = ctx->internals[i] - L;
		uint32_t left = ctx->children[2 * i];
		uint32_t right = ctx->children[2 * i + 1];
		size_t sel = eb_offset(c->selectors, v);
		size_t out_slot = (v * 2 + sel) * P;
		size_t old_slot = (v * 2 + (sel ^ 1)) * P;
		double *out = c->partials + out_slot * 4;
		uint8_t *sc_new = c->scales + out_slot;
		const uint8_t *sc_old = c->scales + old_slot;
		const double(*tl)[5] = ctx->tms[2 * i];
		const double(*tr)[5] = ctx->tms[2 * i + 1];

		if (right < L) {
			/* calc_sample_sample (cpu4.rs:288-318): no rescale */
			const uint8_t *sl = c->samples + (size_t)left * P;
			const uint8_t *sr = c->samples + (size_t)right * P;
			for (size_t p2 = start; p2 < start + count; p2++) {
				if (sc_old[p2])
					c->scale_sums[p2] -= 1;
				sc_new[p2] = 0;
				for (int j = 0; j < 4; j++)
					out[p2 * 4 + j] =
						tl[j][sl[p2]] * tr[j][sr[p2]];
			}
		} else if (left < L) {
			/* calc_sample_partial (cpu4.rs:321-358) */
			const uint8_t *sl = c->samples + (size_t)left * P;
			size_t rv = right - L;
			const double *xr =
				c->partials +
				(rv * 2 + eb_offset(c->selectors, rv)) * P * 4;
			for (size_t p2 = start; p2 < start + count; p2++) {
				double res_r[4] = {0, 0, 0, 0};
				for (int row = 0; row < 4; row++)
					for (int col = 0; col < 4; col++)
						res_r[row] += tr[row][col] *
							      xr[p2 * 4 + col];
				double prod[4];
				for (int j = 0; j < 4; j++)
					prod[j] = tl[j][sl[p2]] * res_r[j];
				scale_one(prod, sc_new + p2, sc_old + p2,
					  c->scale_sums + p2, c->scale_threshold,
					  c->scale_mult);
				memcpy(out + p2 * 4, prod, sizeof(prod));
			}
		} else {
			/* calc_partial_partial (cpu4.rs:361-401) */
			size_t lv = left - L, rv = right - L;
			const double *xl =
				c->partials +
				(lv * 2 + eb_offset(c->selectors, lv)) * P * 4;
			const double *xr =
				c->partials +
				(rv * 2 + eb_offset(c->selectors, rv)) * P * 4;
			for (size_t p2 = start; p2 < start + count; p2++) {
				double res_l[4] = {0, 0, 0, 0};
				double res_r[4] = {0, 0, 0, 0};
				for (int row = 0; row < 4; row++)
					for (int col = 0; col < 4; col++) {
						res_l[row] += tl[row][col] *
							      xl[p2 * 4 + col];
						res_r[row] += tr[row][col] *
							      xr[p2 * 4 + col];
					}
				double prod[4];
				for (int j = 0; j < 4; j++)
					prod[j] = res_l[j] * res_r[j];
				scale_one(prod, sc_new + p2, sc_old + p2,
					  c->scale_sums + p2, c->scale_threshold,
					  c->scale_mult);
				memcpy(out + p2 * 4, prod, sizeof(prod));
			}
		}
	}
}

void orc_cpu4_propose(orc_cpu4 *c, const uint32_t *internals,
		      const uint32_t *children, size_t n,
		      const double *matrices, const double *frequencies)
{
	const size_t P = c->num_patterns, L = c->num_leaves;
	if (n == 0)
		return;
	/* cpu4.rs:53-61: each row gains a fifth entry 1.0 for unknown tips */
	double(*tms)[4][5] = malloc(2 * n * sizeof(*tms));
	for (size_t e = 0; e < 2 * n; e++)
		for (int r = 0; r < 4; r++) {
			for (int k = 0; k < 4; k++)
				tms[e][r][k] = matrices[e * 16 + r * 4 + k];
			tms[e][r][4] = 1.0;
		}
	/* set_selectors (cpu4.rs:93-98) */
	for (size_t i = 0; i < n; i++)
		eb_set_edited(c->selectors, internals[i] - L);

	propose_ctx ctx = {c, internals, children, n,
			   (const double(*)[4][5])tms};
	pool_run(&c->pool, P, propose_slice, &ctx);
	free(tms);

	/* root (cpu4.rs:277-284), then the scale correction (cpu4.rs:63-68) */
	size_t rv = internals[n - 1] - L;
	const double *xroot =
		c->partials + (rv * 2 + eb_offset(c->selectors, rv)) * P * 4;
	for (size_t p = 0; p < P; p++) {
		const double *x = xroot + p * 4;
		double s = x[0] * frequencies[0] + x[1] * frequencies[1] +
			   x[2] * frequencies[2] + x[3] * frequencies[3];
		c->likelihoods[p] = log(s);
	}
	for (size_t p = 0; p < P; p++)
		c->likelihoods[p] -= (double)(c->scale_sums[p] * c->scale_ln);
}

const double *orc_cpu4_likelihoods(const orc_cpu4 *c)
{
	return c->likelihoods;
}

void orc_cpu4_accept(orc_cpu4 *c) /* cpu4.rs:78-83 */
{
	memcpy(c->scale_sums_backup, c->scale_sums,
	       c->num_patterns * sizeof(uint32_t));
	eb_accept(c->selectors, c->num_internals);
}

void orc_cpu4_reject(orc_cpu4 *c) /* cpu4.rs:85-89 */
{
	memcpy(c->scale_sums, c->scale_sums_backup,
	       c->num_patterns * sizeof(uint32_t));
	eb_reject(c->selectors, c->num_internals);
}

size_t orc_cpu4_num_patterns(const orc_cpu4 *c)
{
	return c->num_patterns;
}

size_t orc_cpu4_num_threads(const orc_cpu4 *c)
{
	return c->pool.num_threads;
}

/* ===================================================================== */
/* likelihood/mod.rs                                                       */
/* ===================================================================== */

/* deduplicate (likelihood/mod.rs:74-132).  Columns are compared byte for
 * byte instead of through blake3 digests; the pattern order (first
 * occurrence) and the weights are the same. */
size_t orc_deduplicate(const uint8_t *msa, size_t L, size_t N,
		       uint8_t *leaves, uint32_t *weights,
		       uint32_t *site_to_pattern)
{
	uint8_t *cols = malloc(N * L > 0 ? N * L : 1); /* site-major copy */
	for (size_t s = 0; s < N; s++)
		for (size_t l = 0; l < L; l++)
			cols[s * L + l] = msa[l * N + s];
	size_t cap = 1;
	while (cap < 2 * N + 2)
		cap <<= 1;
	int64_t *table = malloc(cap * sizeof(int64_t)); /* pattern ids */
	for (size_t i = 0; i < cap; i++)
		table[i] = -1;
	size_t *first_site = malloc((N ? N : 1) * sizeof(size_t));
	size_t P = 0;
	for (size_t s = 0; s < N; s++) {
		const uint8_t *col = cols + s * L;
		uint64_t h = 1469598103934665603ull; /* FNV-1a */
		for (size_t l = 0; l < L; l++) {
			h ^= col[l];
			h *= 1099511628211ull;
		}
		size_t slot = (size_t)h & (cap - 1);
		for (;;) {
			int64_t id = table[slot];
			if (id < 0) {
				table[slot] = (int64_t)P;
				first_site[P] = s;
				weights[P] = 1;
				site_to_pattern[s] = (uint32_t)P;
				P++;
				break;
			}
			if (memcmp(cols + first_site[id] * L, col, L) == 0) {
				weights[id] += 1;
				site_to_pattern[s] = (uint32_t)id;
				break;
			}
			slot = (slot + 1) & (cap - 1);
		}
	}
	for (size_t l = 0; l < L; l++)
		for (size_t p = 0; p < P; p++) {
			uint8_t ch = msa[l * N + first_site[p]];
			leaves[l * P + p] = ch == 0 ? 0x0f : ch; /* mod.rs:117-122 */
		}
	free(cols);
	free(table);
	free(first_site);
	return P;
}

double orc_weighted_sum(const double *values, const uint32_t *weights,
			size_t n)
{
	double s = 0.0; /* likelihood/mod.rs:134-139: sum in pattern order */
	for (size_t i = 0; i < n; i++)
		s += values[i] * (double)weights[i];
	return s;
}

double orc_log_sum_exp(const double *values, size_t n)
{
	double max = -INFINITY; /* likelihood/mod.rs:141-151 */
	for (size_t i = 0; i < n; i++)
		max = fmax(max, values[i]);
	if (max == -INFINITY)
		return -INFINITY;
	double s = 0.0;
	for (size_t i = 0; i < n; i++)
		s += exp(values[i] - max);
	return max + log(s);
}

/* ===================================================================== */
/* substitution.rs                                                         */
/* ===================================================================== */

void orc_jc_transition(double d, double *out) /* substitution.rs:131-148 */
{
	double e = exp(-4.0 / 3.0 * d);
	double diag = 0.25 + 0.75 * e, other = 0.25 - 0.25 * e;
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++)
			out[i * 4 + j] = i == j ? diag : other;
}

void orc_k80_transition(double kappa, double d, double *out)
{
	/* substitution.rs:208-232 */
	double frac1 = -4.0 / (kappa + 2.0);
	double frac2 = -(2.0 * kappa + 2.0) / (kappa + 2.0);
	double arg1 = 0.25 * exp(d * frac1), arg2 = 0.5 * exp(d * frac2);
	double diag = 0.25 + arg1 + arg2;
	double ts = 0.25 + arg1 - arg2; /* A<->G, C<->T */
	double tv = 0.25 - arg1;
	for (int i = 0; i < 4; i++)
		for (int j = 0; j < 4; j++)
			out[i * 4 + j] = i == j ? diag
					 : ((i ^ j) == 2) ? ts
							  : tv;
}

void orc_hky_eigen(double kappa, const double *pi, double *V, double *Vinv,
		   double *lambda, double *Q)
{
	/* HKY::update_matrices (substitution.rs:336-388) */
	double a = pi[0], c = pi[1], g = pi[2], t = pi[3];
	double r = a + g, y = c + t;
	double q[16] = {0.0, c, kappa * g, t,  a, 0.0, g, kappa * t,
			kappa * a, c, 0.0, t,  a, kappa * c, g, 0.0};
	double div = 2.0 * (g * t + a * c + a * t + c * g +
			    kappa * (a * g + c * t));
	for (int i = 0; i < 4; i++) {
		double s = q[i * 4] + q[i * 4 + 1] + q[i * 4 + 2] + q[i * 4 + 3];
		q[i * 4 + i] = -s;
		for (int j = 0; j < 4; j++)
			q[i * 4 + j] /= div;
	}
	memcpy(Q, q, sizeof(q));
	double v[16] = {1.0, -y / r, -g / a, 0.0, 1.0, 1.0, 0.0, -t / c,
			1.0, -y / r, 1.0, 0.0,    1.0, 1.0, 0.0, 1.0};
	double vi[16] = {a,      c,      g,     t,
			 -a,     c * r / y, -g,   t * r / y,
			 -a / r, 0.0,    a / r, 0.0,
			 0.0,    -c / y, 0.0,   c / y};
	memcpy(V, v, sizeof(v));
	memcpy(Vinv, vi, sizeof(vi));
	lambda[0] = 0.0;
	lambda[1] = -1.0 / div;
	lambda[2] = -(y + r * kappa) / div;
	lambda[3] = -(r + y * kappa) / div;
}

void orc_gtr_q(const double *rates, const double *pi, double *Q)
{
	/* GTR::update_matrices (substitution.rs:502-541) */
	double a = rates[0], b = rates[1], c = rates[2], d = rates[3],
	       e = rates[4], f = rates[5];
	double pa = pi[0], pc = pi[1], pg = pi[2], pt = pi[3];
	double q[16] = {-a * pc - b * pg - c * pt, a * pc, b * pg, c * pt,
			a * pa, -a * pa - d * pg - e * pt, d * pg, e * pt,
			b * pa, d * pc, -b * pa - d * pc - f * pt, f * pt,
			c * pa, e * pc, f * pg, -c * pa - e * pc - f * pg};
	double div = 2.0 * (a * pa * pc + b * pa * pg + c * pa * pt +
			    d * pc * pg + e * pc * pt + f * pg * pt);
	for (int i = 0; i < 16; i++)
		Q[i] = q[i] / div;
}

void orc_reversible_q(int n, const double *rates, const double *pi,
		      double *Q)
{
	/* Symmetric exchangeabilities r_ij = r_ji in upper-triangle row-major
	 * order (the 4-state GTR convention of substitution.rs:507-527),
	 * Q_ij = r_ij pi_j, normalised so that -sum_i pi_i Q_ii = 1. */
	int k = 0;
	for (int i = 0; i < n; i++)
		Q[i * n + i] = 0.0;
	for (int i = 0; i < n; i++)
		for (int j = i + 1; j < n; j++, k++) {
			Q[i * n + j] = rates[k] * pi[j];
			Q[j * n + i] = rates[k] * pi[i];
		}
	double scale = 0.0;
	for (int i = 0; i < n; i++) {
		double s = 0.0;
		for (int j = 0; j < n; j++)
			if (j != i)
				s += Q[i * n + j];
		Q[i * n + i] = -s;
		scale += s * pi[i];
	}
	for (int i = 0; i < n * n; i++)
		Q[i] /= scale;
}

int orc_reversible_eigen(int n, const double *Q, const double *pi,
			 double *V, double *Vinv, double *lambda)
{
	/* Cyclic Jacobi (Golub & Van Loan, Matrix Computations, sec. 8.5) on
	 * the symmetric B = D^1/2 Q D^-1/2, D = diag(pi).  Then Q = V L V^-1
	 * with V = D^-1/2 U and V^-1 = U^T D^1/2. */
	double *B = malloc(sizeof(double) * n * n);
	double *U = malloc(sizeof(double) * n * n);
	for (int i = 0; i < n; i++)
		for (int j = 0; j < n; j++) {
			double bij = Q[i * n + j] * sqrt(pi[i]) / sqrt(pi[j]);
			double bji = Q[j * n + i] * sqrt(pi[j]) / sqrt(pi[i]);
			B[i * n + j] = 0.5 * (bij + bji);
			U[i * n + j] = i == j ? 1.0 : 0.0;
		}
	int sweep;
	for (sweep = 0; sweep < 100; sweep++) {
		double off = 0.0, tot = 0.0;
		for (int i = 0; i < n; i++)
			for (int j = 0; j < n; j++) {
				double b2 = B[i * n + j] * B[i * n + j];
				tot += b2;
				if (i != j)
					off += b2;
			}
		if (off <= 1e-34 * tot)
			break;
		for (int p = 0; p < n - 1; p++)
			for (int q = p + 1; q < n; q++) {
				double apq = B[p * n + q];
				if (apq == 0.0)
					continue;
				double theta = (B[q * n + q] - B[p * n + p]) /
					       (2.0 * apq);
				double t = (theta >= 0 ? 1.0 : -1.0) /
					   (fabs(theta) + sqrt(theta * theta + 1.0));
				double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
				for (int k = 0; k < n; k++) { /* B <- B J */
					double bkp = B[k * n + p], bkq = B[k * n + q];
					B[k * n + p] = cs * bkp - sn * bkq;
					B[k * n + q] = sn * bkp + cs * bkq;
				}
				for (int k = 0; k < n; k++) { /* B <- J^T B */
					double bpk = B[p * n + k], bqk = B[q * n + k];
					B[p * n + k] = cs * bpk - sn * bqk;
					B[q * n + k] = sn * bpk + cs * bqk;
				}
				for (int k = 0; k < n; k++) { /* U <- U J */
					double ukp = U[k * n + p], ukq = U[k * n + q];
					U[k * n + p] = cs * ukp - sn * ukq;
					U[k * n + q] = sn * ukp + cs * ukq;
				}
			}
	}
	for (int i = 0; i < n; i++) {
		lambda[i] = B[i * n + i];
		for (int j = 0; j < n; j++) {
			V[i * n + j] = U[i * n + j] / sqrt(pi[i]);
			Vinv[j * n + i] = U[i * n + j] * sqrt(pi[i]);
		}
	}
	free(B);
	free(U);
	return sweep;
}

void orc_eigen_transition(int n, const double *V, const double *Vinv,
			  const double *lambda, const double *Q,
			  const double *pi, double d, int shortcuts,
			  double *out)
{
	if (shortcuts && d > 20.0) { /* transition_freqs (:245-252) */
		for (int i = 0; i < n; i++)
			for (int j = 0; j < n; j++)
				out[i * n + j] = pi[j];
		return;
	}
	if (shortcuts && d < 1e-10) { /* transition_q (:258-268) */
		for (int i = 0; i < n; i++)
			for (int j = 0; j < n; j++)
				out[i * n + j] = Q[i * n + j] * d;
		for (int i = 0; i < n; i++)
			out[i * n + i] = 1.0;
		return;
	}
	/* mul3 (substitution.rs:79-100): (V diag(e^{lambda d})) V^-1 */
	double *tmp = malloc(sizeof(double) * n * n);
	for (int i = 0; i < n; i++)
		for (int k = 0; k < n; k++)
			tmp[i * n + k] = V[i * n + k] * exp(lambda[k] * d);
	for (int i = 0; i < n; i++)
		for (int j = 0; j < n; j++) {
			double s = 0.0;
			for (int k = 0; k < n; k++)
				s += tmp[i * n + k] * Vinv[k * n + j];
			out[i * n + j] = s;
		}
	free(tmp);
}

/* ===================================================================== */
/* Gamma categories (likelihood/gamma.rs:205-225).  The reference takes    */
/* the quantile from computare-distributions' Gamma::inverse_cdf (git rev   */
/* 02193b66, not vendored); this restates the published method: P(a, x) by */
/* its power series for x < a + 1 and by the Lentz continued fraction for  */
/* Q(a, x) otherwise (Press et al., Numerical Recipes, sec. 6.2), inverted */
/* by safeguarded Halley iterations on a bracket.                          */
/* ===================================================================== */

static double gamma_series(double a, double x)
{
	double ap = a, sum = 1.0 / a, del = sum;
	for (int n = 0; n < 10000; n++) {
		ap += 1.0;
		del *= x / ap;
		sum += del;
		if (fabs(del) < fabs(sum) * 1e-17)
			break;
	}
	return sum * exp(-x + a * log(x) - lgamma(a));
}

static double gamma_cf_q(double a, double x)
{
	const double tiny = 1e-300;
	double b = x + 1.0 - a, c = 1.0 / tiny, d = 1.0 / b, h = d;
	for (int i = 1; i < 10000; i++) {
		double an = -i * (i - a);
		b += 2.0;
		d = an * d + b;
		if (fabs(d) < tiny)
			d = tiny;
		c = b + an / c;
		if (fabs(c) < tiny)
			c = tiny;
		d = 1.0 / d;
		double del = d * c;
		h *= del;
		if (fabs(del - 1.0) < 1e-17)
			break;
	}
	return exp(-x + a * log(x) - lgamma(a)) * h;
}

double orc_gamma_p(double a, double x)
{
	if (x <= 0.0)
		return 0.0;
	if (x < a + 1.0)
		return gamma_series(a, x);
	return 1.0 - gamma_cf_q(a, x);
}

static double gamma_q(double a, double x)
{
	if (x <= 0.0)
		return 1.0;
	if (x < a + 1.0)
		return 1.0 - gamma_series(a, x);
	return gamma_cf_q(a, x);
}

double orc_gamma_p_inv(double a, double p)
{
	if (p <= 0.0)
		return 0.0;
	if (p >= 1.0)
		return INFINITY;
	/* bracket [lo, hi] with P(lo) < p < P(hi) */
	double lo = 0.0, hi = fmax(1.0, a);
	while (orc_gamma_p(a, hi) < p)
		hi *= 2.0;
	/* starting point: small-x expansion P ~ x^a / Gamma(a + 1), else
	 * the Wilson-Hilferty normal approximation */
	double x;
	if (a < 1.0) {
		x = exp((log(p) + lgamma(a + 1.0)) / a);
	} else {
		double pp = p < 0.5 ? p : 1.0 - p;
		double t = sqrt(-2.0 * log(pp));
		double z = t - (2.30753 + 0.27061 * t) /
				   (1.0 + t * (0.99229 + 0.04481 * t));
		if (p < 0.5)
			z = -z;
		double w = 1.0 - 1.0 / (9.0 * a) + z / (3.0 * sqrt(a));
		x = a * w * w * w;
	}
	if (!(x > lo && x < hi))
		x = 0.5 * (lo + hi);
	double lga = lgamma(a);
	for (int it = 0; it < 200; it++) {
		double f = p < 0.5 ? orc_gamma_p(a, x) - p
				   : (1.0 - p) - gamma_q(a, x);
		if (f < 0.0)
			lo = x;
		else
			hi = x;
		double logpdf = (a - 1.0) * log(x) - x - lga;
		double pdf = exp(logpdf);
		double xn;
		if (pdf > 0.0 && isfinite(pdf)) {
			double u = f / pdf;
			/* Halley: f'' / f' = (a - 1) / x - 1 */
			double corr = 1.0 - 0.5 * u * ((a - 1.0) / x - 1.0);
			xn = x - u / (corr > 0.1 ? corr : 1.0);
		} else {
			xn = 0.5 * (lo + hi);
		}
		if (!(xn > lo && xn < hi))
			xn = 0.5 * (lo + hi);
		if (fabs(xn - x) <= 1e-16 * fabs(xn) || hi - lo <= 4e-16 * hi) {
			x = xn;
			break;
		}
		x = xn;
	}
	return x;
}

void orc_gamma_categories(double alpha, int k, double *rates)
{
	double sum = 0.0; /* gamma.rs:205-225 */
	for (int i = 0; i < k; i++) {
		double p = (2.0 * i + 1.0) / (2.0 * k);
		rates[i] = orc_gamma_p_inv(alpha, p);
		sum += rates[i];
	}
	double mean = sum / k;
	for (int i = 0; i < k; i++)
		rates[i] = rates[i] / mean;
}
