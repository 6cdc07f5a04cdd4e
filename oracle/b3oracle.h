/*
 * b3oracle.h -- CPU oracle for the b3 Felsenstein-pruning likelihood.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * implementation in aspartik_gb300/; it is called from tests/, from
 * __graft_entry__.smoke() and from bench.py's CPU-baseline leg, never from the
 * product path.
 *
 * It restates, in plain C, the reference's CPU path for the pruning likelihood
 * (kaathewisegit/aspartik, crate b3):
 *   - calculator/cpu4.rs           the pattern-sliced FP64 pruner with e^scale_ln
 *                                  rescaling and EditBuf double buffering
 *   - sk/src/editbuf.rs            the 2-bit selector state machine
 *   - likelihood/mod.rs            deduplicate, weighted_sum, log_sum_exp
 *   - likelihood/gamma.rs          median-discretised Gamma category rates
 *   - substitution.rs              JC, K80, HKY (analytic eigensystem), GTR
 *
 * Parity status: parity unpinned against outputs of the reference itself.  The
 * reference is a Rust workspace with an un-vendored git dependency and no Rust
 * toolchain exists here, and its trace-based likelihood tests read a data
 * submodule that is absent, so no reference-produced golden value exists.  The
 * oracle is instead pinned against independent ground truth: closed-form
 * transition matrices, scipy's matrix exponential, brute-force enumeration of
 * ancestral states on small trees, and scipy's inverse incomplete gamma.
 */
#ifndef B3ORACLE_H
#define B3ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- pruner (calculator/cpu4.rs) ------------------------------------- */

typedef struct orc_cpu4 orc_cpu4;

/* Cpu4Calculator::new (cpu4.rs:108-165).  `samples` is leaf-major
 * [num_leaves][num_patterns] 4-bit IUPAC codes; num_threads == 0 picks
 * min(cores, ceil(P / 1000)) as the reference does (cpu4.rs:126-131). */
orc_cpu4 *orc_cpu4_new(size_t num_patterns, const uint8_t *samples,
		       size_t num_samples, uint32_t scale_ln,
		       size_t num_threads);
void orc_cpu4_free(orc_cpu4 *c);

/* Calculator::propose (cpu4.rs:39-76).  internals[n] is the children-first
 * dirty list ending with the root, children[n][2] the sorted child pairs and
 * matrices[n][2][4][4] the row-major transition matrices of the left and right
 * child edge of each listed internal. */
void orc_cpu4_propose(orc_cpu4 *c, const uint32_t *internals,
		      const uint32_t *children, size_t n,
		      const double *matrices, const double *frequencies);
const double *orc_cpu4_likelihoods(const orc_cpu4 *c);
void orc_cpu4_accept(orc_cpu4 *c);
void orc_cpu4_reject(orc_cpu4 *c);
size_t orc_cpu4_num_patterns(const orc_cpu4 *c);
size_t orc_cpu4_num_threads(const orc_cpu4 *c);

/* ---- likelihood/mod.rs helpers --------------------------------------- */

/* deduplicate (likelihood/mod.rs:74-132).  msa is [L][N] raw codes (gap = 0).
 * Writes leaves [L][P] (gap mapped to 0b1111), weights[P] and
 * site_to_pattern[N]; returns P.  Patterns keep first-occurrence order. */
size_t orc_deduplicate(const uint8_t *msa, size_t num_sequences,
		       size_t num_sites, uint8_t *leaves, uint32_t *weights,
		       uint32_t *site_to_pattern);
double orc_weighted_sum(const double *values, const uint32_t *weights,
			size_t n);
double orc_log_sum_exp(const double *values, size_t n);

/* ---- substitution.rs -------------------------------------------------- */

void orc_jc_transition(double distance, double *out);
void orc_k80_transition(double kappa, double distance, double *out);
/* HKY::update_matrices (substitution.rs:336-388): analytic V, V^-1, lambda
 * and the normalised Q (all row-major 4x4). */
void orc_hky_eigen(double kappa, const double *pi, double *V, double *Vinv,
		   double *lambda, double *Q);
/* GTR Q (substitution.rs:502-541); rates are AC, AG, AT, CG, CT, GT. */
void orc_gtr_q(const double *rates, const double *pi, double *Q);
/* Reversible n-state Q from symmetric exchangeabilities given in
 * upper-triangle row-major order, normalised to mean rate 1. */
void orc_reversible_q(int n, const double *rates, const double *pi,
		      double *Q);
/* Eigensystem of a reversible Q through symmetric Jacobi on
 * diag(pi)^1/2 Q diag(pi)^-1/2.  Returns the number of sweeps. */
int orc_reversible_eigen(int n, const double *Q, const double *pi,
			 double *V, double *Vinv, double *lambda);
/* write_transition of HKY/GTR (substitution.rs:403-420, 571-588):
 * P = V diag(exp(lambda d)) V^-1, or the d > 20 / d < 1e-10 shortcuts when
 * `shortcuts` is non-zero. */
void orc_eigen_transition(int n, const double *V, const double *Vinv,
			  const double *lambda, const double *Q,
			  const double *pi, double distance, int shortcuts,
			  double *out);

/* ---- likelihood/gamma.rs ---------------------------------------------- */

/* Regularised lower incomplete gamma P(a, x) and its inverse. */
double orc_gamma_p(double a, double x);
double orc_gamma_p_inv(double a, double p);
/* update_categories (gamma.rs:205-225). */
void orc_gamma_categories(double alpha, int k, double *rates);

#ifdef __cplusplus
}
#endif

#endif
