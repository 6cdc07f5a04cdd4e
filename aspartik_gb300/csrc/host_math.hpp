// host_math.hpp -- host-side model arithmetic (Gamma rate categories).
#pragma once

namespace b3g {

// Quantile of Gamma(shape a, scale 1) at probability p.
double gamma_quantile(double a, double p);
// Median-discretised category rates normalised to mean 1
// (crates/b3/src/likelihood/gamma.rs:205-225).
void gamma_categories(double alpha, int k, double *rates);

// Analytic HKY eigensystem and normalised Q, all 4x4 row-major
// (HKY::update_matrices, crates/b3/src/substitution.rs:336-388).
void hky_eigen(double kappa, const double *pi, double *V, double *Vinv,
	       double *lambda, double *Q);

// Standard normal quantile (host, double precision).
double normal_quantile(double q);
// Median rates of k equal-probability categories of a mean-one LogNormal
// with log-scale standard deviation sd (relaxed clock,
// crates/b3/src/clock.rs:66-84).
void lognormal_categories(double sd, int k, double *rates);

constexpr int kHostMaxStates = 20;
// Reversible model of n <= kHostMaxStates states from upper-triangle
// exchangeabilities and frequencies: normalised Q and its eigensystem, all
// row-major.  Returns the Jacobi sweeps taken, or -1 without convergence.
int reversible_eigen(int n, const double *rates, const double *pi, double *V,
		     double *Vinv, double *lambda, double *Q);

} // namespace b3g
