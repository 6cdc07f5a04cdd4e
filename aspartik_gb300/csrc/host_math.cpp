// host_math.cpp -- host-side model arithmetic that runs only when a model
// parameter changes (never per pattern).
//
// Median-discretised Gamma rate categories (crates/b3/src/likelihood/
// gamma.rs:205-225): r_i = F^-1((2i + 1) / 2K) of Gamma(alpha, 1), then
// divided by their mean.  The reference takes F^-1 from
// computare-distributions (git rev 02193b66, not vendored); this file
// computes the regularised incomplete gamma function by its power series
// below x = a + 1 and by the modified-Lentz continued fraction of the upper
// tail above it (Press et al., Numerical Recipes, 3rd ed., sec. 6.2), and
// inverts it by Newton steps on log x kept inside a shrinking bracket.
#include "host_math.hpp"

#include <algorithm>
#include <cmath>
#include <limits>

namespace b3g {
namespace {

// returns {P(a, x), Q(a, x)}
void incomplete_gamma(double a, double x, double &P, double &Q)
{
	if (x <= 0.0) {
		P = 0.0;
		Q = 1.0;
		return;
	}
	const double log_front = a * std::log(x) - x - std::lgamma(a);
	if (x < a + 1.0) {
		double term = 1.0 / a, sum = term, ap = a;
		for (int n = 0; n < 100000; ++n) {
			ap += 1.0;
			term *= x / ap;
			sum += term;
			if (std::fabs(term) <= std::fabs(sum) * 1e-17)
				break;
		}
		P = sum * std::exp(log_front);
		Q = 1.0 - P;
	} else {
		const double tiny = 1e-300;
		double b = x + 1.0 - a;
		double c = 1.0 / tiny;
		double d = 1.0 / b;
		double h = d;
		for (int i = 1; i < 100000; ++i) {
			const double an = -static_cast<double>(i) * (i - a);
			b += 2.0;
			d = an * d + b;
			if (std::fabs(d) < tiny)
				d = tiny;
			c = b + an / c;
			if (std::fabs(c) < tiny)
				c = tiny;
			d = 1.0 / d;
			const double delta = d * c;
			h *= delta;
			if (std::fabs(delta - 1.0) <= 1e-17)
				break;
		}
		Q = std::exp(log_front) * h;
		P = 1.0 - Q;
	}
}

} // namespace

double gamma_quantile(double a, double p)
{
	if (!(a > 0.0) || !(p >= 0.0) || !(p <= 1.0))
		return std::numeric_limits<double>::quiet_NaN();
	if (p == 0.0)
		return 0.0;
	if (p == 1.0)
		return std::numeric_limits<double>::infinity();
	const bool lower = p <= 0.5;
	const double target = lower ? p : 1.0 - p;
	// residual in the better-conditioned tail
	auto residual = [&](double x) {
		double P, Q;
		incomplete_gamma(a, x, P, Q);
		return lower ? P - target : target - Q;
	};
	double lo = 0.0, hi = a > 1.0 ? a : 1.0;
	while (residual(hi) < 0.0)
		hi *= 4.0;
	// start: P ~ x^a / Gamma(a + 1) for small x, else the mean
	double x = std::exp((std::log(p) + std::lgamma(a + 1.0)) / a);
	if (!(x > lo && x < hi))
		x = 0.5 * (lo + hi);
	const double lga = std::lgamma(a);
	for (int it = 0; it < 300; ++it) {
		const double f = residual(x);
		if (f < 0.0)
			lo = x;
		else
			hi = x;
		// Newton on u = log x: dP/du = x pdf(x)
		const double dens = std::exp(a * std::log(x) - x - lga);
		double next;
		if (dens > 0.0 && std::isfinite(dens)) {
			next = x * std::exp(-f / dens);
		} else {
			next = 0.5 * (lo + hi);
		}
		if (!(next > lo && next < hi))
			next = 0.5 * (lo + hi);
		if (std::fabs(next - x) <= 2e-16 * next) {
			x = next;
			break;
		}
		x = next;
	}
	return x;
}

void hky_eigen(double kappa, const double *pi, double *V, double *Vinv,
	       double *lambda, double *Q)
{
	const double a = pi[0], c = pi[1], g = pi[2], t = pi[3];
	const double r = a + g, y = c + t;
	// unnormalised off-diagonal rates, rows A C G T
	const double q[16] = {0.0,       c,         kappa * g, t,
			      a,         0.0,       g,         kappa * t,
			      kappa * a, c,         0.0,       t,
			      a,         kappa * c, g,         0.0};
	const double div = 2.0 * (g * t + a * c + a * t + c * g +
				  kappa * (a * g + c * t));
	for (int i = 0; i < 4; ++i) {
		const double rs = q[i * 4] + q[i * 4 + 1] + q[i * 4 + 2] + q[i * 4 + 3];
		for (int j = 0; j < 4; ++j)
			Q[i * 4 + j] = (i == j ? -rs : q[i * 4 + j]) / div;
	}
	const double v[16] = {1.0, -y / r, -g / a, 0.0,    1.0, 1.0, 0.0, -t / c,
			      1.0, -y / r, 1.0,    0.0,    1.0, 1.0, 0.0, 1.0};
	const double vi[16] = {a,      c,          g,     t,
			       -a,     c * r / y,  -g,    t * r / y,
			       -a / r, 0.0,        a / r, 0.0,
			       0.0,    -c / y,     0.0,   c / y};
	for (int k = 0; k < 16; ++k) {
		V[k] = v[k];
		Vinv[k] = vi[k];
	}
	lambda[0] = 0.0;
	lambda[1] = -1.0 / div;
	lambda[2] = -(y + r * kappa) / div;
	lambda[3] = -(r + y * kappa) / div;
}

void gamma_categories(double alpha, int k, double *rates)
{
	double sum = 0.0;
	for (int i = 0; i < k; ++i) {
		const double p = (2.0 * i + 1.0) / (2.0 * k);
		rates[i] = gamma_quantile(alpha, p);
		sum += rates[i];
	}
	const double mean = sum / k;
	for (int i = 0; i < k; ++i)
		rates[i] = rates[i] / mean;
}


// Standard normal quantile: bisection-safeguarded Newton steps on
// Phi(x) = erfc(-x / sqrt 2) / 2 from a logistic start, on the lower half
// (Phi^-1(q) = -Phi^-1(1 - q) above 1/2, so the residual never cancels).
double normal_quantile(double q)
{
	if (!(q > 0.0))
		return -std::numeric_limits<double>::infinity();
	if (!(q < 1.0))
		return std::numeric_limits<double>::infinity();
	if (q > 0.5)
		return -normal_quantile(1.0 - q);
	if (q == 0.5)
		return 0.0;
	const double pi = 3.14159265358979323846;
	double lo = -40.0, hi = 0.0;
	double x = std::max(lo, std::sqrt(pi / 8.0) * std::log(q / (1.0 - q)));
	for (int it = 0; it < 200; ++it) {
		const double cdf = 0.5 * std::erfc(-x / std::sqrt(2.0));
		if (cdf < q)
			lo = x;
		else
			hi = x;
		const double pdf = std::exp(-0.5 * x * x) / std::sqrt(2.0 * pi);
		double next = x - (cdf - q) / pdf;
		if (!(next > lo && next < hi) || pdf == 0.0)
			next = 0.5 * (lo + hi);
		if (std::fabs(next - x) <= 1e-15 * std::max(1.0, std::fabs(x)))
			return next;
		x = next;
	}
	return x;
}

// Relaxed-clock rates (RelaxedClock::update_rates, crates/b3/src/clock.rs:
// 66-84): the quantiles at (i + 1/2) / k of a LogNormal with mean one and
// log-scale standard deviation sd (mu = -sd^2 / 2).
void lognormal_categories(double sd, int k, double *rates)
{
	const double mu = -0.5 * sd * sd;
	for (int i = 0; i < k; ++i)
		rates[i] = std::exp(mu + sd * normal_quantile((i + 0.5) / k));
}

// Reversible Q from exchangeabilities and frequencies, normalised to mean
// rate 1 (GTR::update_matrices, crates/b3/src/substitution.rs:502-555), and
// its eigensystem through the symmetric matrix B = Pi^1/2 Q Pi^-1/2: cyclic
// Jacobi rotations (Golub & Van Loan, Matrix Computations, 4th ed., sec.
// 8.5) until the off-diagonal norm is below 1e-17 of the total.  Then
// Q = V diag(lambda) V^-1 with V = Pi^-1/2 U and V^-1 = U^T Pi^1/2.
int reversible_eigen(int n, const double *rates, const double *pi, double *V,
		     double *Vinv, double *lambda, double *Q)
{
	double sq[kHostMaxStates];
	double B[kHostMaxStates * kHostMaxStates];
	double U[kHostMaxStates * kHostMaxStates];
	int k = 0;
	for (int a = 0; a < n; a++) {
		Q[a * n + a] = 0.0;
		for (int b = a + 1; b < n; b++, k++) {
			Q[a * n + b] = rates[k] * pi[b];
			Q[b * n + a] = rates[k] * pi[a];
		}
	}
	double scale = 0.0;
	for (int a = 0; a < n; a++) {
		double rsum = 0.0;
		for (int b = 0; b < n; b++)
			if (b != a)
				rsum += Q[a * n + b];
		Q[a * n + a] = -rsum;
		scale += rsum * pi[a];
	}
	for (int a = 0; a < n; a++) {
		sq[a] = std::sqrt(pi[a]);
		for (int b = 0; b < n; b++)
			Q[a * n + b] /= scale;
	}
	for (int a = 0; a < n; a++)
		for (int b = 0; b < n; b++) {
			B[a * n + b] = 0.5 * (Q[a * n + b] * sq[a] / sq[b] +
					      Q[b * n + a] * sq[b] / sq[a]);
			U[a * n + b] = a == b ? 1.0 : 0.0;
		}
	int sweep = 0;
	for (; sweep < 50; ++sweep) {
		double off = 0.0, tot = 0.0;
		for (int a = 0; a < n; a++)
			for (int b = 0; b < n; b++) {
				const double b2 = B[a * n + b] * B[a * n + b];
				tot += b2;
				if (a != b)
					off += b2;
			}
		if (off <= 1e-34 * tot)
			break;
		for (int p = 0; p < n - 1; p++)
			for (int q = p + 1; q < n; q++) {
				const double apq = B[p * n + q];
				if (apq == 0.0)
					continue;
				const double theta = (B[q * n + q] - B[p * n + p]) / (2.0 * apq);
				const double t = (theta >= 0.0 ? 1.0 : -1.0) /
						 (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
				const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
				for (int r = 0; r < n; r++) { // B J
					const double bp = B[r * n + p], bq = B[r * n + q];
					B[r * n + p] = c * bp - s * bq;
					B[r * n + q] = s * bp + c * bq;
				}
				for (int r = 0; r < n; r++) { // J^T (B J)
					const double bp = B[p * n + r], bq = B[q * n + r];
					B[p * n + r] = c * bp - s * bq;
					B[q * n + r] = s * bp + c * bq;
				}
				B[p * n + q] = B[q * n + p] = 0.0;
				for (int r = 0; r < n; r++) { // U J
					const double up = U[r * n + p], uq = U[r * n + q];
					U[r * n + p] = c * up - s * uq;
					U[r * n + q] = s * up + c * uq;
				}
			}
	}
	for (int i = 0; i < n; i++) {
		lambda[i] = B[i * n + i];
		for (int j = 0; j < n; j++) {
			V[i * n + j] = U[i * n + j] / sq[i];
			Vinv[j * n + i] = U[i * n + j] * sq[i];
		}
	}
	return sweep < 50 ? sweep : -1;
}

} // namespace b3g
