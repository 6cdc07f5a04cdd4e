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

} // namespace b3g
