// Host FP64 numerics of the engine: closed forms used as control-variate
// means, the correlation factorisation of the basket path, and the moment-sum
// estimators. Host code only; runs once per contract, never per path.
#pragma once
#include <vector>

namespace pcf {

double norm_cdf(double x);

// Black-Scholes price, discounted; pf = +1 call, -1 put.
double bs_price(double S0, double K, double r, double sigma, double T, int pf);

// Undiscounted E[payoff(G)] and E[G] for G = exp(sum_m w_m log S(t_m)), m = 0..M,
// t_m = m T / M, S a GBM with rate r and volatility sigma.
double geo_weighted_payoff_mean(double S0, double K, double r, double sigma, double T, int M,
                                const double* w, int pf, double* mean_G);

// Asian geometric control-variate weights: mode 0 trapezoid over S_0..S_M,
// mode 1 equal weights on S_1..S_M.
void asian_geo_weights(int M, int mode, std::vector<double>& w);

// Undiscounted E[payoff(G)] for the geometric basket G = exp(mean_a log S_a(T)),
// log S_a = log S0_a + (r - s_a^2/2) T + s_a ts (L z)_a, Cov(Lz) = corr.
double geo_basket_payoff_mean(int d, const double* S0, const double* sig, const double* corr,
                              double r, double T, double ts, double K, int pf);

// Lower-triangular factor F with F F^T = C (row-major, d x d). Cholesky
// (Cholesky-Banachiewicz) when C is positive definite; otherwise the
// symmetric square-root V diag(sqrt(max(l,0))) from a cyclic Jacobi
// eigen-decomposition, mirroring the LLT-then-eigen fallback of
// include/mvn.h:63-76. The fallback factor is not triangular, so it is
// returned full (is_triangular = false). Returns false if C is not
// symmetric or has a negative eigenvalue below -1e-12.
bool correlation_factor(int d, const double* C, std::vector<double>& F, bool& is_triangular);

struct Estimate {
  double price, se, price_plain, se_plain, price_cv, se_cv, beta;
};

// Estimators from moment sums s = {sum y, sum y^2, sum g, sum g^2, sum y g}
// over n paths: plain mean/SE of y and the control-variate estimate
// ybar - beta (gbar - mu_g), beta = cov(y,g)/var(g), SE from the residual
// variance var(y) - cov^2/var(g). `disc` multiplies prices and SEs.
Estimate estimate(const double* s, double n, double mu_g, double disc, bool use_cv);

}  // namespace pcf
