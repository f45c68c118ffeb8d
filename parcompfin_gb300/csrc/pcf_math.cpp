#include "pcf_math.h"

#include <math.h>

#include <algorithm>

namespace pcf {

double norm_cdf(double x) { return 0.5 * erfc(-x * 0.70710678118654752440); }

static double lognormal_call_put(double mu, double var, double K, int pf, double* mean_G) {
  const double fwd = exp(mu + 0.5 * var);
  if (mean_G) *mean_G = fwd;
  if (var <= 0) return std::max(pf * (fwd - K), 0.0);
  const double sd = sqrt(var);
  const double d1 = (mu - log(K) + var) / sd, d2 = d1 - sd;
  if (pf == 1) return fwd * norm_cdf(d1) - K * norm_cdf(d2);
  return K * norm_cdf(-d2) - fwd * norm_cdf(-d1);
}

double bs_price(double S0, double K, double r, double sigma, double T, int pf) {
  const double mu = log(S0) + (r - 0.5 * sigma * sigma) * T;
  return exp(-r * T) * lognormal_call_put(mu, sigma * sigma * T, K, pf, nullptr);
}

double geo_weighted_payoff_mean(double S0, double K, double r, double sigma, double T, int M,
                                const double* w, int pf, double* mean_G) {
  const double dt = T / M, nu = r - 0.5 * sigma * sigma;
  double mu = log(S0), var = 0, tail = 0;
  for (int m = 0; m <= M; ++m) mu += nu * w[m] * (m * dt);
  // Var(sum_m w_m W(t_m)) = sum_k dt_k (sum_{m>=k} w_m)^2 over increments k.
  for (int k = M; k >= 1; --k) {
    tail += w[k];
    var += dt * tail * tail;
  }
  return lognormal_call_put(mu, var * sigma * sigma, K, pf, mean_G);
}

void asian_geo_weights(int M, int mode, std::vector<double>& w) {
  w.assign((size_t)M + 1, 1.0 / M);
  if (mode == 0) {
    w[0] = 0.5 / M;
    w[M] = 0.5 / M;
  } else {
    w[0] = 0.0;
  }
}

double geo_basket_payoff_mean(int d, const double* S0, const double* sig, const double* corr,
                              double r, double T, double ts, double K, int pf) {
  double mu = 0, var = 0;
  const double w = 1.0 / d;
  for (int a = 0; a < d; ++a) {
    mu += w * (log(S0[a]) + (r - 0.5 * sig[a] * sig[a]) * T);
    for (int b = 0; b < d; ++b) var += w * w * sig[a] * sig[b] * corr[a * d + b];
  }
  return lognormal_call_put(mu, var * ts * ts, K, pf, nullptr);
}

static bool cholesky(int d, const double* C, std::vector<double>& L) {
  L.assign((size_t)d * d, 0.0);
  for (int i = 0; i < d; ++i) {
    for (int j = 0; j <= i; ++j) {
      double s = C[i * d + j];
      for (int k = 0; k < j; ++k) s -= L[i * d + k] * L[j * d + k];
      if (i == j) {
        if (!(s > 0)) return false;
        L[i * d + i] = sqrt(s);
      } else {
        L[i * d + j] = s / L[j * d + j];
      }
    }
  }
  return true;
}

// Cyclic Jacobi eigen-decomposition of a symmetric matrix (Golub & Van Loan,
// "Matrix Computations", sec. 8.5): A = V diag(l) V^T.
static void jacobi_eigen(int d, std::vector<double> A, std::vector<double>& V,
                         std::vector<double>& lam) {
  V.assign((size_t)d * d, 0.0);
  for (int i = 0; i < d; ++i) V[i * d + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < d; ++p)
      for (int q = p + 1; q < d; ++q) off += A[p * d + q] * A[p * d + q];
    if (off < 1e-30) break;
    for (int p = 0; p < d; ++p)
      for (int q = p + 1; q < d; ++q) {
        const double apq = A[p * d + q];
        if (fabs(apq) < 1e-300) continue;
        const double theta = (A[q * d + q] - A[p * d + p]) / (2 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
        const double c = 1 / sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < d; ++k) {
          const double akp = A[k * d + p], akq = A[k * d + q];
          A[k * d + p] = c * akp - s * akq;
          A[k * d + q] = s * akp + c * akq;
        }
        for (int k = 0; k < d; ++k) {
          const double apk = A[p * d + k], aqk = A[q * d + k];
          A[p * d + k] = c * apk - s * aqk;
          A[q * d + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < d; ++k) {
          const double vkp = V[k * d + p], vkq = V[k * d + q];
          V[k * d + p] = c * vkp - s * vkq;
          V[k * d + q] = s * vkp + c * vkq;
        }
      }
  }
  lam.resize(d);
  for (int i = 0; i < d; ++i) lam[i] = A[i * d + i];
}

bool correlation_factor(int d, const double* C, std::vector<double>& F, bool& is_triangular) {
  for (int i = 0; i < d; ++i)
    for (int j = 0; j < i; ++j)
      if (fabs(C[i * d + j] - C[j * d + i]) > 1e-12) return false;
  if (cholesky(d, C, F)) {
    is_triangular = true;
    return true;
  }
  std::vector<double> V, lam;
  jacobi_eigen(d, std::vector<double>(C, C + (size_t)d * d), V, lam);
  for (double l : lam)
    if (l < -1e-12) return false;
  F.assign((size_t)d * d, 0.0);
  for (int i = 0; i < d; ++i)
    for (int k = 0; k < d; ++k) F[i * d + k] = V[i * d + k] * sqrt(std::max(lam[k], 0.0));
  is_triangular = false;
  return true;
}

Estimate estimate(const double* s, double n, double mu_g, double disc, bool use_cv) {
  Estimate e;
  const double ybar = s[0] / n;
  const double vy = n > 1 ? std::max((s[1] - n * ybar * ybar) / (n - 1), 0.0) : 0.0;
  e.price_plain = disc * ybar;
  e.se_plain = disc * sqrt(vy / n);
  e.price_cv = NAN;
  e.se_cv = NAN;
  e.beta = 0;
  if (use_cv && n > 2) {
    const double gbar = s[2] / n;
    const double vg = (s[3] - n * gbar * gbar) / (n - 1);
    const double cov = (s[4] - n * ybar * gbar) / (n - 1);
    if (vg > 0) {
      e.beta = cov / vg;
      e.price_cv = disc * (ybar - e.beta * (gbar - mu_g));
      e.se_cv = disc * sqrt(std::max(vy - cov * cov / vg, 0.0) / n);
    } else {
      e.price_cv = e.price_plain;
      e.se_cv = e.se_plain;
    }
  }
  e.price = use_cv ? e.price_cv : e.price_plain;
  e.se = use_cv ? e.se_cv : e.se_plain;
  return e;
}

}  // namespace pcf
