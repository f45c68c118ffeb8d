/* pcf_oracle -- CPU restatement of moledoc/parcompfin's pricing hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA engine in
 * parcompfin_gb300/. Only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py load it. No product code path may call it.
 *
 * Three kinds of function live here:
 *   1. ref_* -- restatements of the reference's own functions, with the same
 *      generator (std::mt19937 + std::normal_distribution from libstdc++) and
 *      the same floating-point operation order. Each one cites the reference
 *      file:line it follows. Given the seed that the reference takes from
 *      time(), they reproduce its output; tests/golden/ref_outputs.json
 *      (written by running the reference itself, oracle/build_ref.sh) pins
 *      that claim.
 *   2. twin_* -- FP64 twins of the GPU kernels. They consume the identical
 *      Philox4x32-10 draws (philox_host.h) and return the same moment sums the
 *      kernels return, so the deterministic-draw parity is checkable.
 *   3. closed forms -- Black-Scholes and the geometric-average lognormal
 *      closed form (any monitoring weights), used as known answers and as the
 *      control-variate means.
 *
 * Build: g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -shared -fPIC.
 * -ffp-contract=off keeps a*b+c as two roundings on every host architecture,
 * which is what the reference compiles to on x86-64.
 */
#include <stdint.h>
#include <math.h>
#include <string.h>
#include <algorithm>
#include <random>
#include <vector>
#include <omp.h>

#include "philox_host.h"

#define ORC_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

/* include/common.h:56-60 -- payoff(St,E,payoff_fun) = max(pf*(St-E), 0) with an
 * int payoff_fun (the callers pass a double that converts to int). */
inline double payoff(double St, double E, int pf) { return std::max(pf * (St - E), 0.0); }

/* include/common.h:63-72 -- log C(N,i) in one FP64 accumulator: +log n for
 * n = N..i+1, then -log j for j = 2..N-i. logtab[n] holds log((double)n),
 * which is what the reference calls in the loop. */
double comb_ref(int N, int i, const double* logtab) {
  if (i == 0 || i == N) return 0;
  if (i == 1 || i == (N - 1)) return logtab[N];
  double result = 0;
  for (int n = N; n > i; --n) result += logtab[n];
  for (int j = 2; j <= (N - i); ++j) result -= logtab[j];
  return result;
}

std::vector<double> make_logtab(int N) {
  std::vector<double> t((size_t)N + 1);
  t[0] = -INFINITY;
  for (int n = 1; n <= N; ++n) t[n] = log((double)n);
  return t;
}

/* The beta-parametrised lattice, src/binom_embar.cpp:19-27 (identical in
 * src/binom_vanilla_eur.cpp:14-22 and src/binom_vanilla_amer.cpp:14-22). */
struct Lattice { double dt, beta, u, d, R, p, q; };
Lattice lattice(double r, double sigma, double T, int N) {
  Lattice L;
  L.dt = (double)T / (double)N;
  L.beta = 0.5 * (exp(-r * L.dt) + exp((r + pow(sigma, 2)) * L.dt));
  L.u = L.beta + sqrt(pow(L.beta, 2) - 1);
  L.d = L.beta - sqrt(pow(L.beta, 2) - 1);
  L.R = exp(r * L.dt);
  L.p = (L.R - L.d) / (L.u - L.d);
  L.q = 1 - L.p;
  return L;
}

double norm_cdf(double x) { return 0.5 * erfc(-x * 0.70710678118654752440); }

}  // namespace

/* ------------------------------------------------------------------------ */
/* Philox and normals (philox_host.h), exported for the known-answer tests.  */
/* ------------------------------------------------------------------------ */
ORC_EXPORT void orc_philox4x32_10(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  orc::philox4x32_10(ctr, key, out);
}

ORC_EXPORT void orc_normals4(uint64_t seed, uint32_t stream, uint32_t tag, uint64_t quad,
                             uint32_t step, double* z) {
  orc::normals4(seed, stream, tag, quad, step, z);
}

/* ------------------------------------------------------------------------ */
/* Closed forms                                                              */
/* ------------------------------------------------------------------------ */
ORC_EXPORT double orc_bs_price(double S0, double E, double r, double sigma, double T, int pf) {
  const double sd = sigma * sqrt(T);
  const double d1 = (log(S0 / E) + (r + 0.5 * sigma * sigma) * T) / sd;
  const double d2 = d1 - sd;
  if (pf == 1) return S0 * norm_cdf(d1) - E * exp(-r * T) * norm_cdf(d2);
  return E * exp(-r * T) * norm_cdf(-d2) - S0 * norm_cdf(-d1);
}

/* Discounted E[payoff(G)] for G = exp(sum_m w[m] log S(t_m)), t_m = m*T/M,
 * m = 0..M, under GBM. log G is normal with mean log S0 + nu*sum w_m t_m and
 * variance sigma^2 * sum_k dt * (sum_{m>=k} w_m)^2. Also returns E[G]
 * (undiscounted) in *mean_G when non-null. */
ORC_EXPORT double orc_geo_weighted_price(double S0, double E, double r, double sigma, double T,
                                         int M, const double* w, int pf, double* mean_G) {
  const double dt = T / M, nu = r - 0.5 * sigma * sigma;
  double mu = log(S0), tail = 0, var = 0, wsum = 0;
  for (int m = 0; m <= M; ++m) { mu += nu * w[m] * (m * dt); wsum += w[m]; }
  (void)wsum;
  for (int k = M; k >= 1; --k) { tail += w[k]; var += dt * tail * tail; }
  var *= sigma * sigma;
  const double fwd = exp(mu + 0.5 * var);
  if (mean_G) *mean_G = fwd;
  const double disc = exp(-r * T);
  if (var <= 0) return disc * std::max(pf * (fwd - E), 0.0);
  const double sd = sqrt(var);
  const double d1 = (mu - log(E) + var) / sd, d2 = d1 - sd;
  if (pf == 1) return disc * (fwd * norm_cdf(d1) - E * norm_cdf(d2));
  return disc * (E * norm_cdf(-d2) - fwd * norm_cdf(-d1));
}

/* Monitoring weights of the geometric control variate for the Asian kernel.
 * mode 0 (the reference's running average, src/mc_asia.cpp:31-35, which is a
 * trapezoid rule over S_0..S_M to first order): w_0 = w_M = 1/(2M), else 1/M.
 * mode 1 (discrete mean of S_1..S_M): w_0 = 0, w_m = 1/M. */
ORC_EXPORT void orc_asian_geo_weights(int M, int mode, double* w) {
  for (int m = 0; m <= M; ++m) w[m] = 1.0 / M;
  if (mode == 0) { w[0] = 0.5 / M; w[M] = 0.5 / M; }
  else w[0] = 0.0;
}

ORC_EXPORT double orc_geo_asian_price(double S0, double E, double r, double sigma, double T,
                                      int M, int mode, int pf, double* mean_G) {
  std::vector<double> w((size_t)M + 1);
  orc_asian_geo_weights(M, mode, w.data());
  return orc_geo_weighted_price(S0, E, r, sigma, T, M, w.data(), pf, mean_G);
}

/* Geometric basket: log G = sum_a w_a log S_a(T) with S_a = S0_a exp((r -
 * s_a^2/2)T + s_a*ts*(Lz)_a). var = ts^2 * sum_ab w_a w_b s_a s_b C_ab. */
ORC_EXPORT double orc_geo_basket_price(int d, const double* S0, const double* sig,
                                       const double* corr, double r, double T, double ts,
                                       double E, int pf, double* mean_G) {
  double mu = 0, var = 0;
  const double w = 1.0 / d;
  for (int a = 0; a < d; ++a) {
    mu += w * (log(S0[a]) + (r - 0.5 * sig[a] * sig[a]) * T);
    for (int b = 0; b < d; ++b) var += w * w * sig[a] * sig[b] * corr[a * d + b];
  }
  var *= ts * ts;
  const double fwd = exp(mu + 0.5 * var);
  if (mean_G) *mean_G = fwd;
  const double disc = exp(-r * T), sd = sqrt(var);
  const double d1 = (mu - log(E) + var) / sd, d2 = d1 - sd;
  if (pf == 1) return disc * (fwd * norm_cdf(d1) - E * norm_cdf(d2));
  return disc * (E * norm_cdf(-d2) - fwd * norm_cdf(-d1));
}

/* ------------------------------------------------------------------------ */
/* 1. Restatements of the reference's functions (mt19937 streams)            */
/* ------------------------------------------------------------------------ */

/* src/mc_eur.cpp:5-27. The reference seeds with time(); `seed` stands in. */
ORC_EXPORT double ref_mc_eur(double S0, double E, double r, double sigma, double T, int N,
                             double payoff_fun, uint32_t seed) {
  std::mt19937 gen;
  gen.seed(seed);
  std::normal_distribution<> norm{0, sqrt(T)};
  const int pf = (int)payoff_fun;
  double result = 0;
  for (int n = 0; n < N; ++n)
    result += payoff(S0 * exp((r - pow(sigma, 2) / 2) * T + sigma * norm(gen)), E, pf);
  return (exp(-r * T) * result) / (double)N;
}

/* src/mc_eur_omp.cpp:5-30: the same loop split over OpenMP threads, each
 * thread with its own generator seeded with the same time() value (as the
 * reference does), schedule(dynamic,1000), reduction(+). */
ORC_EXPORT double ref_mc_eur_omp(double S0, double E, double r, double sigma, double T, int N,
                                 double payoff_fun, uint32_t seed, int threads) {
  double result = 0;
  const int pf = (int)payoff_fun;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
  {
    std::mt19937 gen;
    gen.seed(seed);
    std::normal_distribution<> norm{0, sqrt(T)};
#pragma omp for nowait schedule(dynamic, 1000) reduction(+ : result)
    for (int n = 0; n < N; ++n)
      result += payoff(S0 * exp((r - pow(sigma, 2) / 2) * T + sigma * norm(gen)), E, pf);
  }
  return (exp(-r * T) * result) / (double)N;
}

/* src/mc_asia.cpp:5-40. */
ORC_EXPORT double ref_mc_asia(double S0, double E, double r, double sigma, double T, int N,
                              int M, double payoff_fun, uint32_t seed) {
  const double dt = (double)T / (double)M;
  std::mt19937 gen;
  gen.seed(seed);
  std::normal_distribution<> norm{0, sqrt(dt)};
  const int pf = (int)payoff_fun;
  double result = 0;
  for (int n = 0; n < N; ++n) {
    double St = S0, I = 0;
    for (int m = 0; m < M; ++m) {
      const double dBi = norm(gen);
      I += St * (1 + r * dt / 2 + sigma * dBi / 2);
      St *= exp((r - pow(sigma, 2) / 2) * dt + sigma * dBi);
    }
    result += payoff(I / (double)M, E, pf);
  }
  return exp(-r * T) * result / (double)N;
}

/* src/mc_asia_omp.cpp:5-48: per-thread generator seeded time()*(1+thread). */
ORC_EXPORT double ref_mc_asia_omp(double S0, double E, double r, double sigma, double T, int N,
                                  int M, double payoff_fun, uint32_t seed, int threads) {
  double result = 0;
  const int pf = (int)payoff_fun;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
  {
    const double dt = (double)T / (double)M;
    const int thr = omp_get_thread_num();
    std::mt19937 gen;
    gen.seed(seed * (uint32_t)(1 + thr));
    std::normal_distribution<> norm{0, sqrt(dt)};
#pragma omp for nowait schedule(dynamic, 1000) reduction(+ : result)
    for (int n = 0; n < N; ++n) {
      double St = S0, I = 0;
      for (int m = 0; m < M; ++m) {
        const double dBi = norm(gen);
        I += St * (1 + r * dt / 2 + sigma * dBi / 2);
        St *= exp((r - pow(sigma, 2) / 2) * dt + sigma * dBi);
      }
      result += payoff(I / (double)M, E, pf);
    }
  }
  return (exp(-r * T) * result) / (double)N;
}

namespace {
/* include/common.h:168-208 (pathsfinder): (M+1) x N time-major matrix,
 * antithetic pairs (n, n+N/2) share w with opposite signs; draws are taken
 * path-pair-major. Returns false for odd N (the reference throws). */
bool pathsfinder(double S0, double r, double sigma, double T, int N, int M, uint32_t seed,
                 std::vector<std::vector<double>>& paths) {
  if (N % 2 != 0) return false;
  const double dt = T / M;
  paths.assign((size_t)M + 1, std::vector<double>((size_t)N));
  std::mt19937 gen;
  gen.seed(seed);
  std::normal_distribution<> norm{0, sqrt(dt)};
  for (int n = 0; n < N / 2; ++n) {
    paths[0][n] = S0;
    paths[0][n + N / 2] = S0;
    for (int m = 1; m < M + 1; ++m) {
      const double w = norm(gen);
      paths[m][n] = paths[m - 1][n] * exp((r - 0.5 * sigma * sigma) * dt + sigma * w);
      paths[m][n + N / 2] = paths[m - 1][n + N / 2] * exp((r - 0.5 * sigma * sigma) * dt - sigma * w);
    }
  }
  return true;
}

/* include/common.h:98-124 (inverse, 3x3 adjugate / determinant; fails when
 * det <= 0) and :128-141 (mat_vec_mul). Returns false on det <= 0. */
bool solve3_cofactor(const double x[3][3], const double y[3], double coef[3]) {
  double det = 0;
  for (int i = 0; i < 3; ++i)
    det += (x[0][i] * (x[1][(i + 1) % 3] * x[2][(i + 2) % 3] - x[1][(i + 2) % 3] * x[2][(i + 1) % 3]));
  if (det <= 0) return false;
  double inv[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      inv[j][i] = ((x[(j + 1) % 3][(i + 1) % 3] * x[(j + 2) % 3][(i + 2) % 3]) -
                   (x[(j + 1) % 3][(i + 2) % 3] * x[(j + 2) % 3][(i + 1) % 3])) / det;
  for (int i = 0; i < 3; ++i) {
    coef[i] = 0;
    for (int j = 0; j < 3; ++j) coef[i] += inv[i][j] * y[j];
  }
  return true;
}
}  // namespace

/* src/mc_amer.cpp:5-114 (serial Longstaff-Schwartz), including its exercise
 * rule payoff(x, E) with x = S - E (src/mc_amer.cpp:100). Returns NaN where
 * the reference would throw (odd N, det <= 0). */
ORC_EXPORT double ref_mc_amer(double S0, double E, double r, double sigma, double T, int N, int M,
                              double payoff_fun, uint32_t seed) {
  const double dt = T / M;
  const int pf = (int)payoff_fun;
  double result = 0;
  std::vector<std::vector<double>> paths;
  if (!pathsfinder(S0, r, sigma, T, N, M, seed, paths)) return NAN;
  std::vector<double> exercise_when((size_t)N, (double)M);
  std::vector<double> exercise_st((size_t)N);
  for (int n = 0; n < N; ++n) exercise_st[n] = payoff(paths[M][n], E, pf);
  for (int m = M - 1; m > 0; --m) {
    std::vector<double> x((size_t)N, -1), y((size_t)N, -1);
    double sum_x = 0, sum_x2 = 0, sum_x3 = 0, sum_x4 = 0, sum_y = 0, sum_yx = 0, sum_yx2 = 0;
    double x_length = 0;
    std::vector<double> fst_po, fst_y;
    std::vector<int> fst_n;
    for (int n = 0; n < N; ++n) {
      const double payoff_val = payoff(paths[m][n], E, pf);
      if (payoff_val > 0) {
        ++x_length;
        const double exer = paths[m][n] - E;
        x[n] = exer;
        const double cont = exp(-r * dt * (exercise_when[n] - m)) *
                            payoff(paths[(size_t)exercise_when[n]][n], E, pf);
        y[n] = cont;
        sum_x += exer;
        sum_x2 += exer * exer;
        sum_x3 += exer * exer * exer;
        sum_x4 += exer * exer * exer * exer;
        sum_y += cont;
        sum_yx += cont * exer;
        sum_yx2 += cont * exer * exer;
        if (x_length <= 2) {
          fst_po.push_back(payoff_val);
          fst_y.push_back(cont);
          fst_n.push_back(n);
        }
      }
    }
    if (x_length == 0) continue;
    if (x_length <= 2) {
      for (size_t i = 0; i < fst_n.size(); ++i)
        if (fst_po[i] > fst_y[i]) {
          exercise_when[fst_n[i]] = m;
          exercise_st[fst_n[i]] = fst_po[i];
        }
      continue;
    }
    const double xTx[3][3] = {{x_length, sum_x, sum_x2}, {sum_x, sum_x2, sum_x3}, {sum_x2, sum_x3, sum_x4}};
    const double xTy[3] = {sum_y, sum_yx, sum_yx2};
    double coef[3];
    if (!solve3_cofactor(xTx, xTy, coef)) return NAN;
    for (int i = 0; i < N; ++i) {
      if (x[i] != -1) {
        const double Y_hat = coef[0] + coef[1] * x[i] + coef[2] * pow(x[i], 2);
        const double payoff_val = payoff(x[i], E, pf);
        if (payoff_val > Y_hat) {
          exercise_when[i] = m;
          exercise_st[i] = payoff_val;
        }
      }
    }
  }
  for (int n = 0; n < N; ++n)
    if (exercise_st[n] != 0) result += exp(-r * exercise_when[n] * dt) * exercise_st[n];
  return std::max(payoff(S0, E, pf), result / (double)N);
}

/* src/binom_embar.cpp:5-50 (serial closed binomial sum, comb() of
 * include/common.h:63-72). O(N^2); logs come from a table of log((double)n). */
ORC_EXPORT double ref_binom_embar(double S0, double E, double r, double sigma, double T, int N,
                                  double payoff_fun) {
  const int pf = (int)payoff_fun;
  const Lattice L = lattice(r, sigma, T, N);
  const std::vector<double> lt = make_logtab(N);
  double result = 0;
  const int until = (N % 2 != 0) ? (N + 1) / 2 : N / 2;
  for (int i = 0; i < until; ++i) {
    const double comb_val = comb_ref(N, i, lt.data());
    const double binom1 = comb_val + i * log(L.p) + (N - i) * log(L.q);
    const double binom2 = comb_val + (N - i) * log(L.p) + i * log(L.q);
    result += exp(binom1) * payoff(S0 * pow(L.u, i) * pow(L.d, N - i), E, pf);
    result += exp(binom2) * payoff(S0 * pow(L.u, N - i) * pow(L.d, i), E, pf);
    if (i == 0 && N % 2 == 0) {
      const double binom_mid = comb_ref(N, N / 2, lt.data()) + N / 2 * log(L.p) + N / 2 * log(L.q);
      result += exp(binom_mid) * payoff(S0 * pow(L.u, N / 2) * pow(L.d, N / 2), E, pf);
    }
  }
  return exp(-r * T) * result;
}

/* src/binom_embar_omp.cpp:5-53: the same sum, terms split over OpenMP threads
 * with schedule(dynamic,1000) and reduction(+). comb() is recomputed per term,
 * with a log() call per factor, exactly as the reference does. */
ORC_EXPORT double ref_binom_embar_omp(double S0, double E, double r, double sigma, double T, int N,
                                      double payoff_fun, int threads) {
  const int pf = (int)payoff_fun;
  const Lattice L = lattice(r, sigma, T, N);
  double result = 0;
  const int until = (N % 2 != 0) ? (N + 1) / 2 : N / 2;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
  {
#pragma omp for schedule(dynamic, 1000) nowait reduction(+ : result)
    for (int i = 0; i < until; ++i) {
      double comb_val;
      if (i == 0 || i == N) comb_val = 0;
      else if (i == 1 || i == N - 1) comb_val = log(N);
      else {
        comb_val = 0;
        for (int n = N; n > i; --n) comb_val += log((double)n);
        for (int j = 2; j <= (N - i); ++j) comb_val -= log((double)j);
      }
      const double binom1 = comb_val + i * log(L.p) + (N - i) * log(L.q);
      const double binom2 = comb_val + (N - i) * log(L.p) + i * log(L.q);
      result += exp(binom1) * payoff(S0 * pow(L.u, i) * pow(L.d, N - i), E, pf);
      result += exp(binom2) * payoff(S0 * pow(L.u, N - i) * pow(L.d, i), E, pf);
      if (i == 0 && N % 2 == 0) {
        double cm = 0;
        for (int n = N; n > N / 2; --n) cm += log((double)n);
        for (int j = 2; j <= N / 2; ++j) cm -= log((double)j);
        const double binom_mid = cm + N / 2 * log(L.p) + N / 2 * log(L.q);
        result += exp(binom_mid) * payoff(S0 * pow(L.u, N / 2) * pow(L.d, N / 2), E, pf);
      }
    }
  }
  return exp(-r * T) * result;
}

/* The same reference-order sum restricted to pair indices i in [i_lo, i_hi)
 * (plus the even-N middle term when N/2 lies in the window). Each comb() is
 * the full sequential chain of include/common.h:63-72, so the window's terms
 * are bit-identical to the reference's; terms outside it are dropped. Returns
 * the undiscounted partial sum. Used to check the GPU's windowed kernel. */
ORC_EXPORT double ref_binom_embar_window(double S0, double E, double r, double sigma, double T,
                                         int N, double payoff_fun, int i_lo, int i_hi) {
  const int pf = (int)payoff_fun;
  const Lattice L = lattice(r, sigma, T, N);
  const std::vector<double> lt = make_logtab(N);
  double result = 0;
  const int until = (N % 2 != 0) ? (N + 1) / 2 : N / 2;
  i_lo = std::max(i_lo, 0);
  i_hi = std::min(i_hi, until);
  for (int i = i_lo; i < i_hi; ++i) {
    const double comb_val = comb_ref(N, i, lt.data());
    const double binom1 = comb_val + i * log(L.p) + (N - i) * log(L.q);
    const double binom2 = comb_val + (N - i) * log(L.p) + i * log(L.q);
    result += exp(binom1) * payoff(S0 * pow(L.u, i) * pow(L.d, N - i), E, pf);
    result += exp(binom2) * payoff(S0 * pow(L.u, N - i) * pow(L.d, i), E, pf);
  }
  if (N % 2 == 0) {
    const double binom_mid = comb_ref(N, N / 2, lt.data()) + N / 2 * log(L.p) + N / 2 * log(L.q);
    result += exp(binom_mid) * payoff(S0 * pow(L.u, N / 2) * pow(L.d, N / 2), E, pf);
  }
  return result;
}

/* comb() of include/common.h:63-72 for a single (N, i), for unit checks. */
ORC_EXPORT double ref_comb(int N, int i) {
  const std::vector<double> lt = make_logtab(N);
  return comb_ref(N, i, lt.data());
}

/* Lattice parameters as the reference computes them (u, d, p, q, R). */
ORC_EXPORT void ref_lattice(double r, double sigma, double T, int N, double* out5) {
  const Lattice L = lattice(r, sigma, T, N);
  out5[0] = L.u; out5[1] = L.d; out5[2] = L.p; out5[3] = L.q; out5[4] = L.R;
}

/* src/binom_vanilla_eur.cpp:5-39 (backward induction, European). */
ORC_EXPORT double ref_binom_vanilla_eur(double S0, double E, double r, double sigma, double T,
                                        int N, double payoff_fun) {
  const Lattice L = lattice(r, sigma, T, N);
  std::vector<double> v;
  v.reserve((size_t)N + 1);
  for (int i = 0; i < N + 1; ++i)
    v.push_back(std::max(((S0 * pow(L.u, i) * pow(L.d, N - i)) - E) * payoff_fun, (double)0.0));
  for (int n = N - 1; n >= 0; --n)
    for (int i = 0; i < n + 1; ++i) v[i] = (L.p * v[i + 1] + L.q * v[i]) / L.R;
  return v[0];
}

/* src/mc_amer_omp.cpp:5-117, the OpenMP build of mc_amer: the paths come
 * from pathsfinder seeded with time() + 100 * threads (include/common.h:192,
 * `parallel` = threads); the regression sums are an OpenMP reduction with
 * schedule(dynamic,1000); the <= 2 in-the-money branch exercises where
 * x = S - E beats y and records x as the exercise value (src/mc_amer_omp.cpp:
 * 72-81, unlike the serial build); the exercise update loop is serial; the
 * final mean sums the paths whose exercise date is not 0. With threads = 1
 * the reductions run in path order, so the result is the reference's bit for
 * bit. Returns NaN where the reference throws (odd N, det <= 0). */
ORC_EXPORT double ref_mc_amer_omp(double S0, double E, double r, double sigma, double T, int N,
                                  int M, double payoff_fun, uint32_t seed, int threads) {
  if (threads > 0) omp_set_num_threads(threads);
  const double dt = T / M;
  const int pf = (int)payoff_fun;
  double result = 0;
  std::vector<std::vector<double>> paths;
  if (!pathsfinder(S0, r, sigma, T, N, M, seed + 100u * (uint32_t)threads, paths)) return NAN;
  std::vector<double> exercise_when((size_t)N, (double)M);
  std::vector<double> exercise_st((size_t)N);
  for (int n = 0; n < N; ++n) exercise_st[n] = payoff(paths[M][n], E, pf);
  for (int m = M - 1; m > 0; --m) {
    std::vector<double> x((size_t)N, -1), y((size_t)N, -1);
    double sum_x = 0, sum_x2 = 0, sum_x3 = 0, sum_x4 = 0, sum_y = 0, sum_yx = 0, sum_yx2 = 0;
    double x_length = 0;
#pragma omp parallel
    {
#pragma omp for schedule(dynamic, 1000) nowait reduction(+ : sum_x, sum_x2, sum_x3, sum_x4, \
                                                              sum_y, sum_yx, sum_yx2, x_length)
      for (int n = 0; n < N; ++n) {
        const double payoff_val = payoff(paths[m][n], E, pf);
        if (payoff_val > 0) {
          ++x_length;
          const double exer = paths[m][n] - E;
          x[n] = exer;
          const double cont = exp(-r * dt * (exercise_when[n] - m)) *
                              payoff(paths[(size_t)exercise_when[n]][n], E, pf);
          y[n] = cont;
          sum_x += exer;
          sum_x2 += exer * exer;
          sum_x3 += exer * exer * exer;
          sum_x4 += exer * exer * exer * exer;
          sum_y += cont;
          sum_yx += cont * exer;
          sum_yx2 += cont * exer * exer;
        }
      }
    }
    if (x_length == 0) continue;
    if (x_length <= 2) {
#pragma omp parallel for
      for (int i = 0; i < N; ++i)
        if (x[i] > y[i]) {
          exercise_when[i] = m;
          exercise_st[i] = x[i];
        }
      continue;
    }
    const double xTx[3][3] = {{x_length, sum_x, sum_x2}, {sum_x, sum_x2, sum_x3}, {sum_x2, sum_x3, sum_x4}};
    const double xTy[3] = {sum_y, sum_yx, sum_yx2};
    double coef[3];
    if (!solve3_cofactor(xTx, xTy, coef)) return NAN;
    for (int i = 0; i < N; ++i) {
      if (x[i] != -1) {
        const double Y_hat = coef[0] + coef[1] * x[i] + coef[2] * pow(x[i], 2);
        const double payoff_val = payoff(x[i], E, pf);
        if (payoff_val > Y_hat) {
          exercise_when[i] = m;
          exercise_st[i] = payoff_val;
        }
      }
    }
  }
#pragma omp parallel
  {
#pragma omp for schedule(dynamic, 1000) nowait reduction(+ : result)
    for (int n = 0; n < N; ++n)
      if (exercise_when[n] != 0) result += exp(-r * exercise_when[n] * dt) * exercise_st[n];
  }
  return std::max(payoff(S0, E, pf), result / (double)N);
}

/* The estimator of src/mc_asia_omp.cpp:5-48 (per-thread mt19937 seeded with
 * time() * (1 + thread), the reference's running sum) with its sample
 * variance: out = {price, standard error}. The served-price checks compare
 * the engine's Asian prices with the reference's estimator at a combined
 * standard error. */
ORC_EXPORT void ref_mc_asia_omp_stats(double S0, double E, double r, double sigma, double T,
                                      int N, int M, double payoff_fun, uint32_t seed, int threads,
                                      double* out) {
  double s1 = 0, s2 = 0;
  const int pf = (int)payoff_fun;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
  {
    const double dt = (double)T / (double)M;
    const int thr = omp_get_thread_num();
    std::mt19937 gen;
    gen.seed(seed * (uint32_t)(1 + thr));
    std::normal_distribution<> norm{0, sqrt(dt)};
#pragma omp for nowait schedule(dynamic, 1000) reduction(+ : s1, s2)
    for (int n = 0; n < N; ++n) {
      double St = S0, I = 0;
      for (int m = 0; m < M; ++m) {
        const double dBi = norm(gen);
        I += St * (1 + r * dt / 2 + sigma * dBi / 2);
        St *= exp((r - pow(sigma, 2) / 2) * dt + sigma * dBi);
      }
      const double y = payoff(I / (double)M, E, pf);
      s1 += y;
      s2 += y * y;
    }
  }
  const double disc = exp(-r * T), mean = s1 / N;
  const double var = N > 1 ? std::max(0.0, (s2 - N * mean * mean) / (N - 1)) : 0.0;
  out[0] = disc * mean;
  out[1] = disc * sqrt(var / N);
}

/* src/binom_vanilla_amer.cpp:5-40 (backward induction with early exercise). */
ORC_EXPORT double ref_binom_vanilla_amer(double S0, double E, double r, double sigma, double T,
                                         int N, double payoff_fun) {
  const int pf = (int)payoff_fun;
  const Lattice L = lattice(r, sigma, T, N);
  std::vector<double> v;
  v.reserve((size_t)N + 1);
  for (int i = 0; i < N + 1; ++i) v.push_back(payoff(S0 * pow(L.u, i) * pow(L.d, N - i), E, pf));
  for (int n = N - 1; n >= 0; --n)
    for (int i = 0; i < n + 1; ++i) {
      const double sij = payoff(S0 * pow(L.u, i) * pow(L.d, n - i), E, pf);
      const double jatk = (L.p * v[i + 1] + L.q * v[i]) / L.R;
      v[i] = std::max(jatk, sij);
    }
  return v[0];
}

namespace {
/* Black-Scholes price with time `rem` to expiry (rem = 0: the payoff). */
double bs_rem(double S, double E, double r, double sigma, double rem, int pf) {
  if (rem <= 0) return payoff(S, E, pf);
  const double sd = sigma * sqrt(rem), dK = E * exp(-r * rem);
  if (sd <= 0) return std::max(pf * (S - dK), 0.0);
  const double d1 = (log(S / E) + (r + 0.5 * sigma * sigma) * rem) / sd, d2 = d1 - sd;
  if (pf == 1) return S * norm_cdf(d1) - dK * norm_cdf(d2);
  return dK * norm_cdf(-d2) - S * norm_cdf(-d1);
}
}  // namespace

/* ------------------------------------------------------------------------ */
/* 2. FP64 twins of the GPU kernels (identical Philox draws)                */
/* ------------------------------------------------------------------------ */
/* Every twin returns moment sums out[0..4] = {sum y, sum y^2, sum g, sum g^2,
 * sum y*g} over the N paths, y the undiscounted payoff, g the control variate
 * of that kernel. Tags: 1 European, 2 Asian, 3 basket, 4 American. */

/* mc_eur kernel twin: path n uses normal z(quad n/4, step 0, lane n%4);
 * S_T = S0 exp((r - s^2/2)T + s sqrt(T) z); g = S_T. */
ORC_EXPORT void twin_mc_eur(double S0, double E, double r, double sigma, double T, int64_t N,
                            int pf, uint64_t seed, uint32_t stream, double* out) {
  double s[5] = {0, 0, 0, 0, 0};
  const double drift = (r - 0.5 * sigma * sigma) * T, vol = sigma * sqrt(T);
  const int64_t nq = (N + 3) / 4;
#pragma omp parallel for reduction(+ : s[:5]) schedule(static)
  for (int64_t q = 0; q < nq; ++q) {
    double z[4];
    orc::normals4(seed, stream, 1u, (uint64_t)q, 0u, z);
    for (int l = 0; l < 4; ++l) {
      if (q * 4 + l >= N) break;
      const double ST = S0 * exp(drift + vol * z[l]);
      const double y = payoff(ST, E, pf), g = ST;
      s[0] += y; s[1] += y * y; s[2] += g; s[3] += g * g; s[4] += y * g;
    }
  }
  for (int k = 0; k < 5; ++k) out[k] = s[k];
}

/* mc_asia kernel twin: path n, increment m (0..M-1) uses lane m%4 of the
 * Philox block (x=n, y=m/4); log S_{m+1} = log S_m + (r - s^2/2)dt + s sqrt(dt) z.
 * mode 0: the reference's running sum I += S_m (1 + r dt/2 + s dB/2)
 *         (src/mc_asia.cpp:31-35), A = I/M;
 * mode 1: A = mean(S_1..S_M).
 * g = payoff of the geometric mean with orc_asian_geo_weights(M, mode). */
ORC_EXPORT void twin_mc_asia(double S0, double E, double r, double sigma, double T, int64_t N,
                             int M, int pf, int mode, uint64_t seed, uint32_t stream,
                             double* out) {
  double s[5] = {0, 0, 0, 0, 0};
  const double dt = T / M, sdt = sqrt(dt);
  const double nu_dt = (r - 0.5 * sigma * sigma) * dt;
  const double c1 = 1 + r * dt / 2, c2 = sigma * sdt / 2;
  std::vector<double> w((size_t)M + 1);
  orc_asian_geo_weights(M, mode, w.data());
#pragma omp parallel for reduction(+ : s[:5]) schedule(static)
  for (int64_t n = 0; n < N; ++n) {
    double lS = 0, I = 0, lg = 0, z[4] = {0, 0, 0, 0};
    for (int m = 0; m < M; ++m) {
      if (m % 4 == 0) orc::normals4(seed, stream, 2u, (uint64_t)n, (uint32_t)(m / 4), z);
      const double zm = z[m % 4];
      const double S = S0 * exp(lS);
      if (mode == 0) I += S * (c1 + c2 * zm);
      lS += nu_dt + sigma * sdt * zm;
      if (mode == 1) I += S0 * exp(lS);
      lg += w[m + 1] * lS;
    }
    const double A = I / M;
    const double G = S0 * exp(lg); /* the weights sum to 1 */
    const double y = payoff(A, E, pf), g = payoff(G, E, pf);
    s[0] += y; s[1] += y * y; s[2] += g; s[3] += g * g; s[4] += y * g;
  }
  for (int k = 0; k < 5; ++k) out[k] = s[k];
}

/* mc_eur_multi kernel twin: asset a of path n uses lane a%4 of the Philox
 * block (x=n, y=a/4); x = L z with L the correlation factor (row-major d x d,
 * lower triangular or full);
 * S_a = S0_a exp((r - s_a^2/2)T + s_a*ts*x_a); basket = mean_a S_a;
 * g = payoff(exp(mean_a log S_a)). ts is sqrt(T), or 1 to reproduce the
 * reference's unscaled draws (include/mvn.h:55-60, src/mc_eur_multi.cpp:30). */
ORC_EXPORT void twin_mc_basket(int d, const double* S0, const double* sig, const double* Lf,
                               double r, double T, double ts, double E, int64_t N, int pf,
                               uint64_t seed, uint32_t stream, double* out) {
  double s[5] = {0, 0, 0, 0, 0};
  const double w = 1.0 / d;
#pragma omp parallel for reduction(+ : s[:5]) schedule(static)
  for (int64_t n = 0; n < N; ++n) {
    std::vector<double> z((size_t)((d + 3) / 4) * 4);
    for (int a0 = 0; a0 < d; a0 += 4)
      orc::normals4(seed, stream, 3u, (uint64_t)n, (uint32_t)(a0 / 4), &z[(size_t)a0]);
    double bsk = 0, lg = 0;
    for (int a = 0; a < d; ++a) {
      double x = 0;
      for (int b = 0; b < d; ++b) x += Lf[a * d + b] * z[b];
      const double ls = log(S0[a]) + (r - 0.5 * sig[a] * sig[a]) * T + sig[a] * ts * x;
      bsk += w * exp(ls);
      lg += w * ls;
    }
    const double y = payoff(bsk, E, pf), g = payoff(exp(lg), E, pf);
    s[0] += y; s[1] += y * y; s[2] += g; s[3] += g * g; s[4] += y * g;
  }
  for (int k = 0; k < 5; ++k) out[k] = s[k];
}

/* mc_amer kernel twin (Longstaff-Schwartz).
 * Paths: antithetic pair p in [0, N/2) uses lane (m-1)%4 of the Philox block
 * (x=p, y=(m-1)/4) for the increment into date m = 1..M; path p takes +z and path p + N/2
 * takes -z (the pairing of include/common.h:195-205).
 * Backward sweep, dates m = M-1..1 (src/mc_amer.cpp:31-107): in-the-money
 * paths only; x = (S - E)/E (the reference regresses on S - E; dividing by E
 * rescales the basis and leaves the fitted values unchanged in exact
 * arithmetic); y = cf * exp(-r dt (tau - m)); normal equations of the basis
 * {1, x, x^2} solved by the adjugate formula (include/common.h:98-141).
 * <= 2 ITM paths: exercise where the exercise value beats y (src/mc_amer.cpp:75-83).
 * Exercise value: payoff(S) by default; with ref_exercise = 1 it is the
 * reference's payoff(S - E, E) (src/mc_amer.cpp:100).
 * out[0..4] moment sums over the N/2 antithetic pairs of the pair means of
 * y = the discounted cash flow and g = the control variate:
 *   g = exp(-r tau dt) * P_E(S_tau, T - tau dt), the discounted Black-Scholes
 *       price at the exercise date (a martingale, so E[g] = P_E(S0, T));
 *   with ref_exercise = 1: g = exp(-rT) payoff(S_M);
 * out[5] = 1 if a regression was singular. */
ORC_EXPORT void twin_mc_amer(double S0, double E, double r, double sigma, double T, int64_t N,
                             int M, int pf, int ref_exercise, uint64_t seed, uint32_t stream,
                             double* out) {
  const double dt = T / M, sdt = sqrt(dt), nu_dt = (r - 0.5 * sigma * sigma) * dt;
  const int64_t H = N / 2;
  std::vector<double> S((size_t)(M + 1) * N);
  std::vector<double> disc((size_t)M + 1);
  for (int k = 0; k <= M; ++k) disc[k] = exp(-r * dt * k);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < H; ++p) {
    double lp = 0, lm = 0, z[4] = {0, 0, 0, 0};
    S[p] = S0;
    S[p + H] = S0;
    for (int m = 1; m <= M; ++m) {
      if ((m - 1) % 4 == 0) orc::normals4(seed, stream, 4u, (uint64_t)p, (uint32_t)((m - 1) / 4), z);
      const double zm = z[(m - 1) % 4];
      lp += nu_dt + sigma * sdt * zm;
      lm += nu_dt - sigma * sdt * zm;
      S[(size_t)m * N + p] = S0 * exp(lp);
      S[(size_t)m * N + p + H] = S0 * exp(lm);
    }
  }
  std::vector<double> cf((size_t)N);
  std::vector<int> tau((size_t)N, M);
  for (int64_t n = 0; n < N; ++n) cf[n] = payoff(S[(size_t)M * N + n], E, pf);
  const double inv_scale = 1.0 / E;
  int singular = 0;
  for (int m = M - 1; m > 0; --m) {
    double a[8] = {0, 0, 0, 0, 0, 0, 0, 0}; /* n, x, x2, x3, x4, y, yx, yx2 */
    const double* Sm = &S[(size_t)m * N];
#pragma omp parallel for reduction(+ : a[:8]) schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      if (payoff(Sm[n], E, pf) > 0) {
        const double x = (Sm[n] - E) * inv_scale;
        const double y = cf[n] * disc[tau[n] - m];
        a[0] += 1; a[1] += x; a[2] += x * x; a[3] += x * x * x; a[4] += x * x * x * x;
        a[5] += y; a[6] += y * x; a[7] += y * x * x;
      }
    }
    if (a[0] == 0) continue;
    double coef[3] = {0, 0, 0};
    const bool few = a[0] <= 2;
    if (!few) {
      const double xtx[3][3] = {{a[0], a[1], a[2]}, {a[1], a[2], a[3]}, {a[2], a[3], a[4]}};
      const double xty[3] = {a[5], a[6], a[7]};
      if (!solve3_cofactor(xtx, xty, coef)) { singular = 1; continue; }
    }
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      const double pv = payoff(Sm[n], E, pf);
      if (pv > 0) {
        const double x = (Sm[n] - E) * inv_scale;
        const double cont = few ? cf[n] * disc[tau[n] - m] : coef[0] + coef[1] * x + coef[2] * x * x;
        const double ex = (ref_exercise && !few) ? payoff(Sm[n] - E, E, pf) : pv;
        if (ex > cont) { cf[n] = ex; tau[n] = m; }
      }
    }
  }
  double s[5] = {0, 0, 0, 0, 0};
  const double dT = exp(-r * T);
  auto cv = [&](int64_t n) {
    if (ref_exercise) return dT * payoff(S[(size_t)M * N + n], E, pf);
    const int t = tau[n];
    if (t == M) return disc[M] * cf[n];
    return disc[t] * bs_rem(S[(size_t)t * N + n], E, r, sigma, (M - t) * dt, pf);
  };
  for (int64_t p = 0; p < H; ++p) {
    const double y = 0.5 * (cf[p] * disc[tau[p]] + cf[p + H] * disc[tau[p + H]]);
    const double g = 0.5 * (cv(p) + cv(p + H));
    s[0] += y; s[1] += y * y; s[2] += g; s[3] += g * g; s[4] += y * g;
  }
  for (int k = 0; k < 5; ++k) out[k] = s[k];
  out[5] = singular;
}

/* ------------------------------------------------------------------------ */
/* 3. Audit of a GPU Longstaff-Schwartz sweep (pcf_mc_amer_audit's record)   */
/* ------------------------------------------------------------------------ */
/* Checks the GPU's exercise policy three ways, with the reference's
 * algorithm (src/mc_amer.cpp:31-113: in-the-money regression on {1, x, x^2},
 * the <= 2 in-the-money branch, exercise where the exercise value beats the
 * fitted continuation value) in the GPU's basis u = pf (S - E)/E:
 *
 * R1  the GPU's own FP32 path matrix `gu` and coefficients `gcoef`, its
 *     decision arithmetic replayed in FP32 exactly (the kernel's formulas,
 *     fmaf included): must reproduce the GPU's exercise dates `gtau` path
 *     for path. On the same state the regression sums are formed in FP64
 *     and solved in FP64 (the adjugate of include/common.h:98-141), giving
 *     the sums' and the fitted values' errors, and the decisions the FP64
 *     coefficients would change.
 * R2  FP64 paths (the twin's Philox draws) with the GPU's coefficients,
 *     decided in FP64: each decision that differs from the GPU's is checked
 *     to lie within FP32 rounding of the exercise boundary, i.e. the FP64
 *     decision function changes sign between the FP64 path value and the
 *     GPU's FP32 one, or its value at the GPU's path is within the FP32
 *     evaluation error of the kernel's formula.
 * R3  the independent FP64 twin (its own FP64 regressions), compared with
 *     the GPU's policy and price.
 *
 * rep[] (doubles): 0 R1 exercise-date mismatches, 1 R1 mode mismatches,
 * 2 max relative error of the GPU's regression sums, 3 max fitted-value error
 * of the GPU's coefficients against the FP64 regression of the same state (/E),
 * 4 the same for the solve alone (FP64 solve of the GPU's sums), 5 decisions
 * the FP64 coefficients would change, 6 their largest margin (/E),
 * 7 relative difference of sum y (GPU vs FP64 moments of the R1 state),
 * 8 the same for sum g, 9 max |u_gpu - u_fp64|, 10 R2 decision flips,
 * 11 R2 flips not within FP32 rounding of the boundary, 12 R2 exercise dates
 * differing from the GPU's, 13 relative difference of sum y (R2 vs GPU),
 * 14 relative difference of the GPU's sum y and the FP64 value of its own
 * exercise dates on FP64 paths, 15 R3 exercise dates differing from the
 * GPU's, 16 relative difference of sum y (R3 vs GPU), 17 the same for sum g,
 * 18 largest |exercise - continuation| / E of an R2 flip, 19 regression dates,
 * 20 in-the-money path-dates of the regression dates, 21 R4 exercise dates
 * differing from the GPU's, 22 relative difference of sum y (R4 vs GPU),
 * 23 exercise dates differing between R4 and R3, 24 relative difference of
 * sum y (R3 vs R4), 25 the first date (in the backward sweep) at which R4's
 * decisions differ from the GPU's (0: never), 26 the paths that differ
 * there, 27 their largest |exercise - continuation| / E under R4's FP64
 * coefficients, 28 the largest difference of the GPU's and R4's fitted
 * continuation values at that date (/E). Up to that date the two states are
 * identical; after it each flip moves the later regressions, which flips
 * further paths near the boundary (the estimator is a discontinuous
 * function of its inputs), so later differences are consequences.
 *
 * R4  the GPU's FP32 path matrix with FP64 regressions and FP64 decisions
 *     (no replay): R4 against the GPU isolates the kernel's arithmetic, R3
 *     against R4 the FP32 representation of the paths alone. */
namespace {
struct AmerAuditIn {
  double S0, E, r, sigma, T;
  int64_t N;
  int M, pf, refx;
};

double rel_diff(double a, double b) { return fabs(a - b) / std::max(fabs(b), 1e-300); }

/* FP64 regression of one date; returns the mode as the kernel defines it
 * (0 skip, 1 at most two in-the-money paths, 2 regression). */
int solve_mode(const double a[8], double coef[3]) {
  coef[0] = coef[1] = coef[2] = 0;
  if (a[0] == 0) return 0;
  if (a[0] <= 2) return 1;
  const double xtx[3][3] = {{a[0], a[1], a[2]}, {a[1], a[2], a[3]}, {a[2], a[3], a[4]}};
  const double xty[3] = {a[5], a[6], a[7]};
  return solve3_cofactor(xtx, xty, coef) ? 2 : 0;
}
}  // namespace

ORC_EXPORT void twin_mc_amer_audit(double S0, double E, double r, double sigma, double T,
                                   int64_t N, int M, int pf, int ref_exercise, uint64_t seed,
                                   uint32_t stream, const float* gcoef, const double* gsums,
                                   const uint16_t* gtau, const float* gu, const double* gmom,
                                   double* rep) {
  for (int k = 0; k < 29; ++k) rep[k] = 0;
  const int64_t H = N / 2;
  const double dtd = T / M;
  /* The kernel's FP32 constants, made as the host makes them. */
  std::vector<float> dtf((size_t)M + 1), edtf((size_t)M + 1);
  for (int k = 0; k <= M; ++k) {
    dtf[k] = (float)exp(-r * dtd * k);
    edtf[k] = (float)exp(r * dtd * k);
  }
  const float Ef = (float)E, nKf = (float)(-pf * E), pff = (float)pf;
  const float EdM = Ef * dtf[M];
  auto U = [&](int m, int64_t n) { return gu[(size_t)(m - 1) * N + n]; };  /* date m */

  /* FP64 paths (the twin's draws), u64 = pf (S/E - 1). */
  const double sdt = sqrt(dtd), nu_dt = (r - 0.5 * sigma * sigma) * dtd;
  std::vector<double> S((size_t)(M + 1) * N);
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < H; ++p) {
    double lp = 0, lm = 0, z[4] = {0, 0, 0, 0};
    S[p] = S0;
    S[p + H] = S0;
    for (int m = 1; m <= M; ++m) {
      if ((m - 1) % 4 == 0) orc::normals4(seed, stream, 4u, (uint64_t)p, (uint32_t)((m - 1) / 4), z);
      const double zm = z[(m - 1) % 4];
      lp += nu_dt + sigma * sdt * zm;
      lm += nu_dt - sigma * sdt * zm;
      S[(size_t)m * N + p] = S0 * exp(lp);
      S[(size_t)m * N + p + H] = S0 * exp(lm);
    }
  }
  auto U64 = [&](int m, int64_t n) { return pf * (S[(size_t)m * N + n] / E - 1.0); };
  double du = 0;
#pragma omp parallel for reduction(max : du) schedule(static)
  for (int64_t n = 0; n < N; ++n)
    for (int m = 1; m <= M; ++m)  /* the path matrix holds max(u, 0) */
      du = std::max(du, fabs((double)U(m, n) - std::max(U64(m, n), 0.0)));
  rep[9] = du;
  std::vector<double> disc((size_t)M + 1);
  for (int k = 0; k <= M; ++k) disc[k] = exp(-r * dtd * k);

  /* ---- R1: the GPU's paths and coefficients, its FP32 decisions ---- */
  std::vector<float> cf1((size_t)N);
  std::vector<int> tau1((size_t)N, M);
  for (int64_t n = 0; n < N; ++n) cf1[n] = fmaxf(U(M, n), 0.f) * EdM;
  /* ---- R2: FP64 paths, the GPU's coefficients, FP64 decisions ---- */
  std::vector<double> cf2((size_t)N);  /* cash flow at tau2 (undiscounted) */
  std::vector<int> tau2((size_t)N, M);
  /* ---- R3: the independent FP64 twin ---- */
  std::vector<double> cf3((size_t)N);
  std::vector<int> tau3((size_t)N, M);
  for (int64_t n = 0; n < N; ++n) cf2[n] = cf3[n] = E * std::max(U64(M, n), 0.0);
  /* ---- R4: the GPU's FP32 paths, FP64 regressions and decisions ---- */
  std::vector<double> cf4((size_t)N);
  std::vector<int> tau4((size_t)N, M);
  for (int64_t n = 0; n < N; ++n) cf4[n] = E * std::max((double)U(M, n), 0.0);

  long long mode_mis = 0, cflips = 0, flips2 = 0, unexpl = 0, rdates = 0, itm_dates = 0;
  /* R4 against the GPU: the first date (in the backward sweep) where their
   * decisions differ, the paths that differ there and how far those lie from
   * the boundary; before it the two states are identical. */
  bool synced4 = true;
  int first4 = 0;
  long long first4_paths = 0;
  double first4_margin = 0, first4_fitdiff = 0;
  double sum_err = 0, fit_err = 0, fit_err_solve = 0, cmargin = 0, fmargin = 0;
  for (int m = M - 1; m >= 1; --m) {
    const int gmode = (int)gcoef[(size_t)m * 4];
    const float c0 = gcoef[(size_t)m * 4 + 1], c1 = gcoef[(size_t)m * 4 + 2],
                c2 = gcoef[(size_t)m * 4 + 3];
    const float dm = dtf[m], em = edtf[m];
    /* R1 sums in FP64 on the GPU's state. */
    double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma omp parallel for reduction(+ : a[:8]) schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      const float uf = U(m, n);
      if (uf > 0.f) {
        const double x = uf, y = cf1[n];
        a[0] += 1; a[1] += x; a[2] += x * x; a[3] += x * x * x; a[4] += x * x * x * x;
        a[5] += y; a[6] += y * x; a[7] += y * x * x;
      }
    }
    for (int k = 5; k < 8; ++k) a[k] *= (double)em;
    for (int k = 0; k < 8; ++k) {
      const double g = gsums[(size_t)m * 8 + k];
      if (a[k] != 0 || g != 0) sum_err = std::max(sum_err, rel_diff(g, a[k]));
    }
    double c64[3], cg[3];
    const int emode = solve_mode(a, c64);
    const double* gs = gsums + (size_t)m * 8;
    solve_mode(gs, cg);
    mode_mis += emode != gmode;
    if (gmode == 2) ++rdates;
    /* R3 sums (FP64 paths, its own state) and its coefficients. */
    double a3[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma omp parallel for reduction(+ : a3[:8]) schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      const double x = U64(m, n);
      if (x > 0) {
        const double y = cf3[n] * disc[tau3[n] - m];
        a3[0] += 1; a3[1] += x; a3[2] += x * x; a3[3] += x * x * x; a3[4] += x * x * x * x;
        a3[5] += y; a3[6] += y * x; a3[7] += y * x * x;
      }
    }
    double c3[3];
    const int mode3 = solve_mode(a3, c3);
    double a4[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma omp parallel for reduction(+ : a4[:8]) schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      const double x = U(m, n);
      if (x > 0) {
        const double y = cf4[n] * disc[tau4[n] - m];
        a4[0] += 1; a4[1] += x; a4[2] += x * x; a4[3] += x * x * x; a4[4] += x * x * x * x;
        a4[5] += y; a4[6] += y * x; a4[7] += y * x * x;
      }
    }
    double c4[3];
    const int mode4 = solve_mode(a4, c4);

    long long l_cflips = 0, l_flips2 = 0, l_unexpl = 0, l_itm = 0, l_d4 = 0;
    double l_fit = 0, l_fits = 0, l_cm = 0, l_fm = 0, l_m4 = 0, l_fd4 = 0;
#pragma omp parallel for reduction(+ : l_cflips, l_flips2, l_unexpl, l_itm, l_d4) \
    reduction(max : l_fit, l_fits, l_cm, l_fm, l_m4, l_fd4) schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      /* R1: the kernel's decision, replayed in FP32. */
      const float uf = U(m, n);
      bool d1 = false;
      float ex1 = 0.f;
      if (gmode != 0 && uf > 0.f) {
        float cont;
        ex1 = uf * Ef;
        if (gmode == 1) {
          cont = cf1[n] * em;
        } else {
          cont = fmaf(fmaf(c2, uf, c1), uf, c0);
          if (ref_exercise) ex1 = fmaxf(fmaf(Ef, uf, nKf), 0.f);
        }
        d1 = ex1 > cont;
      }
      if (gmode == 2 && uf > 0.f) {
        ++l_itm;
        const double x = uf;
        const double fg = (double)c0 + (double)c1 * x + (double)c2 * x * x;
        l_fit = std::max(l_fit, fabs(fg - (c64[0] + c64[1] * x + c64[2] * x * x)) / E);
        l_fits = std::max(l_fits, fabs(fg - (cg[0] + cg[1] * x + cg[2] * x * x)) / E);
        /* The decision the FP64 coefficients would take on the same state. */
        const double ex = ref_exercise ? std::max(E * x - pf * E, 0.0) : E * x;
        const double f64 = ex - (c64[0] + c64[1] * x + c64[2] * x * x);
        if ((f64 > 0) != d1) {
          ++l_cflips;
          l_cm = std::max(l_cm, fabs(f64) / E);
        }
      }
      /* R2: FP64 path value, the GPU's coefficients. */
      const double u2 = U64(m, n);
      bool d2 = false;
      if (gmode != 0 && u2 > 0) {
        double cont, ex = E * u2;
        if (gmode == 1) {
          cont = cf2[n] * disc[tau2[n] - m];
        } else {
          cont = (double)c0 + (double)c1 * u2 + (double)c2 * u2 * u2;
          if (ref_exercise) ex = std::max(E * u2 - pf * E, 0.0);
        }
        d2 = ex > cont;
      }
      if (d2 != d1) {
        ++l_flips2;
        bool explained = (u2 > 0) != (uf > 0.f);  /* in-the-money status itself */
        if (!explained && gmode == 2) {
          auto f = [&](double v) {
            const double ex = ref_exercise ? std::max(E * v - pf * E, 0.0) : E * v;
            return ex - ((double)c0 + (double)c1 * v + (double)c2 * v * v);
          };
          const double fu = f(uf), f2 = f(u2);
          const double x = uf;
          const double eps = ldexp(1.0, -21) * (fabs(E * x) + E + fabs((double)c0) +
                                                fabs((double)c1 * x) + fabs((double)c2 * x * x));
          explained = ((fu > 0) != (f2 > 0)) || fabs(fu) <= eps;
          l_fm = std::max(l_fm, fabs(f2) / E);
        } else if (!explained && gmode == 1) {
          /* Depends on the path's own cash flow, which an earlier flip moved. */
          explained = tau1[n] != tau2[n];
        }
        if (!explained) ++l_unexpl;
      }
      /* Apply the three decisions. */
      if (d1) {
        cf1[n] = ex1 * dm;
        tau1[n] = m;
      }
      if (d2) {
        cf2[n] = (ref_exercise && gmode == 2) ? std::max(E * u2 - pf * E, 0.0) : E * u2;
        tau2[n] = m;
      }
      const double u4 = uf;
      bool d4 = false;
      if (mode4 != 0 && u4 > 0) {
        double cont, ex = E * u4;
        if (mode4 == 1) {
          cont = cf4[n] * disc[tau4[n] - m];
        } else {
          cont = c4[0] + c4[1] * u4 + c4[2] * u4 * u4;
          if (ref_exercise) ex = std::max(E * u4 - pf * E, 0.0);
        }
        d4 = ex > cont;
        if (synced4 && mode4 == 2 && gmode == 2) {
          const double fg = (double)c0 + (double)c1 * u4 + (double)c2 * u4 * u4;
          l_fd4 = std::max(l_fd4, fabs(fg - (c4[0] + c4[1] * u4 + c4[2] * u4 * u4)) / E);
          if (d4 != d1) {
            ++l_d4;
            l_m4 = std::max(l_m4, fabs(ex - cont) / E);
          }
        }
        if (d4) {
          cf4[n] = ex;
          tau4[n] = m;
        }
      }
      const double u3 = u2;
      if (mode3 != 0 && u3 > 0) {
        double cont, ex = E * u3;
        if (mode3 == 1) {
          cont = cf3[n] * disc[tau3[n] - m];
        } else {
          cont = c3[0] + c3[1] * u3 + c3[2] * u3 * u3;
          if (ref_exercise) ex = std::max(E * u3 - pf * E, 0.0);
        }
        if (ex > cont) {
          cf3[n] = ex;
          tau3[n] = m;
        }
      }
    }
    if (synced4 && l_d4 > 0) {
      synced4 = false;
      first4 = m;
      first4_paths = l_d4;
      first4_margin = l_m4;
      first4_fitdiff = l_fd4;
    }
    cflips += l_cflips;
    flips2 += l_flips2;
    unexpl += l_unexpl;
    itm_dates += l_itm;
    fit_err = std::max(fit_err, l_fit);
    fit_err_solve = std::max(fit_err_solve, l_fits);
    cmargin = std::max(cmargin, l_cm);
    fmargin = std::max(fmargin, l_fm);
  }
  long long tmis1 = 0, tmis2 = 0, tmis3 = 0, tmis4 = 0, tmis34 = 0;
  for (int64_t n = 0; n < N; ++n) {
    tmis1 += tau1[n] != (int)gtau[n];
    tmis2 += tau2[n] != (int)gtau[n];
    tmis3 += tau3[n] != (int)gtau[n];
    tmis4 += tau4[n] != (int)gtau[n];
    tmis34 += tau4[n] != tau3[n];
  }
  /* Moments over antithetic pair means (the kernel's estimator). */
  auto cvd = [&](int t, double Stau, double cfd, double SM) {
    if (ref_exercise) return disc[M] * std::max(pf * (SM - E), 0.0);
    if (t == M) return cfd;
    return disc[t] * bs_rem(Stau, E, r, sigma, (M - t) * dtd, pf);
  };
  double y1 = 0, g1 = 0, y2 = 0, y3 = 0, g3 = 0, yv = 0, y4 = 0;
  for (int64_t p = 0; p < H; ++p) {
    double a1 = 0, b1 = 0, a2 = 0, a3 = 0, b3 = 0, av = 0, a4 = 0;
    for (int64_t n : {p, p + H}) {
      /* R1: the GPU's FP32 state valued in FP64. */
      const double c = cf1[n];
      a1 += c;
      const double Stau = E + pf * (c * (double)edtf[tau1[n]]);
      b1 += cvd(tau1[n], Stau, c, E * (1.0 + pf * (double)U(M, n)));
      a2 += cf2[n] * disc[tau2[n]];
      a3 += cf3[n] * disc[tau3[n]];
      a4 += cf4[n] * disc[tau4[n]];
      b3 += cvd(tau3[n], S[(size_t)tau3[n] * N + n], cf3[n] * disc[tau3[n]], S[(size_t)M * N + n]);
      /* The GPU's exercise dates valued on FP64 paths. */
      const int t = gtau[n];
      const double u = U64(t, n);
      double cfv;
      if (t == M) cfv = E * std::max(u, 0.0);
      else if (ref_exercise && (int)gcoef[(size_t)t * 4] == 2) cfv = std::max(E * u - pf * E, 0.0);
      else cfv = E * u;
      av += cfv * disc[t];
    }
    y1 += 0.5 * a1; g1 += 0.5 * b1; y2 += 0.5 * a2; y3 += 0.5 * a3; g3 += 0.5 * b3; yv += 0.5 * av;
    y4 += 0.5 * a4;
  }
  rep[0] = (double)tmis1;
  rep[1] = (double)mode_mis;
  rep[2] = sum_err;
  rep[3] = fit_err;
  rep[4] = fit_err_solve;
  rep[5] = (double)cflips;
  rep[6] = cmargin;
  rep[7] = rel_diff(gmom[0], y1);
  rep[8] = rel_diff(gmom[2], g1);
  rep[10] = (double)flips2;
  rep[11] = (double)unexpl;
  rep[12] = (double)tmis2;
  rep[13] = rel_diff(y2, gmom[0]);
  rep[14] = rel_diff(gmom[0], yv);
  rep[15] = (double)tmis3;
  rep[16] = rel_diff(y3, gmom[0]);
  rep[17] = rel_diff(g3, gmom[2]);
  rep[18] = fmargin;
  rep[19] = (double)rdates;
  rep[20] = (double)itm_dates;
  rep[21] = (double)tmis4;
  rep[22] = rel_diff(y4, gmom[0]);
  rep[23] = (double)tmis34;
  rep[24] = rel_diff(y3, y4);
  rep[25] = (double)first4;
  rep[26] = (double)first4_paths;
  rep[27] = first4_margin;
  rep[28] = first4_fitdiff;
}

/* An audit record as the kernel would write it, made on the CPU: the FP64
 * paths rounded to FP32, the kernel's sweep replayed in FP32 (its decision
 * formulas, fmaf included), each date's coefficients from an FP64
 * regression of that state rounded to FP32. It feeds twin_mc_amer_audit in
 * the CPU tests, clean and with planted mistakes, to show the audit accepts
 * a consistent record and catches a wrong one. gcoef[M*4], gsums[M*8],
 * gtau[N], gu[M*N], gmom[5] as pcf_mc_amer_audit's (ref_exercise = 0). */
ORC_EXPORT void orc_emulate_lsm_record(double S0, double E, double r, double sigma, double T,
                                       int64_t N, int M, int pf, uint64_t seed, uint32_t stream,
                                       float* gcoef, double* gsums, uint16_t* gtau, float* gu,
                                       double* gmom) {
  const int64_t H = N / 2;
  const double dtd = T / M, sdt = sqrt(dtd), nu_dt = (r - 0.5 * sigma * sigma) * dtd;
  for (int64_t p = 0; p < H; ++p) {
    double lp = 0, lm = 0, z[4] = {0, 0, 0, 0};
    for (int m = 1; m <= M; ++m) {
      if ((m - 1) % 4 == 0) orc::normals4(seed, stream, 4u, (uint64_t)p, (uint32_t)((m - 1) / 4), z);
      const double zm = z[(m - 1) % 4];
      lp += nu_dt + sigma * sdt * zm;
      lm += nu_dt - sigma * sdt * zm;
      gu[(size_t)(m - 1) * N + p] = fmaxf((float)(pf * (S0 * exp(lp) / E - 1.0)), 0.f);
      gu[(size_t)(m - 1) * N + p + H] = fmaxf((float)(pf * (S0 * exp(lm) / E - 1.0)), 0.f);
    }
  }
  std::vector<float> dtf((size_t)M + 1), edtf((size_t)M + 1);
  for (int k = 0; k <= M; ++k) {
    dtf[k] = (float)exp(-r * dtd * k);
    edtf[k] = (float)exp(r * dtd * k);
  }
  const float Ef = (float)E, EdM = Ef * dtf[M];
  std::vector<float> cf((size_t)N);
  for (int64_t n = 0; n < N; ++n) {
    cf[n] = fmaxf(gu[(size_t)(M - 1) * N + n], 0.f) * EdM;
    gtau[n] = (uint16_t)M;
  }
  for (int k = 0; k < 4 * M; ++k) gcoef[k] = 0.f;
  for (int k = 0; k < 8 * M; ++k) gsums[k] = 0.0;
  for (int m = M - 1; m >= 1; --m) {
    const float* u = gu + (size_t)(m - 1) * N;
    double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t n = 0; n < N; ++n)
      if (u[n] > 0.f) {
        const double x = u[n], y = cf[n];
        a[0] += 1; a[1] += x; a[2] += x * x; a[3] += x * x * x; a[4] += x * x * x * x;
        a[5] += y; a[6] += y * x; a[7] += y * x * x;
      }
    for (int k = 5; k < 8; ++k) a[k] *= (double)edtf[m];
    for (int k = 0; k < 8; ++k) gsums[(size_t)m * 8 + k] = a[k];
    double c[3];
    const int mode = solve_mode(a, c);
    const float c0 = (float)c[0], c1 = (float)c[1], c2 = (float)c[2];
    gcoef[(size_t)m * 4] = (float)mode;
    gcoef[(size_t)m * 4 + 1] = c0;
    gcoef[(size_t)m * 4 + 2] = c1;
    gcoef[(size_t)m * 4 + 3] = c2;
    if (mode == 0) continue;
    for (int64_t n = 0; n < N; ++n) {
      const float uf = u[n];
      if (!(uf > 0.f)) continue;
      const float ex = uf * Ef;
      const float cont = mode == 1 ? cf[n] * edtf[m] : fmaf(fmaf(c2, uf, c1), uf, c0);
      if (ex > cont) {
        cf[n] = ex * dtf[m];
        gtau[n] = (uint16_t)m;
      }
    }
  }
  double s[5] = {0, 0, 0, 0, 0};
  for (int64_t p = 0; p < H; ++p) {
    const double y = 0.5 * ((double)cf[p] + (double)cf[p + H]);
    s[0] += y; s[1] += y * y;
  }
  for (int k = 0; k < 5; ++k) gmom[k] = s[k];
}
