// Closed binomial sum (the reference's binom_embar) as a parallel reduction.
//
// Reference: binom() of src/binom_embar.cpp:5-50 (OpenMP src/binom_embar_omp.cpp:5-53,
// MPI k-range split src/binom_embar_mpi.cpp:38-57) with comb() of
// include/common.h:63-72:
//   price = e^{-rT} sum_{i < ceil(N/2)} [ e^{comb(N,i) + i lp + (N-i) lq} payoff(S0 u^i d^{N-i})
//                                       + e^{comb(N,i) + (N-i) lp + i lq} payoff(S0 u^{N-i} d^i) ]
//           (+ the middle term for even N), lp = log p, lq = log q.
// comb(N,i) is one FP64 accumulator: + log n for n = N..i+1, then - log j for
// j = 2..N-i. Its rounding drift (~1e-9 relative at N = 5e4) is part of the
// reference's result, so the default mode reproduces that chain exactly.
//
// mode 0 (reference order): every term inside the window is bit-identical
//   to the reference's, up to the last-ulp differences of the GPU's
//   exp/pow. The O(N) chain per term is replaced by an exact shortcut. While
//   the accumulator stays inside one binade [2^e, 2^{e+1}), every step
//   fl(acc +- log n) is an integer operation in units of that binade's ulp
//   u_e = 2^{e-52}: acc/u_e +- D_e[n], with D_e[n] = log n / u_e rounded to
//   nearest, ties excepted. A table of prefix sums of D_e per binade turns a
//   whole stretch of steps into one difference, found by binary search. The
//   steps that cross a binade or hit an exact tie (fraction exactly 1/2,
//   where round-to-even depends on the accumulator) are replayed as real
//   __dadd_rn / __dsub_rn. The integer stretches are exact by construction,
//   so the result equals the sequential chain bit for bit.
// mode 1 (accurate): log C(N,k) p^k q^{N-k} by Loader's saddle-point
//   formula (C. Loader, "Fast and Accurate Computation of Binomial
//   Probabilities", 2000: Stirling-series remainders plus bd0 deviance
//   terms), accurate to ~1e-15 relative per term.
//
// Only terms with k within 8 sqrt(N) of N p or N p' (p' = p u / R, the
// share-measure probability) are evaluated. By Chernoff's bound the weight
// outside is below 2 e^{-128} of S0 R^N + E.
//
// This translation unit is compiled with -fmad=false and the explicit
// __dadd_rn/__dmul_rn intrinsics, so no a*b+c is contracted into an FMA that
// the reference's x86-64 build does not perform.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <vector>

#include "pcf_api_internal.h"
#include "pcf_device.cuh"

namespace pcf {

// The reference's lattice parameters, src/binom_embar.cpp:19-27 and
// src/binom_vanilla_eur.cpp:14-22 (this unit's host code is compiled with
// -ffp-contract=off, like the reference on x86-64).
void lattice(double r, double sigma, double T, int N, double& u, double& d, double& p,
             double& q, double& R) {
  const double dt = (double)T / (double)N;
  const double beta = 0.5 * (exp(-r * dt) + exp((r + pow(sigma, 2)) * dt));
  u = beta + sqrt(pow(beta, 2) - 1);
  d = beta - sqrt(pow(beta, 2) - 1);
  R = exp(r * dt);
  p = (R - d) / (u - d);
  q = 1 - p;
}

namespace {

constexpr int kEmin = -1;  // binades of the comb() accumulator with integer tables
constexpr int kEmax = 23;  // 2^24 > log(N!) for N <= 1e6
constexpr int kNbin = kEmax - kEmin + 1;
constexpr int kBinomBlock = 256;
constexpr int kMaxN = 1000000;
constexpr double kWindow = 8.0;  // half-width of the term window, in sqrt(N)

struct BinomTables {
  const double* logt;               // logt[n] = log((double)n), n = 0..nmax
  const unsigned long long* pref;   // [kNbin][nmax+1] prefix sums of D_e (mod 2^64)
  const int* tie_off;               // [kNbin+1]
  const int* tie_pos;               // sorted tie positions per binade
  int nmax;
};

struct BinomContract {
  double S0, E, u, d, lp, lq, logu, logd;
  double p, q;   // accurate mode
  int N, pf, i_lo, i_hi;  // pair indices i_lo..i_hi (inclusive)
  int has_mid, items, terms, pad;
};

struct BinomLaunch {
  const BinomContract* cs;
  const int* item_start;
  int ncontracts, total_items;
  double* partial;
  unsigned* tickets;
  double* out;
  int mode;
  const double* stirl;  // stirlerr(n), n = 0..15 (accurate mode)
  BinomTables t;
};

__device__ __forceinline__ int binade(double a) {
  return (int)((__double_as_longlong(a) >> 52) & 0x7ff) - 1023;
}
__device__ __forceinline__ long long to_units(double a) {
  return (__double_as_longlong(a) & 0xfffffffffffffLL) | (1LL << 52);
}
__device__ __forceinline__ double from_units(long long A, int e) {
  return __longlong_as_double(((long long)(e + 1023) << 52) | (A & 0xfffffffffffffLL));
}
// Most steps a stretch inside binade e can hold: every log n >= log 2.
__device__ __forceinline__ int stretch_cap(int e) {
  return (int)min(2000000000.0, ldexp(1.4427, e)) + 2;
}

__device__ int last_tie_le(const BinomTables& T, int b, int n) {
  int lo = T.tie_off[b], hi = T.tie_off[b + 1] - 1, ans = -1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const int v = T.tie_pos[mid];
    if (v <= n) { ans = v; lo = mid + 1; } else hi = mid - 1;
  }
  return ans;
}
__device__ int first_tie_ge(const BinomTables& T, int b, int j) {
  int lo = T.tie_off[b], hi = T.tie_off[b + 1] - 1, ans = INT_MAX;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const int v = T.tie_pos[mid];
    if (v >= j) { ans = v; hi = mid - 1; } else lo = mid + 1;
  }
  return ans;
}

// acc + log(hi) + log(hi-1) + ... + log(lo+1), each step rounded, in that order.
__device__ double add_chain_desc(const BinomTables& T, double acc, int hi, int lo) {
  int n = hi;
  const long long LIM = (1LL << 53) - 1;
  while (n > lo) {
    if (acc == 0.0) { acc = T.logt[n]; --n; continue; }
    const int e = binade(acc);
    if (e >= kEmin && e <= kEmax) {
      const int b = e - kEmin;
      const unsigned long long* P = T.pref + (size_t)b * (T.nmax + 1);
      long long A = to_units(acc);
      int mlo = max(lo + 1, n - stretch_cap(e) + 1);
      const int t = last_tie_le(T, b, n);
      if (t >= mlo) mlo = t + 1;
      if (mlo <= n && A + (long long)(P[n] - P[n - 1]) <= LIM) {
        int a = mlo, z = n;  // smallest m in [a, z] with A + sum(m..n) <= LIM
        while (a < z) {
          const int mid = (a + z) >> 1;
          if (A + (long long)(P[n] - P[mid - 1]) <= LIM) z = mid; else a = mid + 1;
        }
        A += (long long)(P[n] - P[a - 1]);
        acc = from_units(A, e);
        n = a - 1;
      }
    }
    if (n > lo) { acc = __dadd_rn(acc, T.logt[n]); --n; }
  }
  return acc;
}

// acc - log(lo) - log(lo+1) - ... - log(hi), each step rounded, in that order.
__device__ double sub_chain_asc(const BinomTables& T, double acc, int lo, int hi) {
  int j = lo;
  const long long FLOOR = (1LL << 52) + 1;
  while (j <= hi) {
    if (acc > 0.0) {
      const int e = binade(acc);
      if (e >= kEmin && e <= kEmax) {
        const int b = e - kEmin;
        const unsigned long long* P = T.pref + (size_t)b * (T.nmax + 1);
        long long A = to_units(acc);
        int mhi = (int)min((long long)hi, (long long)j + stretch_cap(e) - 1);
        const int t = first_tie_ge(T, b, j);
        if (t <= mhi) mhi = t - 1;
        if (mhi >= j && A - (long long)(P[j] - P[j - 1]) >= FLOOR) {
          int a = j, z = mhi;  // largest m in [a, z] with A - sum(j..m) >= FLOOR
          while (a < z) {
            const int mid = (a + z + 1) >> 1;
            if (A - (long long)(P[mid] - P[j - 1]) >= FLOOR) a = mid; else z = mid - 1;
          }
          A -= (long long)(P[a] - P[j - 1]);
          acc = from_units(A, e);
          j = a + 1;
        }
      }
    }
    if (j <= hi) { acc = __dsub_rn(acc, T.logt[j]); ++j; }
  }
  return acc;
}

// include/common.h:63-72, evaluated exactly.
__device__ double comb_ref(const BinomTables& T, int N, int i) {
  if (i == 0 || i == N) return 0.0;
  if (i == 1 || i == N - 1) return T.logt[N];
  const double acc = add_chain_desc(T, 0.0, N, i);
  return sub_chain_asc(T, acc, 2, N - i);
}

__device__ __forceinline__ double payoff_d(double S, double E, int pf) {
  return fmax(__dmul_rn((double)pf, __dsub_rn(S, E)), 0.0);
}

// ---- Loader's saddle-point terms (accurate mode) ----
__device__ double stirlerr(double n, const double* tab) {
  if (n <= 15.0) return tab[(int)n];
  const double S0 = 1.0 / 12, S1 = 1.0 / 360, S2 = 1.0 / 1260, S3 = 1.0 / 1680, S4 = 1.0 / 1188;
  const double nn = n * n;
  if (n > 500) return (S0 - S1 / nn) / n;
  if (n > 80) return (S0 - (S1 - S2 / nn) / nn) / n;
  if (n > 35) return (S0 - (S1 - (S2 - S3 / nn) / nn) / nn) / n;
  return (S0 - (S1 - (S2 - (S3 - S4 / nn) / nn) / nn) / nn) / n;
}

// bd0(x, np) = x log(x / np) + np - x, with the series for x near np.
__device__ double bd0(double x, double np) {
  if (fabs(x - np) < 0.1 * (x + np)) {
    const double v = (x - np) / (x + np);
    double s = (x - np) * v;
    double ej = 2 * x * v;
    const double v2 = v * v;
    for (int j = 1; j < 1000; ++j) {
      ej *= v2;
      const double s1 = s + ej / (2 * j + 1);
      if (s1 == s) return s1;
      s = s1;
    }
    return s;
  }
  return x * log(x / np) + np - x;
}

__device__ double log_dbinom(int k, int N, double p, double q, const double* stirl) {
  if (k == 0) return N * log1p(-p);
  if (k == N) return N * log(p);
  const double lc = stirlerr((double)N, stirl) - stirlerr((double)k, stirl) -
                    stirlerr((double)(N - k), stirl) - bd0((double)k, N * p) -
                    bd0((double)(N - k), N * q);
  const double lf = 1.8378770664093454836 + log((double)k) + log1p(-(double)k / N);  // log(2 pi k (N-k)/N)
  return lc - 0.5 * lf;
}

// src/binom_embar.cpp:35-40: the terms of pair index i in the reference's order.
__device__ double pair_terms(const BinomLaunch& L, const BinomContract& C, int i) {
  const int N = C.N;
  double t1, t2;
  if (L.mode == 0) {
    const double cv = comb_ref(L.t, N, i);
    const double b1 = __dadd_rn(__dadd_rn(cv, __dmul_rn((double)i, C.lp)),
                                __dmul_rn((double)(N - i), C.lq));
    const double b2 = __dadd_rn(__dadd_rn(cv, __dmul_rn((double)(N - i), C.lp)),
                                __dmul_rn((double)i, C.lq));
    t1 = exp(b1);
    t2 = exp(b2);
  } else {
    t1 = exp(log_dbinom(i, N, C.p, C.q, L.stirl));
    t2 = exp(log_dbinom(N - i, N, C.p, C.q, L.stirl));
  }
  const double s1 = __dmul_rn(__dmul_rn(C.S0, pow(C.u, (double)i)), pow(C.d, (double)(N - i)));
  const double s2 = __dmul_rn(__dmul_rn(C.S0, pow(C.u, (double)(N - i))), pow(C.d, (double)i));
  return __dadd_rn(__dmul_rn(t1, payoff_d(s1, C.E, C.pf)), __dmul_rn(t2, payoff_d(s2, C.E, C.pf)));
}

// src/binom_embar.cpp:42-45: the middle term of an even N.
__device__ double mid_term(const BinomLaunch& L, const BinomContract& C) {
  const int N = C.N, h = N / 2;
  double w;
  if (L.mode == 0) {
    const double cv = comb_ref(L.t, N, h);
    w = exp(__dadd_rn(__dadd_rn(cv, __dmul_rn((double)h, C.lp)), __dmul_rn((double)h, C.lq)));
  } else {
    w = exp(log_dbinom(h, N, C.p, C.q, L.stirl));
  }
  const double s = __dmul_rn(__dmul_rn(C.S0, pow(C.u, (double)h)), pow(C.d, (double)h));
  return __dmul_rn(w, payoff_d(s, C.E, C.pf));
}

__device__ __forceinline__ int find_item_contract(const int* start, int n, int item) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kBinomBlock) binom_kernel(BinomLaunch L) {
  __shared__ double sh[32];
  const int item = blockIdx.x;
  if (item >= L.total_items) return;
  const int c = find_item_contract(L.item_start, L.ncontracts, item);
  const BinomContract C = L.cs[c];
  const int j = item - L.item_start[c];
  const int ti = j * kBinomBlock + threadIdx.x;
  double v = 0.0;
  if (ti < C.terms) {
    const int i = C.i_lo + ti;
    if (i <= C.i_hi) v = pair_terms(L, C, i);
    else if (C.has_mid) v = mid_term(L, C);
  }
  double vv[1] = {v}, tot[1];
  block_sum<1>(vv, sh, tot);
  grid_finalize<1>(tot, L.partial + L.item_start[c], L.tickets + c, L.out + c, C.items, j);
}

// ---- host side ----

struct HostTables {
  std::vector<double> logt;
  std::vector<unsigned long long> pref;
  std::vector<int> tie_off, tie_pos;
};

// D_e[n] = round-half-away... of log n / u_e: floor plus [frac > 1/2], with
// frac == 1/2 recorded as a tie. Exact: log n * 2^{52-e} is a power-of-two
// scaling of a double, so floor and fraction are exact.
void build_tables(int nmax, HostTables& H) {
  H.logt.resize((size_t)nmax + 1);
  H.logt[0] = -INFINITY;
  for (int n = 1; n <= nmax; ++n) H.logt[n] = log((double)n);
  H.pref.assign((size_t)kNbin * (nmax + 1), 0ULL);
  H.tie_off.assign(kNbin + 1, 0);
  H.tie_pos.clear();
  for (int b = 0; b < kNbin; ++b) {
    const int e = b + kEmin;
    unsigned long long run = 0;
    unsigned long long* P = &H.pref[(size_t)b * (nmax + 1)];
    P[0] = 0;
    H.tie_off[b] = (int)H.tie_pos.size();
    for (int n = 1; n <= nmax; ++n) {
      const double x = ldexp(H.logt[n], 52 - e);
      const double F = floor(x);
      const double f = x - F;
      unsigned long long D = (unsigned long long)F;
      if (f > 0.5) D += 1;
      else if (f == 0.5) H.tie_pos.push_back(n);
      run += D;
      P[n] = run;
    }
  }
  H.tie_off[kNbin] = (int)H.tie_pos.size();
}

// stirlerr(n) = log(n!) - (n + 1/2) log n + n - log(sqrt(2 pi)), n = 1..15, in
// long double; stirlerr(0) is unused (k = 0 has its own formula).
void stirlerr_table(double* out) {
  out[0] = 0.0;
  for (int n = 1; n <= 15; ++n) {
    const long double ln = (long double)n;
    out[n] = (double)(lgammal(ln + 1) - (ln + 0.5L) * logl(ln) + ln -
                      0.5L * logl(2 * 3.14159265358979323846264338327950288L));
  }
}

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

int ensure_tables(pcf_ctx* c, int nmax) {
  if (c->d_logtab && c->logtab_n >= nmax) return PCF_OK;
  // Grown by doubling from 4096 entries: a one-off small N builds a small
  // table (its build is ~0.1 microsecond per entry and binade), a sequence
  // of growing N rebuilds it a logarithmic number of times.
  int want = 4096;
  while (want < nmax && want < kMaxN) want *= 2;
  want = std::min(std::max(want, nmax), kMaxN);
  HostTables H;
  build_tables(want, H);
  const size_t b_log = sizeof(double) * (want + 1);
  const size_t b_pref = sizeof(unsigned long long) * H.pref.size();
  const size_t b_off = sizeof(int) * H.tie_off.size();
  const size_t b_pos = sizeof(int) * std::max<size_t>(1, H.tie_pos.size());
  const size_t o_pref = a256(b_log), o_off = a256(o_pref + b_pref), o_pos = a256(o_off + b_off);
  const size_t o_stir = a256(o_pos + b_pos);
  const size_t total = a256(o_stir + 16 * sizeof(double));
  if (c->d_logtab) cudaFree(c->d_logtab);
  c->d_logtab = nullptr;
  c->logtab_n = 0;
  if (c->budget_bytes && total > c->budget_bytes)
    return set_error(PCF_ENOMEM, "binomial tables of %zu bytes exceed the context budget", total);
  void* d = nullptr;
  int st = cuda_status(cudaMalloc(&d, total), "cudaMalloc(binomial tables)");
  if (st) return st;
  std::vector<char> h(total, 0);
  memcpy(&h[0], H.logt.data(), b_log);
  memcpy(&h[o_pref], H.pref.data(), b_pref);
  memcpy(&h[o_off], H.tie_off.data(), b_off);
  if (!H.tie_pos.empty()) memcpy(&h[o_pos], H.tie_pos.data(), sizeof(int) * H.tie_pos.size());
  stirlerr_table((double*)&h[o_stir]);
  st = cuda_status(cudaMemcpy(d, h.data(), total, cudaMemcpyHostToDevice), "H2D binomial tables");
  if (st) {
    cudaFree(d);
    return st;
  }
  c->d_logtab = (double*)d;
  c->logtab_n = want;
  c->binom_off[0] = o_pref;
  c->binom_off[1] = o_off;
  c->binom_off[2] = o_pos;
  c->binom_off[3] = o_stir;
  return PCF_OK;
}

int setup_contract(const pcf_binom_contract& k, int idx, BinomContract& C) {
  const int pf = k.payoff_fun;
  if (pf != 1 && pf != -1)
    return set_error(PCF_EINVAL, "contract %d: Unknown payoff function", idx);
  if (!(k.S0 > 0) || !(k.E >= 0) || !(k.sigma > 0) || !(k.T > 0) || !std::isfinite(k.r) ||
      !std::isfinite(k.S0) || !std::isfinite(k.E) || !std::isfinite(k.sigma) ||
      !std::isfinite(k.T))
    return set_error(PCF_EINVAL, "contract %d: need S0 > 0, E >= 0, sigma > 0, T > 0", idx);
  if (k.N < 1 || k.N > kMaxN)
    return set_error(PCF_EINVAL, "contract %d: N must be in [1, %d]", idx, kMaxN);
  const int N = k.N;
  double u, d, p, q, R;
  lattice(k.r, k.sigma, k.T, N, u, d, p, q, R);
  if (!(p > 0 && p < 1)) return set_error(PCF_EINVAL, "contract %d: lattice p = %g not in (0,1)", idx, p);
  memset(&C, 0, sizeof C);
  C.S0 = k.S0;
  C.E = k.E;
  C.u = u;
  C.d = d;
  C.p = p;
  C.q = q;
  C.lp = log(p);
  C.lq = log(q);
  C.logu = log(u);
  C.logd = log(d);
  C.N = N;
  C.pf = pf;
  const int until = (N % 2 != 0) ? (N + 1) / 2 : N / 2;  // src/binom_embar.cpp:31-33
  const double ps = p * u / R;
  const double w = kWindow * sqrt((double)N) + 2;
  const double klo = std::max(0.0, floor(N * std::min(p, ps) - w));
  const double khi = std::min((double)N, ceil(N * std::max(p, ps) + w));
  const long long ilo = (long long)std::max(0.0, std::min(klo, N - khi));
  const long long ihi = std::min((long long)until - 1, (long long)std::max(khi, N - klo));
  C.i_lo = (int)ilo;
  C.i_hi = (int)ihi;
  C.has_mid = (N % 2 == 0 && N / 2 >= klo && N / 2 <= khi) ? 1 : 0;
  C.terms = std::max(0, C.i_hi - C.i_lo + 1) + C.has_mid;
  C.items = std::max(1, (C.terms + kBinomBlock - 1) / kBinomBlock);
  return PCF_OK;
}

}  // namespace

}  // namespace pcf

using namespace pcf;

extern "C" int pcf_binom_embar_batch(pcf_ctx* ctx, int n, const pcf_binom_contract* ks, int mode,
                                     double* prices) {
  return pcf::abi_guard([&]() -> int {
    if (n < 0 || (n > 0 && (!ks || !prices))) return set_error(PCF_EINVAL, "bad arguments");
    if (mode != 0 && mode != 1) return set_error(PCF_EINVAL, "mode must be 0 or 1");
    if (n == 0) return PCF_OK;
    std::vector<BinomContract> cs((size_t)n);
    int nmax = 1;
    for (int i = 0; i < n; ++i) {
      int st = setup_contract(ks[i], i, cs[i]);
      if (st) return st;
      nmax = std::max(nmax, ks[i].N);
    }
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    st = ensure_tables(c, nmax);
    if (st) return st;
    std::vector<int> start((size_t)n + 1, 0);
    for (int i = 0; i < n; ++i) start[i + 1] = start[i] + cs[i].items;
    const int items = start[n];
    const size_t o_cs = 0;
    const size_t o_start = a256(sizeof(BinomContract) * n);
    const size_t h2d = a256(o_start + sizeof(int) * (n + 1));
    const size_t o_part = h2d;
    const size_t o_tick = a256(o_part + sizeof(double) * items);
    const size_t o_out = a256(o_tick + sizeof(unsigned) * n);
    const size_t total = a256(o_out + sizeof(double) * n);
    st = ctx_ensure(c, total, std::max(h2d, sizeof(double) * n));
    if (st) return st;
    char* h = (char*)c->h_buf;
    char* d = (char*)c->d_buf;
    memcpy(h + o_cs, cs.data(), sizeof(BinomContract) * n);
    memcpy(h + o_start, start.data(), sizeof(int) * (n + 1));
    st = cuda_status(cudaMemcpyAsync(d, h, h2d, cudaMemcpyHostToDevice, c->stream), "H2D binom");
    if (!st) st = cuda_status(cudaMemsetAsync(d + o_tick, 0, sizeof(unsigned) * n, c->stream),
                              "memset binom tickets");
    if (st) return st;
    BinomLaunch L;
    L.cs = (const BinomContract*)(d + o_cs);
    L.item_start = (const int*)(d + o_start);
    L.ncontracts = n;
    L.total_items = items;
    L.partial = (double*)(d + o_part);
    L.tickets = (unsigned*)(d + o_tick);
    L.out = (double*)(d + o_out);
    L.mode = mode;
    char* tb = (char*)c->d_logtab;
    L.t.logt = (const double*)tb;
    L.t.pref = (const unsigned long long*)(tb + c->binom_off[0]);
    L.t.tie_off = (const int*)(tb + c->binom_off[1]);
    L.t.tie_pos = (const int*)(tb + c->binom_off[2]);
    L.stirl = (const double*)(tb + c->binom_off[3]);
    L.t.nmax = c->logtab_n;
    binom_kernel<<<items, kBinomBlock, 0, c->stream>>>(L);
    st = cuda_status(cudaGetLastError(), "binom kernel launch");
    if (st) return st;
    c->launches += 1;
    st = cuda_status(cudaMemcpyAsync(h, L.out, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                     c->stream), "D2H binom");
    if (!st) st = cuda_status(cudaStreamSynchronize(c->stream), "binom kernel");
    if (st) return st;
    for (int i = 0; i < n; ++i) prices[i] = exp(-ks[i].r * ks[i].T) * ((double*)h)[i];  // :49
    return PCF_OK;
  });
}

extern "C" int pcf_binom_embar(pcf_ctx* ctx, double S0, double E, double r, double sigma,
                               double T, int N, int payoff_fun, int mode, double* price) {
  return pcf::abi_guard([&]() -> int {
    if (!price) return set_error(PCF_EINVAL, "price is NULL");
    pcf_binom_contract k{S0, E, r, sigma, T, N, payoff_fun};
    return pcf_binom_embar_batch(ctx, 1, &k, mode, price);
  });
}
