/* Seed injection and C entry points for the reference's pricing functions.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref). Linked into one shared object per
 * reference source file by oracle/build_ref.sh, with -Wl,-Bsymbolic so that
 * the reference's calls to time() bind to the definition below. The reference
 * seeds std::mt19937 with time() (e.g. src/mc_eur.cpp:19); here time() returns
 * the seed the caller set, which makes every run reproducible.
 *
 * REF_FN names the reference function and REF_KIND selects its signature:
 *   1: double f(S0,E,r,sigma,T,int N,double pf)                 mc_eur, binom
 *   2: double f(S0,E,r,sigma,T,int N,int M,double pf)           mc_asia, mc_amer
 *   3: double f(S0,E,r,sigma,T,int N,int M,double pf,int thr)   mc_amer (OpenMP)
 */
#include <ctime>
#include <omp.h>

static time_t g_seed = 0;

extern "C" time_t time(time_t* t) {
  if (t) *t = g_seed;
  return g_seed;
}

extern "C" void ref_set_seed(long long s) { g_seed = (time_t)s; }
extern "C" void ref_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }

#if REF_KIND == 1
double REF_FN(double, double, double, double, double, int, double);
extern "C" double ref_call(double S0, double E, double r, double sigma, double T, int N, int M,
                           double pf, int threads) {
  (void)M; (void)threads;
  return REF_FN(S0, E, r, sigma, T, N, pf);
}
#elif REF_KIND == 2
double REF_FN(double, double, double, double, double, int, int, double);
extern "C" double ref_call(double S0, double E, double r, double sigma, double T, int N, int M,
                           double pf, int threads) {
  (void)threads;
  return REF_FN(S0, E, r, sigma, T, N, M, pf);
}
#elif REF_KIND == 3
double REF_FN(double, double, double, double, double, int, int, double, int);
extern "C" double ref_call(double S0, double E, double r, double sigma, double T, int N, int M,
                           double pf, int threads) {
  return REF_FN(S0, E, r, sigma, T, N, M, pf, threads);
}
#endif
