// Drop-in command-line programs for the reference's pricing binaries.
//
// The reference builds one program per method and variant (bin/mc_eur,
// bin/mc_eur_omp, bin/mc_eur_mpi, bin/mc_eur_hybrid, ... ; src/*.cpp main()).
// Each reads its parameters from argv, prices once and prints one CSV line
// with reporting() (include/common.h:212-249). This program accepts the same
// argv and prints the same 16 columns,
//   Method,Payoff,S0,E,r,sigma,T,N,M,Parallel,Nr_of_assets,T_overall,
//   T_calculation,Result,Abs_Error,Error
// with numbers formatted like std::setprecision(10) (%.10g), pricing on the
// GPU through the C ABI. It is one binary; the name it is invoked under
// (bin/<reference name>, a symlink) or its first argument selects the
// program:
//   mc_eur[_omp|_mpi|_hybrid]        payoff S0 E r sigma T N [threads]
//   mc_eur_multi[_omp|_mpi|_hybrid]  payoff S0 E r sigma T N assets rho [threads]
//   mc_asia[_omp|_mpi|_hybrid]       payoff S0 E r sigma T N M [threads]
//   mc_amer[_omp|_mpi|_hybrid]       payoff S0 E r sigma T N M [threads]
//   binom_embar[_omp|_mpi|_hybrid]   payoff S0 E r sigma T N [threads]
//   binom_vanilla_eur, binom_vanilla_amer   payoff S0 E r sigma T N
// The threads argument is accepted and reported in the Parallel column, as
// the reference's OpenMP (threads), MPI (ranks) and hybrid
// (ranks*1000 + threads) programs report it.
//
// Environment (all optional):
//   PCF_COMPARISON       the value Abs_Error/Error compare against; default:
//                        `comparison = <x>;` read from include/comparison.h
//                        in the working directory (the reference's run
//                        scripts write that file), else 0
//   PCF_SEED             Philox seed; default time(NULL), like the reference
//   PCF_REF_EXERCISE     mc_amer: unset or 1 (the default) keeps the
//                        reference's exercise rule (src/mc_amer.cpp:100),
//                        so the program prints what the reference's prints
//                        (about 94 for an at-the-money put); 0 exercises at
//                        payoff(S), correct Longstaff-Schwartz
//   PCF_CV=1             report the control-variate estimate
//   PCF_BINOM_MODE=1     binom_embar: accurate weights; default 0 reproduces
//                        the reference's rounding
//   PCF_FULL_PRECISION=1 print Result, Abs_Error and Error with %.17g
//   PCF_METHOD           replaces the Method column (default: the
//                        reference's label of the variant invoked)
//   PCF_DEVICE           CUDA device (default 0)
//   PCF_RANKS            the process count the MPI and hybrid programs report
//                        (default 1: one process drives the GPU)
// Errors: the reference throws std::invalid_argument (an unknown payoff, an
// odd LSM path count, a singular regression) and aborts. Here the message
// goes to stderr and the exit status is 1.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <chrono>
#include <string>

#include "../../include/pcf.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Variant {
  const char* label;  // Method column
  int threads_arg;    // 1 if argv carries a threads argument
};

int fail(const char* msg) {
  fprintf(stderr, "%s\n", msg);
  return 1;
}

// std::stod / std::stoi semantics: leading whitespace, a number, anything
// after it ignored; no number is an error.
bool arg_d(char** argv, int argc, int idx, double* out) {
  if (idx >= argc) return false;
  char* end = nullptr;
  *out = strtod(argv[idx], &end);
  return end != argv[idx];
}
bool arg_i(char** argv, int argc, int idx, long long* out) {
  if (idx >= argc) return false;
  char* end = nullptr;
  *out = strtoll(argv[idx], &end, 10);
  return end != argv[idx];
}

bool env_flag(const char* name, bool dflt = false) {
  const char* v = getenv(name);
  if (!v || !*v) return dflt;
  return strcmp(v, "0") != 0;
}

double comparison_value() {
  if (const char* v = getenv("PCF_COMPARISON")) return strtod(v, nullptr);
  FILE* f = fopen("include/comparison.h", "r");
  if (!f) return 0.0;
  char buf[4096];
  const size_t n = fread(buf, 1, sizeof buf - 1, f);
  fclose(f);
  buf[n] = 0;
  const char* p = strstr(buf, "comparison");
  if (!p) return 0.0;
  p = strchr(p, '=');
  return p ? strtod(p + 1, nullptr) : 0.0;
}

void print_num(double x, bool full) { printf(full ? "%.17g" : "%.10g", x); }

// include/common.h:212-249: the column order of reporting().
void report(const char* method, const char* payoff, double S0, double E, double r,
            double sigma, double T, long long N, int M, long long parallel, int assets,
            double t_overall, double t_calc, double result, double comparison) {
  const bool full = env_flag("PCF_FULL_PRECISION");
  const char* label = getenv("PCF_METHOD");
  printf("%s,%s,", label && *label ? label : method, payoff);
  const double lead[5] = {S0, E, r, sigma, T};
  for (double v : lead) {
    print_num(v, false);
    printf(",");
  }
  printf("%lld,%d,%lld,%d,", N, M, parallel, assets);
  print_num(t_overall, false);
  printf(",");
  print_num(t_calc, false);
  printf(",");
  print_num(result, full);
  printf(",");
  print_num(fabs(result - comparison), full);
  printf(",");
  print_num(result - comparison, full);
  printf("\n");
}

const char* base_name(const char* p) {
  const char* s = strrchr(p, '/');
  return s ? s + 1 : p;
}

bool ends_with(const std::string& s, const char* suf, std::string* stem) {
  const size_t n = strlen(suf);
  if (s.size() < n || s.compare(s.size() - n, n, suf) != 0) return false;
  *stem = s.substr(0, s.size() - n);
  return true;
}

int usage() {
  fprintf(stderr,
          "usage: pcf_cli <program> args...   or invoke as bin/<program>\n"
          "  mc_eur[_omp|_mpi|_hybrid]       payoff S0 E r sigma T N [threads]\n"
          "  mc_eur_multi[_omp|_mpi|_hybrid] payoff S0 E r sigma T N assets rho [threads]\n"
          "  mc_asia[_omp|_mpi|_hybrid]      payoff S0 E r sigma T N M [threads]\n"
          "  mc_amer[_omp|_mpi|_hybrid]      payoff S0 E r sigma T N M [threads]\n"
          "  binom_embar[_omp|_mpi|_hybrid]  payoff S0 E r sigma T N [threads]\n"
          "  binom_vanilla_eur, binom_vanilla_amer  payoff S0 E r sigma T N\n");
  return 2;
}

}  // namespace

int main(int argc, char** argv) {
  const Clock::time_point start_overall = Clock::now();
  std::string prog = base_name(argv[0]);
  if (prog.compare(0, 4, "pcf_") == 0) prog = prog.substr(4);
  int a0 = 0;  // argv index of the program name
  if (prog == "cli") {
    if (argc < 2) return usage();
    prog = argv[1];
    a0 = 1;
  }
  std::string stem = prog;
  Variant var{"Serial", 0};
  if (prog == "binom_vanilla_eur" || prog == "binom_vanilla_amer") var = Variant{"Serial_vanilla", 0};
  else if (ends_with(prog, "_omp", &stem)) var = Variant{"OMP", 1};
  else if (ends_with(prog, "_mpi", &stem)) var = Variant{"MPI", 0};
  else if (ends_with(prog, "_hybrid", &stem)) var = Variant{"Hybrid", 1};
  char** av = argv + a0;
  const int ac = argc - a0;

  const int nbase = stem == "mc_eur_multi" ? 10 : (stem == "mc_asia" || stem == "mc_amer") ? 9
                                                                                             : 8;
  if (stem != "mc_eur" && stem != "mc_eur_multi" && stem != "mc_asia" && stem != "mc_amer" &&
      stem != "binom_embar" && stem != "binom_vanilla_eur" && stem != "binom_vanilla_amer")
    return usage();
  if (ac < nbase + var.threads_arg) return usage();
  const char* payoff = av[1];
  double S0, E, r, sigma, T, rho = 0.0;
  long long N, M = 0, assets = 1, threads = 0;
  if (!arg_d(av, ac, 2, &S0) || !arg_d(av, ac, 3, &E) || !arg_d(av, ac, 4, &r) ||
      !arg_d(av, ac, 5, &sigma) || !arg_d(av, ac, 6, &T) || !arg_i(av, ac, 7, &N))
    return fail("invalid numeric argument");
  int next = 8;
  if (stem == "mc_eur_multi") {
    if (!arg_i(av, ac, 8, &assets) || !arg_d(av, ac, 9, &rho))
      return fail("invalid numeric argument");
    next = 10;
  } else if (stem == "mc_asia" || stem == "mc_amer") {
    if (!arg_i(av, ac, 8, &M)) return fail("invalid numeric argument");
    next = 9;
  }
  if (var.threads_arg && !arg_i(av, ac, next, &threads)) return fail("invalid numeric argument");
  const char* rk = getenv("PCF_RANKS");
  const long long ranks = rk && *rk ? atoll(rk) : 1;
  long long parallel = 0;
  if (strcmp(var.label, "OMP") == 0) parallel = threads;
  else if (strcmp(var.label, "MPI") == 0) parallel = ranks;
  else if (strcmp(var.label, "Hybrid") == 0) parallel = ranks * 1000 + threads;

  // src/mc_eur.cpp:38-41: call -> 1, put -> -1, anything else is an error.
  int pf;
  if (strcmp(payoff, "call") == 0) pf = 1;
  else if (strcmp(payoff, "put") == 0) pf = -1;
  else return fail("Unknown payoff function");

  const char* sv = getenv("PCF_SEED");
  const unsigned long long seed =
      sv ? strtoull(sv, nullptr, 10) : (unsigned long long)time(nullptr);
  const bool cv = env_flag("PCF_CV");
  const char* dv = getenv("PCF_DEVICE");
  pcf_ctx* ctx = nullptr;
  int st = pcf_ctx_create(dv ? atoi(dv) : 0, &ctx);
  if (st) {
    fprintf(stderr, "%s: %s\n", pcf_strerror(st), pcf_last_error());
    return 1;
  }

  double result = 0.0;
  pcf_mc_result res;
  const Clock::time_point start = Clock::now();
  if (stem == "mc_eur") {
    st = pcf_mc_eur(ctx, S0, E, r, sigma, T, N, pf, seed, cv, &res);
  } else if (stem == "mc_eur_multi") {
    st = pcf_mc_eur_multi(ctx, S0, E, r, sigma, T, N, pf, (int)assets, rho, seed, cv, &res);
  } else if (stem == "mc_asia") {
    st = pcf_mc_asia(ctx, S0, E, r, sigma, T, N, (int)M, pf, 0, seed, cv, &res);
  } else if (stem == "mc_amer") {
    st = pcf_mc_amer(ctx, S0, E, r, sigma, T, N, (int)M, pf, env_flag("PCF_REF_EXERCISE", true), seed,
                     cv, &res);
  } else if (stem == "binom_embar") {
    st = pcf_binom_embar(ctx, S0, E, r, sigma, T, (int)N, pf, env_flag("PCF_BINOM_MODE"),
                         &result);
  } else {
    st = pcf_binom_vanilla(ctx, S0, E, r, sigma, T, (int)N, pf, stem == "binom_vanilla_amer",
                           &result);
  }
  const Clock::time_point end = Clock::now();
  if (st) {
    fprintf(stderr, "%s\n", pcf_last_error());
    pcf_ctx_destroy(ctx);
    return 1;
  }
  if (stem.compare(0, 5, "binom") != 0) result = cv ? res.price_cv : res.price_plain;
  const double t_calc = std::chrono::duration<double>(end - start).count();
  const double t_overall = std::chrono::duration<double>(end - start_overall).count();
  const int m_col = (stem == "mc_asia" || stem == "mc_amer") ? (int)M : 0;
  report(var.label, payoff, S0, E, r, sigma, T, N, m_col, parallel, (int)assets, t_overall,
         t_calc, result, comparison_value());
  pcf_ctx_destroy(ctx);
  return 0;
}
