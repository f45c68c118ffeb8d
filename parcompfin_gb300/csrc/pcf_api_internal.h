// Host-side internals shared by the C-ABI translation units: the context
// object and the helpers that validate, allocate and report errors.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>

#include <algorithm>
#include <exception>
#include <new>
#include <vector>

#include "../../include/pcf.h"
#include "pcf_internal.h"
#include "pcf_tune.h"

struct pcf_ctx {
  int device = 0;
  int sm_count = 1;
  cudaStream_t stream = nullptr;
  // Scratch arena for launch parameters, partial sums and results; grown on
  // demand and reused by every call on this context.
  void* d_buf = nullptr;
  size_t d_cap = 0;
  void* h_buf = nullptr;  // pinned staging
  size_t h_cap = 0;
  // Longstaff-Schwartz path matrix and per-path state, kept resident.
  void* d_paths = nullptr;
  size_t paths_cap = 0;
  // log((double)n) table for the reference-order binomial sum.
  double* d_logtab = nullptr;  // one allocation: log table, prefix tables, ties
  int logtab_n = 0;
  size_t binom_off[4] = {0, 0, 0, 0};  // offsets of prefix sums, tie offsets, ties, stirlerr
  // Serving slots of pcf_serve_trace, kept between calls (pcf_server.cpp).
  void* serve = nullptr;
  // Upper bound on device bytes this context may hold (0 = unlimited).
  size_t budget_bytes = 0;
  // Test hook (pcf_ctx_set_test_barrier): the cooperative group barriers of
  // pcf_mc_amer and pcf_binom_vanilla expect this many arrivals beyond their
  // grid, so they cannot complete, and give up after test_poll_limit polls.
  unsigned test_barrier_extra = 0;
  unsigned test_poll_limit = 0;
  long long launches = 0;
};

namespace pcf {

int set_error(int status, const char* fmt, ...);

// Runs the body of a C entry point and turns a C++ exception thrown inside it
// (host memory exhausted in a std::vector, a failed thread start) into a
// status with its message: no exception crosses the C ABI.
template <class Body>
int abi_guard(Body&& body) noexcept {
  try {
    return body();
  } catch (const std::bad_alloc&) {
    return set_error(PCF_ENOMEM, "host memory exhausted");
  } catch (const std::exception& e) {
    return set_error(PCF_EINVAL, "internal error: %s", e.what());
  } catch (...) {
    return set_error(PCF_EINVAL, "internal error");
  }
}
int cuda_status(cudaError_t e, const char* what);
int ctx_ensure(pcf_ctx* c, size_t dev_bytes, size_t host_bytes);
pcf_ctx* resolve_ctx(pcf_ctx* ctx, int* status);
void ctx_release_extras(pcf_ctx* c);
void serve_release(pcf_ctx* c);  // frees the serving slots (pcf_server.cpp)
int check_common(double S0, double E, double r, double sigma, double T, long long N, int pf);
void fill_result(const double* s, long long n, double mu_g, double disc, bool use_cv,
                 pcf_mc_result* out);

// Contract builders; the work-item sizes come from the tuning table.
McContract make_eur(double S0, double E, double r, double sigma, double T, long long N, int pf,
                    unsigned long long seed, uint32_t stream, const TuneTable& t);
McContract make_asia(double S0, double E, double r, double sigma, double T, long long N, int M,
                     int pf, int mode, unsigned long long seed, uint32_t stream,
                     const TuneTable& t);
double asia_cv_mean(double S0, double E, double r, double sigma, double T, int M, int pf,
                    int mode);
int make_basket(int d, const double* S0, const double* sig, const double* corr, double r,
                double T, double E, long long N, int pf, double ts, unsigned long long seed,
                uint32_t stream, std::vector<float>& fb, McContract& k, double& mu_g,
                const TuneTable& t);

// The reference's beta-parametrised lattice (binom.cu).
void lattice(double r, double sigma, double T, int N, double& u, double& d, double& p,
             double& q, double& R);

// American (Longstaff-Schwartz) contracts in a batch (lsm.cu).
struct LsmRequest {
  double S0, E, r, sigma, T;
  long long N;
  int M, pf, ref_exercise;
  unsigned long long seed;
  unsigned stream;
  double* d_out;   // kMoments sums, device
  int* d_flags;    // {wait gave up, singular dates}, device, zeroed before a launch
};
struct LsmBatch;
int check_lsm_request(double S0, double E, double r, double sigma, double T, long long N, int M,
                      int pf);
void fill_amer_result(const double* s, long long N, double S0, double E, double r, double sigma,
                      double T, int pf, bool use_cv, pcf_mc_result* out);
// Caller-provided memory for building a batch without allocating: bump
// allocation from a device region and a pinned host region (256-byte aligned).
// A failed allocation records how far the region would have had to reach
// (d_short / h_short), so a caller that owns the regions can grow them and
// build again.
struct ExtMem {
  char* d = nullptr;
  size_t d_cap = 0, d_used = 0, d_short = 0;
  char* h = nullptr;
  size_t h_cap = 0, h_used = 0, h_short = 0;
  char* dalloc(size_t n) {
    const size_t o = (d_used + 255) & ~(size_t)255;
    if (o + n > d_cap) {
      d_short = std::max(d_short, o + n);
      return nullptr;
    }
    d_used = o + n;
    return d + o;
  }
  char* halloc(size_t n) {
    const size_t o = (h_used + 255) & ~(size_t)255;
    if (o + n > h_cap) {
      h_short = std::max(h_short, o + n);
      return nullptr;
    }
    h_used = o + n;
    return h + o;
  }
};
int lsm_batch_bytes(pcf_ctx* c, const std::vector<LsmRequest>& reqs, size_t* dev,
                    size_t* host);
// With mem == NULL the batch allocates its own device memory and uploads
// synchronously; otherwise it takes memory from mem and only queues the upload on s.
int lsm_batch_create(pcf_ctx* c, const std::vector<LsmRequest>& reqs, cudaStream_t s,
                     ExtMem* mem, LsmBatch** out);
int lsm_batch_launch(pcf_ctx* c, LsmBatch* b, cudaStream_t s);
// The two parts of lsm_batch_launch: the cluster launches, then the
// cooperative ones (which need every block resident, so they run alone).
int lsm_batch_launch_clusters(pcf_ctx* c, LsmBatch* b, cudaStream_t s);
int lsm_batch_launch_coop(pcf_ctx* c, LsmBatch* b, cudaStream_t s);
int lsm_batch_kernels(const LsmBatch* b);
int lsm_batch_cluster_kernels(const LsmBatch* b);
void lsm_batch_destroy(LsmBatch* b);

}  // namespace pcf
