// C-ABI layer of libpcf.so: contexts, parameter validation, launch planning
// and estimators for the pricing entry points declared in include/pcf.h.
#include "pcf_api_internal.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "pcf_math.h"

namespace pcf {

static thread_local char g_err[512];  // the calling thread's last error (no allocation)
static thread_local pcf_ctx* g_default_ctx = nullptr;

int set_error(int status, const char* fmt, ...) {
  char buf[sizeof g_err];  // an argument may be the previous message itself
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  memcpy(g_err, buf, sizeof buf);
  return status;
}

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return PCF_OK;
  const int st = (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? PCF_ENODEV
                 : (e == cudaErrorMemoryAllocation)                          ? PCF_ENOMEM
                                                                              : PCF_ECUDA;
  return set_error(st, "%s: %s", what, cudaGetErrorString(e));
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

void ctx_release_extras(pcf_ctx* c) {
  if (c->d_paths) cudaFree(c->d_paths);
  c->d_paths = nullptr;
  c->paths_cap = 0;
  if (c->d_logtab) cudaFree(c->d_logtab);
  c->d_logtab = nullptr;
  c->logtab_n = 0;
}

int ctx_ensure(pcf_ctx* c, size_t dev_bytes, size_t host_bytes) {
  if (dev_bytes > c->d_cap) {
    if (c->d_buf) cudaFree(c->d_buf);
    c->d_buf = nullptr;
    c->d_cap = 0;
    const size_t want = std::max(align256(dev_bytes), (size_t)1 << 20);
    if (c->budget_bytes && want > c->budget_bytes)
      return set_error(PCF_ENOMEM, "scratch of %zu bytes exceeds the context budget of %zu",
                       want, c->budget_bytes);
    int st = cuda_status(cudaMalloc(&c->d_buf, want), "cudaMalloc(scratch)");
    if (st) return st;
    c->d_cap = want;
  }
  if (host_bytes > c->h_cap) {
    if (c->h_buf) cudaFreeHost(c->h_buf);
    c->h_buf = nullptr;
    c->h_cap = 0;
    const size_t want = std::max(align256(host_bytes), (size_t)1 << 16);
    int st = cuda_status(cudaMallocHost(&c->h_buf, want), "cudaMallocHost(staging)");
    if (st) return st;
    c->h_cap = want;
  }
  return PCF_OK;
}

pcf_ctx* resolve_ctx(pcf_ctx* ctx, int* status) {
  *status = PCF_OK;
  if (ctx) {
    cudaSetDevice(ctx->device);
    return ctx;
  }
  if (!g_default_ctx) {
    // The default context is kept for the thread's lifetime; it is not torn
    // down at exit because the CUDA runtime may already be gone by then.
    *status = pcf_ctx_create(0, &g_default_ctx);
    if (*status) return nullptr;
  }
  cudaSetDevice(g_default_ctx->device);
  return g_default_ctx;
}

// Runs one batch of MC contracts of one method and returns the moment sums
// (C * kMoments doubles). Contracts must have units_per_item and items set.
int run_mc(pcf_ctx* c, McMethod m, std::vector<McContract>& cs, const std::vector<float>& fb,
           int max_d, int block, bool tensor, bool persistent, bool cv,
           std::vector<double>& sums) {
  const int C = (int)cs.size();
  std::vector<int> start((size_t)C + 1, 0);
  for (int i = 0; i < C; ++i) {
    if ((long long)start[i] + cs[i].items > 0x7fffffffLL)
      return set_error(PCF_EINVAL, "too many work items in one launch");
    start[i + 1] = start[i] + cs[i].items;
  }
  const int items = start[C];
  // Staged host -> device block: contracts | item_start | basket factors.
  const size_t o_con = 0;
  const size_t o_start = align256(o_con + sizeof(McContract) * C);
  const size_t o_fb = align256(o_start + sizeof(int) * (C + 1));
  const size_t h2d = align256(o_fb + sizeof(float) * fb.size());
  // Device-only: partials | tickets + queue | out.
  const size_t o_part = h2d;
  const size_t o_tick = align256(o_part + sizeof(double) * kMoments * (size_t)items);
  const size_t o_out = align256(o_tick + sizeof(unsigned) * (C + 1));
  const size_t total = align256(o_out + sizeof(double) * kMoments * C);
  const size_t host = std::max(h2d, sizeof(double) * kMoments * C);
  int st = ctx_ensure(c, total, host);
  if (st) return st;
  char* h = (char*)c->h_buf;
  char* d = (char*)c->d_buf;
  memcpy(h + o_con, cs.data(), sizeof(McContract) * C);
  memcpy(h + o_start, start.data(), sizeof(int) * (C + 1));
  if (!fb.empty()) memcpy(h + o_fb, fb.data(), sizeof(float) * fb.size());
  st = cuda_status(cudaMemcpyAsync(d, h, h2d, cudaMemcpyHostToDevice, c->stream), "H2D params");
  if (st) return st;
  st = cuda_status(cudaMemsetAsync(d + o_tick, 0, sizeof(unsigned) * (C + 1), c->stream),
                   "memset tickets");
  if (st) return st;
  McLaunch L;
  L.contracts = (const McContract*)(d + o_con);
  L.item_start = (const int*)(d + o_start);
  L.basket_data = (const float*)(d + o_fb);
  L.ncontracts = C;
  L.total_items = items;
  L.partial = (double*)(d + o_part);
  L.tickets = (unsigned*)(d + o_tick);
  L.queue = L.tickets + C;
  L.out = (double*)(d + o_out);
  L.persistent = persistent ? 1 : 0;
  L.cv = cv ? 1 : 0;
  int grid = items;
  if (persistent)
    grid = std::min(items, c->sm_count * mc_max_active_blocks(m, max_d, block, tensor));
  st = cuda_status(launch_mc(m, L, grid, max_d, block, tensor, c->stream), "mc kernel launch");
  if (st) return st;
  c->launches += 1;
  st = cuda_status(cudaMemcpyAsync(h, L.out, sizeof(double) * kMoments * C,
                                   cudaMemcpyDeviceToHost, c->stream),
                   "D2H sums");
  if (st) return st;
  st = cuda_status(cudaStreamSynchronize(c->stream), "mc kernel");
  if (st) return st;
  sums.assign((double*)h, (double*)h + (size_t)kMoments * C);
  return PCF_OK;
}

void fill_result(const double* s, long long n, double mu_g, double disc, bool use_cv,
                 pcf_mc_result* out) {
  const Estimate e = estimate(s, (double)n, mu_g, disc, use_cv);
  out->price = e.price;
  out->std_error = e.se;
  out->price_plain = e.price_plain;
  out->std_error_plain = e.se_plain;
  out->price_cv = e.price_cv;
  out->std_error_cv = e.se_cv;
  out->cv_beta = e.beta;
  out->cv_mean = mu_g;
  out->discount = disc;
  for (int k = 0; k < kMoments; ++k) out->sums[k] = s[k];
  out->n_paths = n;
}

static bool finite_all(std::initializer_list<double> v) {
  for (double x : v)
    if (!std::isfinite(x)) return false;
  return true;
}

int check_common(double S0, double E, double r, double sigma, double T, long long N, int pf) {
  if (pf != 1 && pf != -1)
    return set_error(PCF_EINVAL, "Unknown payoff function: payoff_fun must be +1 (call) or -1 (put)");
  if (!finite_all({S0, E, r, sigma, T})) return set_error(PCF_EINVAL, "non-finite parameter");
  if (!(S0 > 0)) return set_error(PCF_EINVAL, "S0 must be > 0");
  if (!(E >= 0)) return set_error(PCF_EINVAL, "E must be >= 0");
  if (!(sigma >= 0)) return set_error(PCF_EINVAL, "sigma must be >= 0");
  if (!(T > 0)) return set_error(PCF_EINVAL, "T must be > 0");
  if (N < 1) return set_error(PCF_EINVAL, "N must be >= 1");
  return PCF_OK;
}

static void split_seed(unsigned long long seed, McContract& k) {
  k.seed_lo = (uint32_t)seed;
  k.seed_hi = (uint32_t)(seed >> 32);
}

McContract make_eur(double S0, double E, double r, double sigma, double T, long long N, int pf,
                    unsigned long long seed, uint32_t stream, const TuneTable& t) {
  McContract k;
  memset(&k, 0, sizeof k);
  const double log2e = 1.4426950408889634;
  k.S0 = (float)S0;
  k.K = (float)E;
  k.pf = (float)pf;
  k.a2 = (float)((r - 0.5 * sigma * sigma) * T * log2e);
  k.b2 = (float)(sigma * sqrt(T) * log2e);
  k.l2S0 = (float)(log(S0) * log2e);
  k.nK = (float)(-pf * E);
  k.N = N;
  k.units_per_item = t.eur_block * eur_quads_per_thread(N, t);
  k.items = (int)(((N + 3) / 4 + k.units_per_item - 1) / k.units_per_item);
  split_seed(seed, k);
  k.stream = stream;
  return k;
}

McContract make_asia(double S0, double E, double r, double sigma, double T, long long N, int M,
                     int pf, int mode, unsigned long long seed, uint32_t stream,
                     const TuneTable& t) {
  McContract k;
  memset(&k, 0, sizeof k);
  const double log2e = 1.4426950408889634;
  const double dt = T / M;
  k.S0 = (float)S0;
  k.K = (float)E;
  k.pf = (float)pf;
  k.a2 = (float)((r - 0.5 * sigma * sigma) * dt * log2e);
  k.b2 = (float)(sigma * sqrt(dt) * log2e);
  k.c1 = (float)(1 + r * dt / 2);
  k.c2 = (float)(sigma * sqrt(dt) / 2);
  k.w_last = (float)(mode == 0 ? 0.5 / M : 1.0 / M);
  k.nK = (float)(-pf * E);
  k.M = M;
  k.mode = mode;
  k.N = N;
  k.units_per_item = t.asia_block * asia_paths_per_thread(M, t);
  k.items = (int)((N + k.units_per_item - 1) / k.units_per_item);
  split_seed(seed, k);
  k.stream = stream;
  return k;
}

double asia_cv_mean(double S0, double E, double r, double sigma, double T, int M, int pf,
                    int mode) {
  std::vector<double> w;
  asian_geo_weights(M, mode, w);
  return geo_weighted_payoff_mean(S0, E, r, sigma, T, M, w.data(), pf, nullptr);
}

// Builds the basket contract and appends its factor block to fb.
int make_basket(int d, const double* S0, const double* sig, const double* corr, double r,
                double T, double E, long long N, int pf, double ts, unsigned long long seed,
                uint32_t stream, std::vector<float>& fb, McContract& k, double& mu_g,
                const TuneTable& t) {
  if (d < 1 || d > 64) return set_error(PCF_EINVAL, "assets must be in [1, 64]");
  for (int a = 0; a < d; ++a) {
    if (!(S0[a] > 0) || !(sig[a] >= 0) || !std::isfinite(S0[a]) || !std::isfinite(sig[a]))
      return set_error(PCF_EINVAL, "asset %d: S0 must be > 0 and sigma >= 0", a);
    if (fabs(corr[a * d + a] - 1.0) > 1e-12)
      return set_error(PCF_EINVAL, "correlation diagonal must be 1");
  }
  std::vector<double> F;
  bool tri = true;
  if (!correlation_factor(d, corr, F, tri))
    return set_error(PCF_EINVAL, "correlation matrix is not symmetric positive semi-definite");
  memset(&k, 0, sizeof k);
  const double log2e = 1.4426950408889634;
  k.S0 = 1.f;
  k.K = (float)E;
  k.pf = (float)pf;
  k.M = d;
  k.mode = tri ? 0 : 1;
  k.nK = (float)(-pf * E);
  k.N = N;
  k.units_per_item = basket_units_per_item(d, t);
  k.items = (int)((N + k.units_per_item - 1) / k.units_per_item);
  split_seed(seed, k);
  k.stream = stream;
  k.basket_off = (int)fb.size();
  for (int a = 0; a < d; ++a)
    fb.push_back((float)((log(S0[a]) + (r - 0.5 * sig[a] * sig[a]) * T) * log2e));
  for (int a = 0; a < d; ++a) fb.push_back((float)(sig[a] * ts * log2e));
  for (int i = 0; i < d * d; ++i) fb.push_back((float)F[i]);
  mu_g = geo_basket_payoff_mean(d, S0, sig, corr, r, T, ts, E, pf);
  return PCF_OK;
}

}  // namespace pcf

using namespace pcf;

extern "C" {

const char* pcf_version(void) { return "parcompfin_gb300 0.1.0 (sm_103a)"; }

const char* pcf_strerror(int s) {
  switch (s) {
    case PCF_OK: return "ok";
    case PCF_EINVAL: return "invalid argument";
    case PCF_ENOMEM: return "out of memory";
    case PCF_ESINGULAR: return "singular regression (determinant <= 0)";
    case PCF_ETIMEOUT: return "device wait timed out";
    case PCF_ECUDA: return "CUDA error";
    case PCF_ENODEV: return "no CUDA device";
  }
  return "unknown status";
}

const char* pcf_last_error(void) { return g_err; }

int pcf_ctx_create(int device, pcf_ctx** out) {
  return pcf::abi_guard([&]() -> int {
    if (!out) return set_error(PCF_EINVAL, "out is NULL");
    *out = nullptr;
    int n = 0;
    int st = cuda_status(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (st) return st;
    if (device < 0 || device >= n)
      return set_error(n == 0 ? PCF_ENODEV : PCF_EINVAL, "device %d not present (%d devices)",
                       device, n);
    st = cuda_status(cudaSetDevice(device), "cudaSetDevice");
    if (st) return st;
    pcf_ctx* c = new pcf_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    st = cuda_status(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
    if (st) {
      delete c;
      return st;
    }
    *out = c;
    return PCF_OK;
  });
}

int pcf_ctx_destroy(pcf_ctx* c) {
  return pcf::abi_guard([&]() -> int {
    if (!c) return PCF_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    serve_release(c);
    ctx_release_extras(c);
    if (c->d_buf) cudaFree(c->d_buf);
    if (c->h_buf) cudaFreeHost(c->h_buf);
    cudaStreamDestroy(c->stream);
    if (c == g_default_ctx) g_default_ctx = nullptr;
    delete c;
    return PCF_OK;
  });
}

void* pcf_ctx_stream(pcf_ctx* c) {
  int st;
  c = resolve_ctx(c, &st);
  return c ? (void*)c->stream : nullptr;
}

long long pcf_ctx_launch_count(pcf_ctx* c) {
  int st;
  c = resolve_ctx(c, &st);
  return c ? c->launches : -1;
}

int pcf_ctx_release(pcf_ctx* c) {
  return pcf::abi_guard([&]() -> int {
    int st;
    c = resolve_ctx(c, &st);
    if (!c) return st;
    cudaSetDevice(c->device);
    st = cuda_status(cudaStreamSynchronize(c->stream), "context stream");
    serve_release(c);
    ctx_release_extras(c);
    if (c->d_buf) cudaFree(c->d_buf);
    if (c->h_buf) cudaFreeHost(c->h_buf);
    c->d_buf = nullptr;
    c->h_buf = nullptr;
    c->d_cap = c->h_cap = 0;
    return st;
  });
}

int pcf_ctx_set_memory_limit(pcf_ctx* c, unsigned long long bytes) {
  return pcf::abi_guard([&]() -> int {
    int st;
    c = resolve_ctx(c, &st);
    if (!c) return st;
    c->budget_bytes = (size_t)bytes;
    return PCF_OK;
  });
}

int pcf_ctx_set_test_barrier(pcf_ctx* ctx, unsigned extra_arrivals, unsigned poll_limit) {
  return pcf::abi_guard([&]() -> int {
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    if (extra_arrivals && poll_limit < 1)
      return set_error(PCF_EINVAL, "poll_limit must be >= 1 with extra arrivals");
    c->test_barrier_extra = extra_arrivals;
    c->test_poll_limit = extra_arrivals ? poll_limit : 0;
    return PCF_OK;
  });
}

int pcf_mc_eur(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T, long long N,
               int payoff_fun, unsigned long long seed, int use_cv, pcf_mc_result* out) {
  return pcf::abi_guard([&]() -> int {
    if (!out) return set_error(PCF_EINVAL, "out is NULL");
    int st = check_common(S0, E, r, sigma, T, N, payoff_fun);
    if (st) return st;
    if (N > (1LL << 46)) return set_error(PCF_EINVAL, "N must be <= 2^46");
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    const TuneTable tt = tune_table(c->device);
    std::vector<McContract> cs{make_eur(S0, E, r, sigma, T, N, payoff_fun, seed, 0, tt)};
    std::vector<double> sums;
    st = run_mc(c, MC_EUR, cs, {}, 0, tt.eur_block, false, false, use_cv != 0, sums);
    if (st) return st;
    fill_result(sums.data(), N, S0 * exp(r * T), exp(-r * T), use_cv != 0, out);
    return PCF_OK;
  });
}

int pcf_mc_asia(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T, long long N,
                int M, int payoff_fun, int mode, unsigned long long seed, int use_cv,
                pcf_mc_result* out) {
  return pcf::abi_guard([&]() -> int {
    if (!out) return set_error(PCF_EINVAL, "out is NULL");
    int st = check_common(S0, E, r, sigma, T, N, payoff_fun);
    if (st) return st;
    if (M < 1 || M > (1 << 20)) return set_error(PCF_EINVAL, "M must be in [1, 2^20]");
    if (mode != 0 && mode != 1) return set_error(PCF_EINVAL, "mode must be 0 or 1");
    if (N > (1LL << 38)) return set_error(PCF_EINVAL, "N must be <= 2^38");
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    const TuneTable tt = tune_table(c->device);
    std::vector<McContract> cs{make_asia(S0, E, r, sigma, T, N, M, payoff_fun, mode, seed, 0, tt)};
    std::vector<double> sums;
    st = run_mc(c, MC_ASIA, cs, {}, 0, tt.asia_block, false, false, use_cv != 0, sums);
    if (st) return st;
    fill_result(sums.data(), N, asia_cv_mean(S0, E, r, sigma, T, M, payoff_fun, mode),
                exp(-r * T), use_cv != 0, out);
    return PCF_OK;
  });
}

int pcf_mc_basket(pcf_ctx* ctx, int d, const double* S0, const double* sigma, const double* corr,
                  double r, double T, double E, long long N, int payoff_fun, int scale_by_sqrt_T,
                  unsigned long long seed, int use_cv, pcf_mc_result* out) {
  return pcf::abi_guard([&]() -> int {
    if (!out || !S0 || !sigma || !corr) return set_error(PCF_EINVAL, "NULL pointer argument");
    int st = check_common(1.0, E, r, 0.0, T, N, payoff_fun);
    if (st) return st;
    if (N > (1LL << 38)) return set_error(PCF_EINVAL, "N must be <= 2^38");
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    std::vector<float> fb;
    McContract k;
    double mu_g = 0;
    const TuneTable tt = tune_table(c->device);
    st = make_basket(d, S0, sigma, corr, r, T, E, N, payoff_fun, scale_by_sqrt_T ? sqrt(T) : 1.0,
                     seed, 0, fb, k, mu_g, tt);
    if (st) return st;
    std::vector<McContract> cs{k};
    std::vector<double> sums;
    st = run_mc(c, MC_BASKET, cs, fb, d, mc_block(PCF_METHOD_BASKET, d, tt), basket_tensor(d, tt),
                false, use_cv != 0, sums);
    if (st) return st;
    fill_result(sums.data(), N, mu_g, exp(-r * T), use_cv != 0, out);
    return PCF_OK;
  });
}

int pcf_mc_eur_multi(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T,
                     long long N, int payoff_fun, int assets, double rho,
                     unsigned long long seed, int use_cv, pcf_mc_result* out) {
  return pcf::abi_guard([&]() -> int {
    if (assets < 1 || assets > 64) return set_error(PCF_EINVAL, "assets must be in [1, 64]");
    if (!std::isfinite(rho) || rho < -1 || rho > 1)
      return set_error(PCF_EINVAL, "rho must be in [-1, 1]");
    // include/mvn.h:55-60: covariance with 1 on the diagonal and rho elsewhere.
    std::vector<double> s0((size_t)assets, S0), sg((size_t)assets, sigma),
        cor((size_t)assets * assets, rho);
    for (int a = 0; a < assets; ++a) cor[(size_t)a * assets + a] = 1.0;
    return pcf_mc_basket(ctx, assets, s0.data(), sg.data(), cor.data(), r, T, E, N, payoff_fun, 0,
                         seed, use_cv, out);
  });
}

}  // extern "C"
