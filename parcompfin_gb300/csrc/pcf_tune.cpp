// Work shapes of the kernels and the autotuner (pcf_autotune, pcf_tune_*).
//
// The reference fixes its only scheduling knob by hand: OpenMP chunks of
// 1000 paths (schedule(dynamic,1000), src/mc_eur_omp.cpp:24,
// src/mc_amer_omp.cpp:41). Here the work shapes of every launch -- the block
// size of the Monte Carlo launches, the paths each thread prices in a work
// item, the tensor-core basket kernel's tiles per item, the Longstaff-
// Schwartz cluster size and slice -- come from a per-device table. Its
// built-in values were measured by hand on GB300; pcf_autotune times
// candidate shapes per method and shape class on the device with CUDA
// events, through plans of synthetic contracts of that class, and keeps a
// candidate only when it beats the shape in force by more than 2 % (so noise
// does not move the table). PCF_TUNE_CACHE names a file that keeps the table
// between processes.
#include "pcf_tune.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "pcf_plan_internal.h"

namespace pcf {

namespace {

constexpr int kMaxDev = 64;
std::mutex g_tune_mu;
TuneTable g_tune[kMaxDev];
bool g_cache_tried[kMaxDev];

int clamp_int(long long v, int lo, int hi) { return (int)std::max<long long>(lo, std::min<long long>(hi, v)); }

int log2_floor(long long x) {
  int k = 0;
  while (x > 1) {
    x >>= 1;
    ++k;
  }
  return k;
}

std::string device_name(int dev) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
    cudaGetLastError();
    return "unknown";
  }
  char buf[320];
  snprintf(buf, sizeof buf, "%s sm_%d%d x%d", p.name, p.major, p.minor, p.multiProcessorCount);
  return buf;
}

// "key=v,v,v" lines.
bool parse_ints(const char* s, int* out, int n) {
  for (int i = 0; i < n; ++i) {
    char* end = nullptr;
    const long v = strtol(s, &end, 10);
    if (end == s) return false;
    out[i] = (int)v;
    s = end;
    if (i + 1 < n) {
      if (*s != ',') return false;
      ++s;
    }
  }
  return true;
}

bool valid(const TuneTable& t) {
  auto blk = [](int b) { return b == 128 || b == 256 || b == 512; };
  if (!blk(t.eur_block) || !blk(t.asia_block)) return false;
  for (int b : t.basket_block)
    if (!blk(b)) return false;
  if (t.tc_min_d < 17 || t.tc_min_d > 33) return false;
  for (int v : t.eur_items)
    if (v < 1 || v > 4096) return false;
  for (int v : t.asia_steps)
    if (v < 16 || v > 65536) return false;
  for (int v : t.basket_ppt)
    if (v < 1 || v > 64) return false;
  for (int v : t.tc_tiles)
    if (v < 1 || v > 64) return false;
  for (int v : t.lsm_shift)
    if (v < -1 || v > 1) return false;
  return t.eur_max_quads >= 1 && t.eur_max_quads <= 1024;
}

void load_cache(int dev, TuneTable& t) {
  const char* path = getenv("PCF_TUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  TuneTable x;
  bool dev_ok = false, ok = true;
  char line[512];
  const std::string me = device_name(dev);
  while (fgets(line, sizeof line, f)) {
    line[strcspn(line, "\r\n")] = 0;
    char* eq = strchr(line, '=');
    if (!eq) continue;
    *eq = 0;
    const char* k = line;
    const char* v = eq + 1;
    if (!strcmp(k, "device")) dev_ok = me == v;
    else if (!strcmp(k, "eur_block")) ok &= parse_ints(v, &x.eur_block, 1);
    else if (!strcmp(k, "eur_items")) ok &= parse_ints(v, x.eur_items, kTuneEurClasses);
    else if (!strcmp(k, "eur_max_quads")) ok &= parse_ints(v, &x.eur_max_quads, 1);
    else if (!strcmp(k, "asia_block")) ok &= parse_ints(v, &x.asia_block, 1);
    else if (!strcmp(k, "asia_steps")) ok &= parse_ints(v, x.asia_steps, kTuneAsiaClasses);
    else if (!strcmp(k, "basket_block")) ok &= parse_ints(v, x.basket_block, 4);
    else if (!strcmp(k, "basket_ppt")) ok &= parse_ints(v, x.basket_ppt, 4);
    else if (!strcmp(k, "tc_tiles")) ok &= parse_ints(v, x.tc_tiles, 2);
    else if (!strcmp(k, "tc_min_d")) ok &= parse_ints(v, &x.tc_min_d, 1);
    else if (!strcmp(k, "lsm_shift")) ok &= parse_ints(v, x.lsm_shift, kTuneLsmClasses);
  }
  fclose(f);
  if (dev_ok && ok && valid(x)) {
    x.tuned = true;
    t = x;
  }
}

// One knob: "key=v,v" (cache file) or "key": [v, v] / "key": v (JSON).
void ints(std::string& o, const char* k, const int* v, int n, bool json, bool list) {
  char b[64];
  o += json ? "\"" : "";
  o += k;
  o += json ? (list ? "\": [" : "\": ") : "=";
  for (int i = 0; i < n; ++i) {
    snprintf(b, sizeof b, "%s%d", i ? (json ? ", " : ",") : "", v[i]);
    o += b;
  }
  o += json ? (list ? "]" : "") : "\n";
}

std::string serialise(const TuneTable& t, bool json) {
  std::string o;
  auto one = [&](const char* k, int v) {
    ints(o, k, &v, 1, json, false);
    if (json) o += ", ";
  };
  auto many = [&](const char* k, const int* v, int n) {
    ints(o, k, v, n, json, true);
    if (json) o += ", ";
  };
  if (json) o += "{";
  one("eur_block", t.eur_block);
  many("eur_items", t.eur_items, kTuneEurClasses);
  one("eur_max_quads", t.eur_max_quads);
  one("asia_block", t.asia_block);
  many("asia_steps", t.asia_steps, kTuneAsiaClasses);
  many("basket_block", t.basket_block, 4);
  many("basket_ppt", t.basket_ppt, 4);
  many("tc_tiles", t.tc_tiles, 2);
  one("tc_min_d", t.tc_min_d);
  many("lsm_shift", t.lsm_shift, kTuneLsmClasses);
  if (json) o += std::string("\"tuned\": ") + (t.tuned ? "true" : "false") + "}";
  return o;
}

int save_cache(int dev, const TuneTable& t) {
  const char* path = getenv("PCF_TUNE_CACHE");
  if (!path || !*path) return PCF_OK;
  FILE* f = fopen(path, "w");
  if (!f) return set_error(PCF_EINVAL, "cannot write the tuning cache %s", path);
  fprintf(f, "device=%s\n%s", device_name(dev).c_str(), serialise(t, false).c_str());
  fclose(f);
  return PCF_OK;
}

}  // namespace

int eur_class(long long N) {
  const int l = log2_floor(std::max(1LL, N));
  return l < 18 ? 0 : l < 22 ? 1 : l < 26 ? 2 : 3;
}
int asia_class(int M) { return M <= 16 ? 0 : M <= 64 ? 1 : M <= 256 ? 2 : 3; }
int basket_class_of(int d) { return d <= 4 ? 0 : d <= 8 ? 1 : d <= 16 ? 2 : d <= 32 ? 3 : 4; }
int lsm_class(long long N) { return clamp_int(log2_floor(std::max(1LL, N)) - 14, 0, kTuneLsmClasses - 1); }

TuneTable tune_table(int device) {
  if (device < 0 || device >= kMaxDev) return TuneTable{};
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (!g_cache_tried[device]) {
    g_cache_tried[device] = true;
    load_cache(device, g_tune[device]);
  }
  return g_tune[device];
}

void tune_set(int device, const TuneTable& t) {
  if (device < 0 || device >= kMaxDev) return;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_cache_tried[device] = true;
  g_tune[device] = t;
}

void tune_reset(int device) { tune_set(device, TuneTable{}); }

std::string tune_json(const TuneTable& t) { return serialise(t, true); }

// European: about `eur_items` work items per contract, at most eur_max_quads
// quads per thread; four or more quads per thread are rounded down to a
// multiple of 4 (the kernel flushes its Kahan sums every four quads).
int eur_quads_per_thread(long long N, const TuneTable& t) {
  const long long nq = (N + 3) / 4;
  long long per = nq / ((long long)t.eur_block * t.eur_items[eur_class(N)]);
  per = std::max(1LL, std::min((long long)t.eur_max_quads, per));
  return (int)(per >= 4 ? per & ~3LL : per);
}

// Asian: at least asia_steps monitoring steps per thread per work item.
int asia_paths_per_thread(int M, const TuneTable& t) {
  const int steps = t.asia_steps[asia_class(M)];
  const int per = std::max(1, std::min(32, (steps + M - 1) / M));
  return per > 1 ? (per + 1) & ~1 : per;  // threads price their paths in pairs
}

bool basket_tensor(int d, const TuneTable& t) { return d > 32 || (d > 16 && d >= t.tc_min_d); }

int basket_units_per_item(int d, const TuneTable& t) {
  const int c = basket_class_of(d);
  if (!basket_tensor(d, t)) return t.basket_block[c] * t.basket_ppt[c];
  return 128 * t.tc_tiles[c - 3];  // the tensor-core kernel's 128-path tiles
}

int mc_block(int method, int d, const TuneTable& t) {
  if (method == PCF_METHOD_EUR) return t.eur_block;
  if (method == PCF_METHOD_ASIA) return t.asia_block;
  return basket_tensor(d, t) ? 128 : t.basket_block[basket_class_of(d)];
}

}  // namespace pcf

using namespace pcf;

namespace {

// Times a plan of `reqs` on the context's stream: one untimed launch, then
// the best of five, each bracketed by CUDA events (ms).
int time_plan(pcf_ctx* c, const std::vector<pcf_mc_request>& reqs, double* ms) {
  pcf_plan* p = nullptr;
  int st = pcf_plan_create(c, (int)reqs.size(), reqs.data(), &p);
  if (st) return st;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  st = cuda_status(cudaEventCreate(&e0), "tune event");
  if (!st) st = cuda_status(cudaEventCreate(&e1), "tune event");
  if (!st) st = pcf_plan_launch(p);
  double best = 1e30;
  for (int k = 0; k < 5 && !st; ++k) {
    st = cuda_status(cudaEventRecord(e0, c->stream), "tune event record");
    if (!st) st = pcf_plan_launch(p);
    if (!st) st = cuda_status(cudaEventRecord(e1, c->stream), "tune event record");
    if (!st) st = cuda_status(cudaEventSynchronize(e1), "tune run");
    float t = 0.f;
    if (!st) st = cuda_status(cudaEventElapsedTime(&t, e0, e1), "tune elapsed");
    if (!st) best = std::min(best, (double)t);
  }
  if (!st) {  // a plan whose kernels gave up (a timed-out wait) is no candidate
    std::vector<pcf_mc_result> res(reqs.size());
    st = pcf_plan_results(p, res.data());
    if (st == PCF_ESINGULAR) st = PCF_OK;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  pcf_plan_destroy(p);
  *ms = best;
  return st;
}

pcf_mc_request base_request(int method, double E, double sigma, long long N, unsigned stream) {
  pcf_mc_request q;
  memset(&q, 0, sizeof q);
  q.method = method;
  q.payoff_fun = method == PCF_METHOD_AMER ? -1 : 1;
  q.S0 = 100.0;
  q.E = E;
  q.r = 0.04;
  q.sigma = sigma;
  q.T = 1.0;
  q.N = N;
  q.use_cv = 1;
  q.scale_by_sqrt_T = 1;
  q.seed = 20261;
  q.stream = stream;
  return q;
}

struct Tuner {
  pcf_ctx* c;
  int dev;
  TuneTable t;
  std::string trials;
  int st = PCF_OK;
  std::vector<pcf_mc_request> user;  // the caller's batch: every knob is timed on it

  // Times the batch (the caller's, if one was given) under each candidate
  // edit of the table and keeps the fastest, provided it beats the table in
  // force by more than 2 %.
  // `applies`: whether the caller's batch holds work this knob shapes (a
  // knob that shapes none of it is left alone rather than tuned on noise).
  // The shape in force is timed first and again last, and a candidate must
  // beat the better of the two.
  template <typename Edit>
  void choose(const char* what, const std::vector<int>& cands, int current,
              const std::vector<pcf_mc_request>& synthetic, Edit edit,
              bool applies = true) {
    const std::vector<pcf_mc_request>& reqs = user.empty() ? synthetic : user;
    if (st || reqs.empty() || (!user.empty() && !applies)) return;
    double t_cur = 1e30, t_best = 1e30;
    int best = current;
    char buf[160];
    std::vector<int> order{current};
    for (int v : cands)
      if (v != current) order.push_back(v);
    order.push_back(current);
    for (int v : order) {
      TuneTable x = t;
      edit(x, v);
      tune_set(dev, x);
      double ms = 0;
      st = time_plan(c, reqs, &ms);
      if (st) break;
      snprintf(buf, sizeof buf, "%s{\"knob\": \"%s\", \"value\": %d, \"ms\": %.5f}",
               trials.empty() ? "" : ", ", what, v, ms);
      trials += buf;
      if (v == current) {
        t_cur = std::min(t_cur, ms);
      } else if (ms < t_best) {
        t_best = ms;
        best = v;
      }
    }
    if (!st && best != current && t_best < 0.98 * t_cur) edit(t, best);
    tune_set(dev, t);
  }

  // What the caller's batch holds, for `applies`: a request of `method` with
  // N in [nlo, nhi) and M (baskets: d) in [mlo, mhi].
  bool has(int method, long long nlo = 0, long long nhi = (1LL << 62), int mlo = 0,
           int mhi = 1 << 30) const {
    for (const pcf_mc_request& q : user) {
      const int m = method == PCF_METHOD_BASKET ? q.assets : q.M;
      if (q.method == method && q.N >= nlo && q.N < nhi && m >= mlo && m <= mhi) return true;
    }
    return false;
  }
};

}  // namespace

namespace {

int run_tuner(pcf_ctx* c, int flags, const pcf_mc_request* ureqs, int un, char* report,
              int report_len) {
  int st;
  if (flags == 0) flags = PCF_TUNE_MC | PCF_TUNE_LSM;
  Tuner tu;
  tu.c = c;
  tu.dev = c->device;
  tu.t = tune_table(c->device);
  if (ureqs) tu.user.assign(ureqs, ureqs + un);
  const TuneTable before = tu.t;
  unsigned sid = 0;
  auto batch = [&](int method, int count, long long N, int M, int d) {
    std::vector<pcf_mc_request> v;
    for (int i = 0; i < count; ++i) {
      pcf_mc_request q = base_request(method, 92.0 + 16.0 * i / std::max(1, count - 1),
                                      0.2 + 0.15 * (i % 3) / 2.0, N, sid++);
      q.M = M;
      q.assets = d;
      q.rho = 0.3;
      v.push_back(q);
    }
    return v;
  };
  const std::vector<int> blocks{128, 256, 512};
  if (flags & PCF_TUNE_MC) {
    // European: classes of N represented by 2^16, 2^20, 2^24, 2^27 paths.
    const long long eN[4] = {1LL << 16, 1LL << 20, 1LL << 24, 1LL << 27};
    const int eC[4] = {64, 32, 8, 2};
    std::vector<pcf_mc_request> all;
    for (int k = 0; k < 4; ++k) {
      auto b = batch(PCF_METHOD_EUR, eC[k], eN[k], 0, 0);
      all.insert(all.end(), b.begin(), b.end());
    }
    const long long eLo[4] = {0, 1LL << 18, 1LL << 22, 1LL << 26};
    const long long eHi[4] = {1LL << 18, 1LL << 22, 1LL << 26, 1LL << 62};
    tu.choose("eur_block", blocks, tu.t.eur_block, all, [](TuneTable& x, int v) { x.eur_block = v; },
              tu.has(PCF_METHOD_EUR));
    for (int k = 0; k < 4; ++k) {
      char w[32];
      snprintf(w, sizeof w, "eur_items[%d]", k);
      tu.choose(w, {8, 16, 32, 64, 128}, tu.t.eur_items[k], batch(PCF_METHOD_EUR, eC[k], eN[k], 0, 0),
                [k](TuneTable& x, int v) { x.eur_items[k] = v; },
                tu.has(PCF_METHOD_EUR, eLo[k], eHi[k]));
    }
    // Asian: classes of M represented by 12, 52, 252 and 1000 steps.
    const int aM[4] = {12, 52, 252, 1000};
    const int aC[4] = {32, 32, 32, 8};
    all.clear();
    for (int k = 0; k < 4; ++k) {
      auto b = batch(PCF_METHOD_ASIA, aC[k], 1LL << 17, aM[k], 0);
      all.insert(all.end(), b.begin(), b.end());
    }
    const int aLo[4] = {0, 17, 65, 257}, aHi[4] = {16, 64, 256, 1 << 30};
    tu.choose("asia_block", blocks, tu.t.asia_block, all,
              [](TuneTable& x, int v) { x.asia_block = v; }, tu.has(PCF_METHOD_ASIA));
    for (int k = 0; k < 4; ++k) {
      char w[32];
      snprintf(w, sizeof w, "asia_steps[%d]", k);
      tu.choose(w, {128, 256, 512, 1024, 2048}, tu.t.asia_steps[k],
                batch(PCF_METHOD_ASIA, aC[k], 1LL << 17, aM[k], 0),
                [k](TuneTable& x, int v) { x.asia_steps[k] = v; },
                tu.has(PCF_METHOD_ASIA, 0, 1LL << 62, aLo[k], aHi[k]));
    }
    // Baskets: 4, 8, 16 assets on the CUDA cores, 32 and 64 on the tensor cores.
    const int bD[5] = {4, 8, 16, 32, 64};
    const int bLo[5] = {1, 5, 9, 17, 33};
    for (int k = 0; k < 5; ++k) {
      const auto b = batch(PCF_METHOD_BASKET, k < 3 ? 8 : 4, 1LL << 20, 0, bD[k]);
      const bool here = tu.has(PCF_METHOD_BASKET, 0, 1LL << 62, bLo[k], bD[k]);
      char w[32];
      if (k < 3) {
        snprintf(w, sizeof w, "basket_block[%d]", k);
        tu.choose(w, blocks, tu.t.basket_block[k], b,
                  [k](TuneTable& x, int v) { x.basket_block[k] = v; }, here);
        snprintf(w, sizeof w, "basket_ppt[%d]", k);
        tu.choose(w, {2, 4, 8, 16, 32}, tu.t.basket_ppt[k], b,
                  [k](TuneTable& x, int v) { x.basket_ppt[k] = v; }, here);
      } else {
        snprintf(w, sizeof w, "tc_tiles[%d]", k - 3);
        tu.choose(w, {2, 4, 8, 16, 32}, tu.t.tc_tiles[k - 3], b,
                  [k](TuneTable& x, int v) { x.tc_tiles[k - 3] = v; }, here);
      }
    }
    // 17 to 32 assets: the CUDA-core kernel (its shape first) against the
    // tensor cores, basket by basket size; the tensor cores take every size
    // from the smallest one from which on they win at each size timed. On
    // the caller's batch, the threshold itself is the knob.
    const auto b24 = batch(PCF_METHOD_BASKET, 4, 1LL << 20, 0, 24);
    const bool mid = tu.has(PCF_METHOD_BASKET, 0, 1LL << 62, 17, 32);
    tu.choose("basket_ppt[3]", {2, 4, 8, 16}, tu.t.basket_ppt[3], b24,
              [](TuneTable& x, int v) { x.basket_ppt[3] = v; x.tc_min_d = 33; }, mid);
    tu.t.tc_min_d = before.tc_min_d;  // the edit above timed the CUDA-core route only
    tune_set(c->device, tu.t);
    if (!tu.user.empty()) {
      tu.choose("tc_min_d", {17, 20, 24, 28, 33}, tu.t.tc_min_d, {},
                [](TuneTable& x, int v) { x.tc_min_d = v; }, mid);
    } else {
      const int dset[5] = {17, 20, 24, 28, 32};
      bool tc_wins[5];
      for (int k = 0; k < 5 && !tu.st; ++k) {
        const auto b = batch(PCF_METHOD_BASKET, 4, 1LL << 21, 0, dset[k]);
        double ms[2] = {0, 0};
        for (int route = 0; route < 2 && !tu.st; ++route) {
          TuneTable x = tu.t;
          x.tc_min_d = route ? 17 : 33;
          tune_set(c->device, x);
          tu.st = time_plan(c, b, &ms[route]);
          char buf[160];
          snprintf(buf, sizeof buf,
                   ", {\"knob\": \"basket_route_d%d\", \"value\": %d, \"ms\": %.5f}", dset[k],
                   route, ms[route]);
          tu.trials += buf;
        }
        tc_wins[k] = ms[1] < ms[0];
      }
      if (!tu.st) {
        int from = 33;
        for (int k = 4; k >= 0 && tc_wins[k]; --k) from = dset[k];
        tu.t.tc_min_d = from;
      }
      tune_set(c->device, tu.t);
    }
  }
  if (flags & PCF_TUNE_LSM) {
    // American puts, 50 dates, N = 2^15 .. 2^21 (the served stream's range).
    for (int k = 1; k < kTuneLsmClasses; ++k) {
      const long long N = 1LL << (14 + k);
      const int count = N <= (1 << 16) ? 64 : N <= (1 << 18) ? 32 : N <= (1 << 20) ? 16 : 8;
      char w[32];
      snprintf(w, sizeof w, "lsm_shift[%d]", k);
      const long long lo = 1LL << (14 + k);
      const long long hi = k == kTuneLsmClasses - 1 ? (1LL << 62) : 1LL << (15 + k);
      tu.choose(w, {-1, 0, 1}, tu.t.lsm_shift[k], batch(PCF_METHOD_AMER, count, N, 50, 0),
                [k](TuneTable& x, int v) { x.lsm_shift[k] = v; },
                tu.has(PCF_METHOD_AMER, lo, hi));
    }
  }
  if (tu.st) {
    tune_set(c->device, before);
    return tu.st;
  }
  tu.t.tuned = true;
  tune_set(c->device, tu.t);
  st = PCF_OK;
  if (flags & PCF_TUNE_SAVE) st = save_cache(c->device, tu.t);
  if (report && report_len > 0) {
    const std::string r = "{\"device\": \"" + device_name(c->device) + "\", \"mode\": \"" +
                          (tu.user.empty() ? "classes" : "batch") + "\", \"table\": " +
                          tune_json(tu.t) + ", \"built_in\": " + tune_json(TuneTable{}) +
                          ", \"trials\": [" + tu.trials + "]}";
    snprintf(report, (size_t)report_len, "%s", r.c_str());
  }
  return st;
}

}  // namespace

extern "C" int pcf_autotune(pcf_ctx* ctx, int flags, char* report, int report_len) {
  return pcf::abi_guard([&]() -> int {
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    return run_tuner(c, flags, nullptr, 0, report, report_len);
  });
}

extern "C" int pcf_autotune_batch(pcf_ctx* ctx, int flags, int n, const pcf_mc_request* reqs,
                                  char* report, int report_len) {
  return pcf::abi_guard([&]() -> int {
    if (n <= 0 || !reqs) return set_error(PCF_EINVAL, "the tuning batch is empty");
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    return run_tuner(c, flags, reqs, n, report, report_len);
  });
}

extern "C" int pcf_tune_report(pcf_ctx* ctx, char* report, int report_len) {
  return pcf::abi_guard([&]() -> int {
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    if (!report || report_len <= 0) return set_error(PCF_EINVAL, "report buffer is empty");
    const std::string r = "{\"device\": \"" + device_name(c->device) + "\", \"table\": " +
                          tune_json(tune_table(c->device)) + "}";
    snprintf(report, (size_t)report_len, "%s", r.c_str());
    return PCF_OK;
  });
}

extern "C" int pcf_tune_reset(pcf_ctx* ctx) {
  return pcf::abi_guard([&]() -> int {
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    tune_reset(c->device);
    return PCF_OK;
  });
}
