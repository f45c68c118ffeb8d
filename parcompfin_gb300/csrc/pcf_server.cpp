// Continuous-batching serving loop (pcf_serve_trace in include/pcf.h).
//
// The loop owns S slots. Each slot has a CUDA stream, an event, and a device
// and a pinned host region reserved at start-up (a share of the free HBM), so
// no allocation happens while serving. The slots belong to the context and
// are kept between calls (a server reserves its memory once, not per trace);
// pcf_ctx_destroy frees them, and a call asking for another slot count
// replaces them. A slot runs one batch through:
//   PILOT  every request at a small path count n0, to estimate the variance
//          of its estimator;
//   MAIN   every request at the path count N that reaches its target
//          standard error, in chunks that fit the slot's memory (American
//          path matrices dominate it). A European, Asian or basket request
//          continues its pilot: the main run prices paths [n0, N) of the same
//          stream, and the pilot's sums and the main run's sums add up to the
//          sums over paths [0, N) (the same paths as one run of N; only the
//          order of the additions differs). A request whose pilot already
//          reaches the target is done after the pilot. An American pilot
//          runs at the American floor of 2^16 paths, so most American
//          requests are done after it; the others run again at N (a
//          regression needs every path in one sweep).
// Between polls the loop admits every request whose arrival time has passed
// into the free slots, spread evenly over them (at most max_batch each), so
// work admitted while other slots run overlaps with them on the device, and
// one slot's host-side plan build overlaps another's kernels. Latency is arrival -> result on the host,
// measured on the wall clock.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <thread>
#include <vector>

#include "pcf_plan_internal.h"

using namespace pcf;

namespace {

using Clock = std::chrono::steady_clock;

struct Slot {
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;
  char* d = nullptr;
  size_t d_cap = 0;
  char* h = nullptr;
  size_t h_cap = 0;
  enum { FREE, PILOT, MAIN } state = FREE;
  std::vector<int> ids;                 // requests of the batch
  std::vector<pcf_mc_request> main_q;   // main-run requests (same order as ids)
  std::vector<long long> main_x0;       // first path of each main request (0: a fresh run)
  std::vector<pcf_mc_result> carry;     // the pilot result a main request continues
  std::vector<long long> pilot_n;
  size_t chunk_lo = 0, chunk_hi = 0;    // [lo, hi) of ids in the running main chunk
  pcf_plan* plan = nullptr;
};

// The slots of a context, kept between pcf_serve_trace calls.
struct ServeCache {
  std::vector<Slot> slots;
  size_t per_slot = 0;
};

void free_slots(std::vector<Slot>& slots) {
  for (Slot& s : slots) {
    if (s.plan) {
      cudaStreamSynchronize(s.s);
      pcf_plan_destroy(s.plan);
      s.plan = nullptr;
    }
    if (s.d) cudaFree(s.d);
    if (s.h) cudaFreeHost(s.h);
    if (s.ev) cudaEventDestroy(s.ev);
    if (s.s) cudaStreamDestroy(s.s);
  }
  slots.clear();
}

long long round_up(long long x, long long m) { return (x + m - 1) / m * m; }

// Fewest paths an American request runs with a standard-error target: below
// it the regression's own noise dominates the pilot's variance estimate.
constexpr long long kAmerFloor = 1LL << 16;

// Device bytes a request's main run needs (American: its path matrix, and
// the per-path state a streaming sweep keeps beside it).
size_t main_bytes(const pcf_mc_request& q) {
  if (q.method != PCF_METHOD_AMER) return 4096;
  const long long Hp = ((q.N / 2) + 3) & ~3LL;
  return (size_t)4 * q.M * 2 * Hp + (size_t)12 * Hp + 4096;
}

}  // namespace

extern "C" int pcf_serve_trace(pcf_ctx* ctx, const pcf_server_config* cfg_in, int n,
                               const pcf_mc_request* reqs, const double* arrival,
                               pcf_served_result* out, pcf_server_stats* stats) {
  if (n < 0 || (n > 0 && (!reqs || !arrival || !out))) return set_error(PCF_EINVAL, "bad arguments");
  pcf_server_config cfg = cfg_in ? *cfg_in : pcf_server_config{};
  if (cfg.pilot_paths <= 0) cfg.pilot_paths = 1 << 14;
  if (cfg.max_paths <= 0) cfg.max_paths = 1LL << 26;
  if (cfg.max_amer_paths <= 0) cfg.max_amer_paths = 1LL << 21;
  if (cfg.max_batch <= 0) cfg.max_batch = 2048;
  if (cfg.slots <= 0) cfg.slots = 12;
  if (cfg.hbm_fraction <= 0 || cfg.hbm_fraction > 0.9) cfg.hbm_fraction = 0.5;
  for (int i = 1; i < n; ++i)
    if (arrival[i] < arrival[i - 1]) return set_error(PCF_EINVAL, "arrival times must not decrease");
  int st;
  pcf_ctx* c = resolve_ctx(ctx, &st);
  if (!c) return st;

  // Reserve the slots' memory once per context.
  ServeCache* sc = static_cast<ServeCache*>(c->serve);
  if (sc && (int)sc->slots.size() != cfg.slots) {
    serve_release(c);
    sc = nullptr;
  }
  if (!sc) {
    size_t free_b = 0, total_b = 0;
    st = cuda_status(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    if (st) return st;
    size_t budget = (size_t)(cfg.hbm_fraction * (double)free_b);
    if (c->budget_bytes) budget = std::min(budget, c->budget_bytes);
    // A slot runs its American path matrices in chunks that fit (a
    // 2^21-path, 50-date contract is 420 MB): 3 GB per slot is ample, and
    // reserving less keeps start-up short.
    const size_t per_slot = std::min(budget / cfg.slots, (size_t)3 << 30);
    const size_t host_per_slot = (size_t)16 << 20;
    sc = new ServeCache;
    sc->slots.resize(cfg.slots);
    sc->per_slot = per_slot;
    for (Slot& s : sc->slots) {
      st = cuda_status(cudaStreamCreateWithFlags(&s.s, cudaStreamNonBlocking), "slot stream");
      if (!st)
        st = cuda_status(cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming), "slot event");
      if (!st) st = cuda_status(cudaMalloc((void**)&s.d, per_slot), "slot device memory");
      if (!st) st = cuda_status(cudaMallocHost((void**)&s.h, host_per_slot), "slot pinned memory");
      if (st) {
        free_slots(sc->slots);
        delete sc;
        return st;
      }
      s.d_cap = per_slot;
      s.h_cap = host_per_slot;
    }
    c->serve = sc;
  }
  std::vector<Slot>& slots = sc->slots;
  const size_t per_slot = sc->per_slot;
  // Leaves every slot free for the next call (a failed batch may hold a plan).
  auto release = [&]() {
    for (Slot& s : slots) {
      if (s.plan) {
        cudaStreamSynchronize(s.s);
        pcf_plan_destroy(s.plan);
        s.plan = nullptr;
      }
      s.state = Slot::FREE;
      s.ids.clear();
      s.main_q.clear();
      s.main_x0.clear();
      s.carry.clear();
      s.pilot_n.clear();
    }
  };

  for (int i = 0; i < n; ++i) {
    memset(&out[i], 0, sizeof out[i]);
    out[i].arrival_s = arrival[i];
    out[i].status = PCF_OK;
  }
  const auto t0 = Clock::now();
  auto now = [&]() { return std::chrono::duration<double>(Clock::now() - t0).count(); };
  std::deque<int> pending;
  int next = 0, done = 0, batches = 0, failures = 0;
  long long paths = 0;
  int first_error = PCF_OK;

  auto fail_batch = [&](Slot& s, int code) {
    for (int id : s.ids) {
      out[id].status = code;
      out[id].done_s = now();
      ++done;
    }
    if (first_error == PCF_OK) first_error = code;
    ++failures;
    s.ids.clear();
    s.state = Slot::FREE;
  };

  // Builds the next main chunk [chunk_lo, chunk_hi) into the slot and queues it.
  auto launch_main_chunk = [&](Slot& s) -> int {
    ExtMem mem;
    mem.d = s.d;
    mem.d_cap = s.d_cap;
    mem.h = s.h;
    mem.h_cap = s.h_cap;
    size_t used = 1 << 20, k = s.chunk_lo;
    while (k < s.ids.size() && (k == s.chunk_lo || used + main_bytes(s.main_q[k]) <= s.d_cap)) {
      used += main_bytes(s.main_q[k]);
      ++k;
    }
    s.chunk_hi = k;
    int e = plan_build(c, (int)(s.chunk_hi - s.chunk_lo), &s.main_q[s.chunk_lo], s.s, &mem, &s.plan,
                       &s.main_x0[s.chunk_lo]);
    if (!e) e = plan_launch(s.plan);
    if (!e) e = plan_fetch(s.plan);
    if (!e) e = cuda_status(cudaEventRecord(s.ev, s.s), "slot event record");
    return e;
  };

  while (done < n) {
    bool progress = false;
    const double t = now();
    while (next < n && arrival[next] <= t) pending.push_back(next++);
    // Advance slots whose work has landed.
    for (Slot& s : slots) {
      if (s.state == Slot::FREE) continue;
      const cudaError_t qe = cudaEventQuery(s.ev);
      if (qe == cudaErrorNotReady) continue;
      progress = true;
      if (qe != cudaSuccess) {
        const int code = cuda_status(qe, "batch on the device");
        if (s.plan) {
          pcf_plan_destroy(s.plan);
          s.plan = nullptr;
        }
        fail_batch(s, code);
        continue;
      }
      std::vector<pcf_mc_result> res(s.plan ? s.plan->n : 0);
      int e = s.plan ? plan_fill_results(s.plan, res.data()) : PCF_OK;
      if (e == PCF_ESINGULAR || e == PCF_ETIMEOUT) {
        // per-request NaNs already set; keep serving
      } else if (e) {
        pcf_plan_destroy(s.plan);
        s.plan = nullptr;
        fail_batch(s, e);
        continue;
      }
      pcf_plan_destroy(s.plan);  // host side only: memory belongs to the slot
      s.plan = nullptr;
      if (s.state == Slot::PILOT) {
        // Path count that reaches the target relative SE, from the pilot.
        s.main_q.clear();
        s.main_x0.clear();
        s.carry.clear();
        std::vector<int> main_ids;
        const double tp = now();
        for (size_t j = 0; j < s.ids.size(); ++j) {
          const int id = s.ids[j];
          pcf_mc_request q = reqs[id];
          const pcf_mc_result& r = res[j];
          const double se = q.use_cv ? r.std_error_cv : r.std_error_plain;
          const double price = fabs(q.use_cv ? r.price_cv : r.price_plain);
          const long long n0 = s.pilot_n[j];
          long long N = n0;
          if (std::isfinite(se) && se > 0 && price > 0) {
            const double target = cfg.target_rel_se * price;
            const double need = (se * se * (double)n0) / (target * target) * 1.05;
            N = (long long)std::min(std::max(need, (double)n0), 9.0e18);
          }
          paths += n0;
          out[id].paths = n0;
          long long x0 = 0;
          if (q.method == PCF_METHOD_AMER) {
            N = std::max(N, kAmerFloor);
            N = std::min(N, cfg.max_amer_paths);
            N = round_up(N, 2);
          } else {
            N = std::min(N, cfg.max_paths);
          }
          if (N <= n0 && std::isfinite(r.price)) {  // the pilot reaches the target
            out[id].result = r;
            out[id].done_s = tp;
            ++done;
            continue;
          }
          if (q.method != PCF_METHOD_AMER) {
            x0 = n0;
            N -= n0;
          }
          q.N = N;
          main_ids.push_back(id);
          s.main_q.push_back(q);
          s.main_x0.push_back(x0);
          s.carry.push_back(r);
        }
        s.ids.swap(main_ids);
        if (s.ids.empty()) {
          s.state = Slot::FREE;
          continue;
        }
        s.chunk_lo = 0;
        s.state = Slot::MAIN;
        e = launch_main_chunk(s);
        if (e) fail_batch(s, e);
      } else {  // MAIN chunk finished
        const double td = now();
        for (size_t j = s.chunk_lo; j < s.chunk_hi; ++j) {
          const int id = s.ids[j];
          const pcf_mc_result& b = res[j - s.chunk_lo];
          if (s.main_x0[j] > 0) {  // pilot sums + main sums: paths [0, N)
            const pcf_mc_result& a = s.carry[j];
            double sum[kMoments];
            for (int k = 0; k < kMoments; ++k) sum[k] = a.sums[k] + b.sums[k];
            fill_result(sum, a.n_paths + b.n_paths, a.cv_mean, a.discount,
                        s.main_q[j].use_cv != 0, &out[id].result);
          } else {
            out[id].result = b;
          }
          out[id].done_s = td;
          out[id].paths += s.main_q[j].N;
          paths += s.main_q[j].N;
          ++done;
        }
        s.chunk_lo = s.chunk_hi;
        if (s.chunk_lo < s.ids.size()) {
          e = launch_main_chunk(s);
          if (e) {
            // requests before chunk_lo are done; fail the rest
            std::vector<int> rest(s.ids.begin() + s.chunk_lo, s.ids.end());
            s.ids = rest;
            fail_batch(s, e);
          }
        } else {
          s.ids.clear();
          s.state = Slot::FREE;
        }
      }
    }
    // Admit arrived requests into free slots, an even share each (a burst
    // of 1000 requests runs as pipelined batches, one slot's host-side build
    // overlapping another's kernels: measured 6.99 ms as one batch, 4.29 ms
    // over four slots, 4.05 ms over eight, 3.92 ms over twelve).
    int free_slots = 0;
    for (const Slot& s : slots) free_slots += s.state == Slot::FREE;
    for (Slot& s : slots) {
      if (pending.empty()) break;
      if (s.state != Slot::FREE) continue;
      progress = true;
      const size_t share = std::min<size_t>(
          (size_t)cfg.max_batch, (pending.size() + free_slots - 1) / (size_t)free_slots);
      --free_slots;
      s.ids.clear();
      s.pilot_n.clear();
      std::vector<pcf_mc_request> q;
      const double ta = now();
      while (!pending.empty() && s.ids.size() < share) {
        const int id = pending.front();
        pending.pop_front();
        s.ids.push_back(id);
        out[id].admit_s = ta;
        pcf_mc_request r = reqs[id];
        if (cfg.target_rel_se > 0) {
          // A multiple of 4: the main run of a European, Asian or basket
          // request starts at path n0. An American pilot runs at the
          // American floor: most American requests need no more, and their
          // pilot is then their result.
          r.N = r.method == PCF_METHOD_AMER ? round_up(std::max(cfg.pilot_paths, kAmerFloor), 2)
                                            : round_up(cfg.pilot_paths, 4);
        }
        s.pilot_n.push_back(r.N);
        q.push_back(r);
      }
      ++batches;
      ExtMem mem;
      mem.d = s.d;
      mem.d_cap = s.d_cap;
      mem.h = s.h;
      mem.h_cap = s.h_cap;
      int e;
      if (cfg.target_rel_se > 0) {
        e = plan_build(c, (int)q.size(), q.data(), s.s, &mem, &s.plan);
        if (!e) e = plan_launch(s.plan);
        if (!e) e = plan_fetch(s.plan);
        if (!e) e = cuda_status(cudaEventRecord(s.ev, s.s), "slot event record");
        s.state = Slot::PILOT;
      } else {
        s.main_q = q;
        s.main_x0.assign(q.size(), 0);
        s.carry.assign(q.size(), pcf_mc_result{});
        for (size_t j = 0; j < q.size(); ++j) out[s.ids[j]].paths = 0;
        s.chunk_lo = 0;
        s.state = Slot::MAIN;
        e = launch_main_chunk(s);
      }
      if (e) {
        if (s.plan) {
          pcf_plan_destroy(s.plan);
          s.plan = nullptr;
        }
        fail_batch(s, e);
      }
    }
    if (!progress) {
      if (next < n && pending.empty()) {
        // Nothing to do until the next arrival or completion.
        const double wait = arrival[next] - now();
        if (wait > 200e-6) std::this_thread::sleep_for(std::chrono::microseconds(50));
      } else {
        std::this_thread::sleep_for(std::chrono::microseconds(10));
      }
    }
  }
  release();

  if (stats) {
    memset(stats, 0, sizeof *stats);
    std::vector<double> lat;
    double last = 0;
    for (int i = 0; i < n; ++i) {
      if (out[i].status != PCF_OK) continue;
      lat.push_back(1e3 * (out[i].done_s - out[i].arrival_s));
      last = std::max(last, out[i].done_s);
    }
    std::sort(lat.begin(), lat.end());
    stats->completed = (int)lat.size();
    stats->batches = batches;
    const double first = n ? arrival[0] : 0.0;
    stats->wall_s = last - first;
    if (!lat.empty()) {
      auto pct = [&](double p) {
        const size_t k = (size_t)std::min<double>(lat.size() - 1, floor(p * (lat.size() - 1) + 0.5));
        return lat[k];
      };
      stats->p50_ms = pct(0.50);
      stats->p99_ms = pct(0.99);
      double sum = 0;
      for (double x : lat) sum += x;
      stats->mean_ms = sum / lat.size();
      stats->max_ms = lat.back();
    }
    stats->paths = paths;
    stats->contracts_per_s = stats->wall_s > 0 ? stats->completed / stats->wall_s : 0;
    stats->paths_per_s = stats->wall_s > 0 ? paths / stats->wall_s : 0;
    stats->reserved_bytes = per_slot * cfg.slots;
  }
  return failures ? first_error : PCF_OK;
}

namespace pcf {

void serve_release(pcf_ctx* c) {
  ServeCache* sc = static_cast<ServeCache*>(c->serve);
  if (!sc) return;
  free_slots(sc->slots);
  delete sc;
  c->serve = nullptr;
}

}  // namespace pcf
