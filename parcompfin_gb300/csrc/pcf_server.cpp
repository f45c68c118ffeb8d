// Continuous-batching serving loop: pcf_serve_trace (a request trace replayed
// against the wall clock) and the live server pcf_server_* (requests
// submitted by caller threads while others run), in include/pcf.h.
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
// Between polls the loop admits every request that has arrived into the free
// slots, spread evenly over them (at most max_batch each), so work admitted
// while other slots run overlaps with them on the device, and one slot's
// host-side plan build overlaps another's kernels. While work is on the
// device the loop polls its slots' events without sleeping (it yields the
// core between polls): a timed sleep of even 10 us overslept by tens of
// microseconds and added them to every batch's latency. Latency is arrival
// -> result on the host, measured on the wall clock.
//
// The loop (ServeLoop) is shared by both front ends: the trace replay feeds
// it arrivals from the caller's thread; the live server runs it on a worker
// thread that takes submitted requests from a queue and publishes each
// finished result for pcf_server_poll / pcf_server_wait.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <exception>
#include <functional>
#include <mutex>
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

// The slots of a context, kept between calls.
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

void fill_defaults(pcf_server_config& cfg) {
  if (cfg.pilot_paths <= 0) cfg.pilot_paths = 1 << 14;
  if (cfg.max_paths <= 0) cfg.max_paths = 1LL << 26;
  if (cfg.max_amer_paths <= 0) cfg.max_amer_paths = 1LL << 21;
  if (cfg.max_batch <= 0) cfg.max_batch = 2048;
  if (cfg.slots <= 0) cfg.slots = 12;
  if (cfg.hbm_fraction <= 0 || cfg.hbm_fraction > 0.9) cfg.hbm_fraction = 0.5;
}

// The context's slots for cfg.slots slots, reserving them on first use.
int reserve_slots(pcf_ctx* c, const pcf_server_config& cfg, ServeCache** out) {
  ServeCache* sc = static_cast<ServeCache*>(c->serve);
  if (sc && (int)sc->slots.size() != cfg.slots) {
    serve_release(c);
    sc = nullptr;
  }
  if (!sc) {
    size_t free_b = 0, total_b = 0;
    int st = cuda_status(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
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
  *out = sc;
  return PCF_OK;
}

// The loop over the slots. Requests are admitted by id (0, 1, 2, ... in
// arrival order) with their parameters; `finish` receives each request's
// record once it is done (its price on the host, or its error).
class ServeLoop {
 public:
  ServeLoop(pcf_ctx* c, const pcf_server_config& cfg, ServeCache* sc, Clock::time_point t0,
            std::function<void(int, const pcf_served_result&)> finish)
      : c_(c), cfg_(cfg), slots_(sc->slots), t0_(t0), finish_(std::move(finish)) {}

  double now() const { return std::chrono::duration<double>(Clock::now() - t0_).count(); }

  void admit(int id, const pcf_mc_request& q, double arrival_s) {
    if ((size_t)id >= rq_.size()) {
      rq_.resize((size_t)id + 1);
      rec_.resize((size_t)id + 1);
    }
    rq_[id] = q;
    memset(&rec_[id], 0, sizeof rec_[id]);
    rec_[id].arrival_s = arrival_s;
    rec_[id].status = PCF_OK;
    pending_.push_back(id);
  }

  bool idle() const {
    if (!pending_.empty()) return false;
    for (const Slot& s : slots_)
      if (s.state != Slot::FREE) return false;
    return true;
  }

  // One pass: advance the slots whose work has landed, then admit pending
  // requests into free slots. Returns whether anything happened.
  bool pass() {
    bool progress = false;
    for (Slot& s : slots_) progress |= advance(s);
    progress |= admit_pending();
    return progress;
  }

  // Leaves every slot free (a failed batch may hold a plan).
  // Also run on unwinding, so an exception leaves no plan in a slot.
  ~ServeLoop() { release(); }

  void release() {
    for (Slot& s : slots_) {
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
  }

  int done = 0, batches = 0, failures = 0, first_error = PCF_OK;
  long long paths = 0;

 private:
  void complete(int id) {
    ++done;
    finish_(id, rec_[id]);
  }

  void fail_batch(Slot& s, int code) {
    for (int id : s.ids) {
      rec_[id].status = code;
      rec_[id].done_s = now();
      complete(id);
    }
    if (first_error == PCF_OK) first_error = code;
    ++failures;
    s.ids.clear();
    s.state = Slot::FREE;
  }

  ExtMem slot_mem(Slot& s) {
    ExtMem mem;
    mem.d = s.d;
    mem.d_cap = s.d_cap;
    mem.h = s.h;
    mem.h_cap = s.h_cap;
    return mem;
  }

  // Builds the next main chunk [chunk_lo, chunk_hi) into the slot and queues it.
  int launch_main_chunk(Slot& s) {
    ExtMem mem = slot_mem(s);
    size_t used = 1 << 20, k = s.chunk_lo;
    while (k < s.ids.size() && (k == s.chunk_lo || used + main_bytes(s.main_q[k]) <= s.d_cap)) {
      used += main_bytes(s.main_q[k]);
      ++k;
    }
    s.chunk_hi = k;
    int e = plan_build(c_, (int)(s.chunk_hi - s.chunk_lo), &s.main_q[s.chunk_lo], s.s, &mem,
                       &s.plan, &s.main_x0[s.chunk_lo]);
    if (!e) e = plan_launch(s.plan);
    if (!e) e = plan_fetch(s.plan);
    if (!e) e = cuda_status(cudaEventRecord(s.ev, s.s), "slot event record");
    return e;
  }

  bool advance(Slot& s) {
    if (s.state == Slot::FREE) return false;
    const cudaError_t qe = cudaEventQuery(s.ev);
    if (qe == cudaErrorNotReady) return false;
    if (qe != cudaSuccess) {
      const int code = cuda_status(qe, "batch on the device");
      if (s.plan) {
        pcf_plan_destroy(s.plan);
        s.plan = nullptr;
      }
      fail_batch(s, code);
      return true;
    }
    std::vector<pcf_mc_result> res(s.plan ? s.plan->n : 0);
    int e = s.plan ? plan_fill_results(s.plan, res.data()) : PCF_OK;
    if (e != PCF_OK && e != PCF_ESINGULAR && e != PCF_ETIMEOUT) {
      pcf_plan_destroy(s.plan);
      s.plan = nullptr;
      fail_batch(s, e);
      return true;
    }
    // (PCF_ESINGULAR / PCF_ETIMEOUT: the requests concerned carry NaN prices.)
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
        pcf_mc_request q = rq_[id];
        const pcf_mc_result& r = res[j];
        const double se = q.use_cv ? r.std_error_cv : r.std_error_plain;
        const double price = fabs(q.use_cv ? r.price_cv : r.price_plain);
        const long long n0 = s.pilot_n[j];
        long long N = n0;
        if (std::isfinite(se) && se > 0 && price > 0) {
          const double target = cfg_.target_rel_se * price;
          const double need = (se * se * (double)n0) / (target * target) * 1.05;
          N = (long long)std::min(std::max(need, (double)n0), 9.0e18);
        }
        paths += n0;
        rec_[id].paths = n0;
        long long x0 = 0;
        if (q.method == PCF_METHOD_AMER) {
          N = std::max(N, kAmerFloor);
          N = std::min(N, cfg_.max_amer_paths);
          N = round_up(N, 2);
        } else {
          N = std::min(N, cfg_.max_paths);
        }
        if (N <= n0 && std::isfinite(r.price)) {  // the pilot reaches the target
          rec_[id].result = r;
          rec_[id].done_s = tp;
          complete(id);
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
        return true;
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
          fill_result(sum, a.n_paths + b.n_paths, a.cv_mean, a.discount, s.main_q[j].use_cv != 0,
                      &rec_[id].result);
        } else {
          rec_[id].result = b;
        }
        rec_[id].done_s = td;
        rec_[id].paths += s.main_q[j].N;
        paths += s.main_q[j].N;
        complete(id);
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
    return true;
  }

  // Admits pending requests into free slots, an even share each (a burst of
  // 1000 requests runs as pipelined batches, one slot's host-side build
  // overlapping another's kernels: measured 6.99 ms as one batch, 4.29 ms
  // over four slots, 4.05 ms over eight, 3.92 ms over twelve).
  bool admit_pending() {
    bool progress = false;
    int free_n = 0;
    for (const Slot& s : slots_) free_n += s.state == Slot::FREE;
    for (Slot& s : slots_) {
      if (pending_.empty()) break;
      if (s.state != Slot::FREE) continue;
      progress = true;
      const size_t share = std::min<size_t>((size_t)cfg_.max_batch,
                                            (pending_.size() + free_n - 1) / (size_t)free_n);
      --free_n;
      s.ids.clear();
      s.pilot_n.clear();
      std::vector<pcf_mc_request> q;
      const double ta = now();
      // The batch also stops where its American path matrices would no
      // longer fit the slot (a pilot runs in one piece).
      size_t used = 1 << 20;
      while (!pending_.empty() && s.ids.size() < share) {
        const int id = pending_.front();
        pcf_mc_request r = rq_[id];
        if (cfg_.target_rel_se > 0) {
          // A multiple of 4: the main run of a European, Asian or basket
          // request starts at path n0. An American pilot runs at the
          // American floor: most American requests need no more, and their
          // pilot is then their result.
          r.N = r.method == PCF_METHOD_AMER
                    ? round_up(std::max(cfg_.pilot_paths, kAmerFloor), 2)
                    : round_up(cfg_.pilot_paths, 4);
        }
        const size_t need = cfg_.target_rel_se > 0 ? main_bytes(r) : 4096;
        if (!s.ids.empty() && used + need > s.d_cap) break;
        used += need;
        pending_.pop_front();
        s.ids.push_back(id);
        rec_[id].admit_s = ta;
        s.pilot_n.push_back(r.N);
        q.push_back(r);
      }
      ++batches;
      ExtMem mem = slot_mem(s);
      int e;
      if (cfg_.target_rel_se > 0) {
        e = plan_build(c_, (int)q.size(), q.data(), s.s, &mem, &s.plan);
        if (!e) e = plan_launch(s.plan);
        if (!e) e = plan_fetch(s.plan);
        if (!e) e = cuda_status(cudaEventRecord(s.ev, s.s), "slot event record");
        s.state = Slot::PILOT;
      } else {
        s.main_q = q;
        s.main_x0.assign(q.size(), 0);
        s.carry.assign(q.size(), pcf_mc_result{});
        for (size_t j = 0; j < q.size(); ++j) rec_[s.ids[j]].paths = 0;
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
    return progress;
  }

  pcf_ctx* c_;
  pcf_server_config cfg_;
  std::vector<Slot>& slots_;
  Clock::time_point t0_;
  std::function<void(int, const pcf_served_result&)> finish_;
  std::vector<pcf_mc_request> rq_;
  std::vector<pcf_served_result> rec_;
  std::deque<int> pending_;
};

// Latency statistics over finished records (status PCF_OK).
void fill_stats(const pcf_served_result* out, int n, double first_arrival, int batches,
                long long paths, size_t reserved, pcf_server_stats* stats) {
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
  stats->wall_s = last - first_arrival;
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
  stats->reserved_bytes = reserved;
}

}  // namespace

extern "C" int pcf_serve_trace(pcf_ctx* ctx, const pcf_server_config* cfg_in, int n,
                               const pcf_mc_request* reqs, const double* arrival,
                               pcf_served_result* out, pcf_server_stats* stats) {
  return pcf::abi_guard([&]() -> int {
    if (n < 0 || (n > 0 && (!reqs || !arrival || !out))) return set_error(PCF_EINVAL, "bad arguments");
    pcf_server_config cfg = cfg_in ? *cfg_in : pcf_server_config{};
    fill_defaults(cfg);
    for (int i = 1; i < n; ++i)
      if (arrival[i] < arrival[i - 1]) return set_error(PCF_EINVAL, "arrival times must not decrease");
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    ServeCache* sc = nullptr;
    st = reserve_slots(c, cfg, &sc);
    if (st) return st;
    for (int i = 0; i < n; ++i) {
      memset(&out[i], 0, sizeof out[i]);
      out[i].arrival_s = arrival[i];
      out[i].status = PCF_OK;
    }
    ServeLoop loop(c, cfg, sc, Clock::now(),
                   [out](int id, const pcf_served_result& r) { out[id] = r; });
    int next = 0;
    while (loop.done < n) {
      const double t = loop.now();
      while (next < n && arrival[next] <= t) {
        loop.admit(next, reqs[next], arrival[next]);
        ++next;
      }
      if (!loop.pass()) {
        if (next < n && loop.idle()) {
          // Nothing to do until the next arrival.
          if (arrival[next] - loop.now() > 200e-6)
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        } else {
          std::this_thread::yield();  // work on the device: poll again at once
        }
      }
    }
    loop.release();
    if (stats)
      fill_stats(out, n, n ? arrival[0] : 0.0, loop.batches, loop.paths,
                 sc->per_slot * sc->slots.size(), stats);
    return loop.failures ? loop.first_error : PCF_OK;
  });
}

// ---- the live server -------------------------------------------------------

struct pcf_server {
  pcf_ctx* c = nullptr;
  pcf_server_config cfg{};
  ServeCache* sc = nullptr;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable work_cv;  // the worker: new requests or stop
  std::condition_variable done_cv;  // waiters: a request finished
  std::condition_variable idle_cv;  // pcf_server_stop: no submit/poll/wait call in progress
  int callers = 0;                  // submit/poll/wait calls in progress
  std::vector<pcf_mc_request> incoming;  // submitted, not yet taken by the worker
  long long first_incoming = 0;          // ticket of incoming[0]
  std::deque<pcf_served_result> out;     // by ticket
  std::deque<char> finished;             // by ticket
  long long submitted = 0, completed = 0;
  int batches = 0, failures = 0, first_error = PCF_OK;
  long long paths = 0;
  bool stop = false;
  bool dead = false;  // the worker ended on an exception; submissions are refused
  std::thread worker;
};

namespace {

void serve_worker_loop(pcf_server* s) {
  cudaSetDevice(s->c->device);
  ServeLoop loop(s->c, s->cfg, s->sc, s->t0, [s](int id, const pcf_served_result& r) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->out[(size_t)id] = r;
    s->finished[(size_t)id] = 1;
    ++s->completed;
    s->done_cv.notify_all();
  });
  std::vector<pcf_mc_request> take;
  std::vector<double> arrived;
  for (;;) {
    long long first = 0;
    bool stopping;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      take.swap(s->incoming);
      first = s->first_incoming;
      s->first_incoming += (long long)take.size();
      arrived.resize(take.size());
      for (size_t k = 0; k < take.size(); ++k)
        arrived[k] = s->out[(size_t)(first + (long long)k)].arrival_s;
      stopping = s->stop;
    }
    for (size_t k = 0; k < take.size(); ++k)
      loop.admit((int)(first + (long long)k), take[k], arrived[k]);
    take.clear();
    const bool progress = loop.pass();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->batches = loop.batches;
      s->failures = loop.failures;
      s->first_error = loop.first_error;
      s->paths = loop.paths;
    }
    if (stopping && loop.idle()) {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->incoming.empty()) break;
    }
    if (!progress) {
      if (loop.idle()) {
        std::unique_lock<std::mutex> lk(s->mu);
        s->work_cv.wait_for(lk, std::chrono::milliseconds(5),
                            [s] { return !s->incoming.empty() || s->stop; });
      } else {
        std::this_thread::yield();  // work on the device: poll again at once
      }
    }
  }
  loop.release();
}

// The worker thread: a C++ exception in the loop (host memory exhausted)
// would end the process from a thread, so it ends the server instead: every
// request not yet finished gets the error as its status, so that no waiter
// blocks for ever, and later submissions are refused.
void serve_worker(pcf_server* s) {
  try {
    serve_worker_loop(s);
  } catch (...) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->dead = true;
    s->failures += 1;
    if (s->first_error == PCF_OK) s->first_error = PCF_ENOMEM;
    for (size_t i = 0; i < s->finished.size(); ++i)
      if (!s->finished[i]) {
        s->out[i].status = PCF_ENOMEM;
        s->finished[i] = 1;
        ++s->completed;
      }
    s->incoming.clear();
    s->first_incoming = s->submitted;
    s->done_cv.notify_all();
  }
}

}  // namespace

extern "C" int pcf_server_start(pcf_ctx* ctx, const pcf_server_config* cfg_in,
                                pcf_server** out) {
  return pcf::abi_guard([&]() -> int {
    if (!out) return set_error(PCF_EINVAL, "out is NULL");
    *out = nullptr;
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    pcf_server* s = new pcf_server();
    s->c = c;
    s->cfg = cfg_in ? *cfg_in : pcf_server_config{};
    fill_defaults(s->cfg);
    st = reserve_slots(c, s->cfg, &s->sc);
    if (st) {
      delete s;
      return st;
    }
    s->t0 = Clock::now();
    try {
      s->worker = std::thread(serve_worker, s);
    } catch (const std::exception& e) {  // no C++ exception crosses the ABI
      delete s;
      return set_error(PCF_EINVAL, "cannot start the server's worker thread: %s", e.what());
    }
    *out = s;
    return PCF_OK;
  });
}

namespace {

// Counts a submit/poll/wait call in progress (under the server's mutex, held
// by the caller for the guard's lifetime or reacquired by a condition-variable
// wait before it ends), so that pcf_server_stop frees the server only after
// every such call has returned.
struct CallGuard {
  pcf_server* s;
  explicit CallGuard(pcf_server* srv) : s(srv) { ++s->callers; }
  ~CallGuard() {
    if (--s->callers == 0) s->idle_cv.notify_all();
  }
};

}  // namespace

extern "C" int pcf_server_submit(pcf_server* s, const pcf_mc_request* req, long long* ticket) {
  return pcf::abi_guard([&]() -> int {
    if (!s || !req || !ticket) return set_error(PCF_EINVAL, "bad arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    CallGuard guard(s);
    if (s->stop) return set_error(PCF_EINVAL, "the server is stopping");
    if (s->dead) return set_error(PCF_ENOMEM, "the server's worker ended on an error");
    if (s->submitted > 0x7ffffff0LL) return set_error(PCF_EINVAL, "too many requests for one server");
    pcf_served_result r;
    memset(&r, 0, sizeof r);
    r.arrival_s = std::chrono::duration<double>(Clock::now() - s->t0).count();
    r.status = PCF_OK;
    try {  // no C++ exception crosses the ABI; on failure nothing is queued
      s->out.push_back(r);
      s->finished.push_back(0);
      s->incoming.push_back(*req);
    } catch (const std::exception&) {
      s->out.resize((size_t)s->submitted);
      s->finished.resize((size_t)s->submitted);
      return set_error(PCF_ENOMEM, "cannot queue the request");
    }
    *ticket = s->submitted++;
    s->work_cv.notify_one();
    return PCF_OK;
  });
}

extern "C" int pcf_server_poll(pcf_server* s, long long ticket, pcf_served_result* out) {
  return pcf::abi_guard([&]() -> int {
    if (!s || !out) return set_error(PCF_EINVAL, "bad arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    CallGuard guard(s);
    if (ticket < 0 || ticket >= s->submitted) return set_error(PCF_EINVAL, "unknown ticket");
    if (!s->finished[(size_t)ticket]) return PCF_PENDING;
    *out = s->out[(size_t)ticket];
    return PCF_OK;
  });
}

extern "C" int pcf_server_wait(pcf_server* s, long long ticket, double timeout_s,
                               pcf_served_result* out) {
  return pcf::abi_guard([&]() -> int {
    if (!s || !out) return set_error(PCF_EINVAL, "bad arguments");
    std::unique_lock<std::mutex> lk(s->mu);
    CallGuard guard(s);
    if (ticket < 0 || ticket >= s->submitted) return set_error(PCF_EINVAL, "unknown ticket");
    const auto ready = [&] { return s->finished[(size_t)ticket] != 0; };
    if (timeout_s < 0) {
      s->done_cv.wait(lk, ready);
    } else if (!s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
      return PCF_PENDING;
    }
    *out = s->out[(size_t)ticket];
    return PCF_OK;
  });
}

extern "C" int pcf_server_stop(pcf_server* s, pcf_server_stats* stats) {
  return pcf::abi_guard([&]() -> int {
    if (!s) return PCF_OK;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->work_cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    {
      // Every request is finished now, so waiters wake; the server is freed
      // only after the last call in progress has returned.
      std::unique_lock<std::mutex> lk(s->mu);
      s->done_cv.notify_all();
      s->idle_cv.wait(lk, [s] { return s->callers == 0; });
    }
    int st = s->failures ? s->first_error : PCF_OK;
    if (stats) {
      std::vector<pcf_served_result> v(s->out.begin(), s->out.end());
      double first = v.empty() ? 0.0 : v[0].arrival_s;
      fill_stats(v.data(), (int)v.size(), first, s->batches, s->paths,
                 s->sc->per_slot * s->sc->slots.size(), stats);
    }
    delete s;
    return st;
  });
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
