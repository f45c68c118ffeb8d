// Batched pricing plans (pcf_plan_*, pcf_price_batch in include/pcf.h).
//
// A plan groups requests by method and uploads, once, each group's contract
// table, the item prefix table and the basket factors. A launch is then one
// memset plus one persistent kernel per Monte Carlo method group, and the
// American contracts' launches. The memset clears the groups' completion
// tickets, the work-queue heads and the American flag words. No host traffic
// happens at launch, so a plan can be replayed or captured in a CUDA graph.
// Results are read back in one copy.
//
// plan_build() either owns its memory (the public API: cudaMalloc, synchronous
// upload) or builds inside caller-provided memory without allocating and only
// queues the upload (the serving loop, which reserves its memory up front).
#include "pcf_plan_internal.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "pcf_math.h"

using namespace pcf;

namespace {

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

int build_request(const pcf_mc_request& q, int idx, McContract& k, std::vector<float>& fb,
                  double& mu_g, double& disc, const TuneTable& t) {
  int st = check_common(q.method == PCF_METHOD_BASKET && q.basket_S0 ? 1.0 : q.S0, q.E, q.r,
                        q.sigma, q.T, q.N, q.payoff_fun);
  if (st) return set_error(st, "request %d: %s", idx, pcf_last_error());
  disc = exp(-q.r * q.T);
  switch (q.method) {
    case PCF_METHOD_EUR:
      if (q.N > (1LL << 46)) return set_error(PCF_EINVAL, "request %d: N too large", idx);
      k = make_eur(q.S0, q.E, q.r, q.sigma, q.T, q.N, q.payoff_fun, q.seed, q.stream, t);
      mu_g = q.S0 * exp(q.r * q.T);
      return PCF_OK;
    case PCF_METHOD_ASIA:
      if (q.M < 1 || q.M > (1 << 20) || (q.mode != 0 && q.mode != 1) || q.N > (1LL << 38))
        return set_error(PCF_EINVAL, "request %d: bad Asian M/mode/N", idx);
      k = make_asia(q.S0, q.E, q.r, q.sigma, q.T, q.N, q.M, q.payoff_fun, q.mode, q.seed,
                    q.stream, t);
      mu_g = asia_cv_mean(q.S0, q.E, q.r, q.sigma, q.T, q.M, q.payoff_fun, q.mode);
      return PCF_OK;
    case PCF_METHOD_BASKET: {
      const int d = q.assets;
      if (d < 1 || d > 64 || q.N > (1LL << 38))
        return set_error(PCF_EINVAL, "request %d: basket size must be in [1, 64]", idx);
      std::vector<double> s0((size_t)d), sg((size_t)d), cor((size_t)d * d);
      for (int a = 0; a < d; ++a) {
        s0[a] = q.basket_S0 ? q.basket_S0[a] : q.S0;
        sg[a] = q.basket_sigma ? q.basket_sigma[a] : q.sigma;
      }
      if (q.corr) {
        memcpy(cor.data(), q.corr, sizeof(double) * d * d);
      } else {
        if (!(q.rho >= -1 && q.rho <= 1))
          return set_error(PCF_EINVAL, "request %d: rho must be in [-1, 1]", idx);
        for (int i = 0; i < d * d; ++i) cor[i] = q.rho;
        for (int a = 0; a < d; ++a) cor[(size_t)a * d + a] = 1.0;
      }
      st = make_basket(d, s0.data(), sg.data(), cor.data(), q.r, q.T, q.E, q.N, q.payoff_fun,
                       q.scale_by_sqrt_T ? sqrt(q.T) : 1.0, q.seed, q.stream, fb, k, mu_g, t);
      if (st) return set_error(st, "request %d: %s", idx, pcf_last_error());
      return PCF_OK;
    }
    default:
      return set_error(PCF_EINVAL, "request %d: method %d not supported in a batch", idx,
                       q.method);
  }
}

// Basket launches are split by width class so narrow baskets do not run in
// the register-heavy instantiation of wide ones; 17 to 32 assets go to the
// tensor-core group or, below the tuning table's threshold, to a CUDA-core
// group of their own.
int basket_group(int d, const TuneTable& t) {
  if (d > 16 && d <= 32 && !basket_tensor(d, t)) return 5;
  return basket_class_of(d);
}

}  // namespace

namespace pcf {

int plan_build(pcf_ctx* c, int n, const pcf_mc_request* reqs, cudaStream_t s, ExtMem* mem,
               pcf_plan** out, const long long* path0) {
  *out = nullptr;
  pcf_plan* p = new pcf_plan();
  p->ctx = c;
  p->stream = s;
  p->n = n;
  p->npaths.resize(n);
  p->mu_g.resize(n);
  p->disc.resize(n);
  p->use_cv.resize(n);
  p->out_slot.resize(n);
  // Groups: European, Asian, then one per basket width class. Work shapes
  // come from the device's tuning table.
  const TuneTable tt = tune_table(c->device);
  const int kGroups = 8;
  std::vector<Group> g(kGroups);
  g[0].method = MC_EUR;
  g[1].method = MC_ASIA;
  for (int k = 2; k < kGroups; ++k) g[k].method = MC_BASKET;
  int st;
  for (int i = 0; i < n; ++i) {
    const int m = reqs[i].method;
    if (m == PCF_METHOD_AMER) {
      const pcf_mc_request& q = reqs[i];
      st = check_lsm_request(q.S0, q.E, q.r, q.sigma, q.T, q.N, q.M, q.payoff_fun);
      if (st) {
        delete p;
        return set_error(st, "request %d: %s", i, pcf_last_error());
      }
      p->amer.push_back(i);
      p->amer_q.push_back(q);
      p->npaths[i] = q.N;
      p->use_cv[i] = q.use_cv != 0;
      continue;
    }
    if (m < 0 || m > 2) {
      delete p;
      return set_error(PCF_EINVAL, "request %d: method %d not supported in a batch", i, m);
    }
    const int gi = m == PCF_METHOD_BASKET ? 2 + basket_group(reqs[i].assets, tt) : m;
    McContract k;
    st = build_request(reqs[i], i, k, g[gi].fb, p->mu_g[i], p->disc[i], tt);
    if (st) {
      delete p;
      return st;
    }
    if (path0 && path0[i]) {
      if (path0[i] < 0 || path0[i] % 4 != 0) {
        delete p;
        return set_error(PCF_EINVAL, "request %d: path offset must be a multiple of 4", i);
      }
      k.x0 = m == PCF_METHOD_EUR ? path0[i] / 4 : path0[i];
    }
    if (m == PCF_METHOD_BASKET) {
      g[gi].max_d = std::max(g[gi].max_d, reqs[i].assets);
      g[gi].tensor = basket_tensor(reqs[i].assets, tt);
    }
    g[gi].block = mc_block(m, m == PCF_METHOD_BASKET ? reqs[i].assets : 0, tt);
    p->npaths[i] = reqs[i].N;
    p->use_cv[i] = reqs[i].use_cv != 0;
    g[gi].cs.push_back(k);
    g[gi].req.push_back(i);
  }
  // Longest items first: the queue then ends on short items (load balance).
  for (Group& gr : g) {
    std::vector<int> ord(gr.cs.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int a, int b) { return gr.cs[a].M > gr.cs[b].M; });
    std::vector<McContract> cs2;
    std::vector<int> req2;
    for (int o : ord) {
      cs2.push_back(gr.cs[o]);
      req2.push_back(gr.req[o]);
    }
    gr.cs.swap(cs2);
    gr.req.swap(req2);
    if (!gr.cs.empty()) p->groups.push_back(gr);
  }
  // Device layout: per group [contracts | item_start | factors] (the uploaded
  // prefix), then per group [partials], the tickets (+ queues, + American
  // flags) and the out table (n x kMoments).
  size_t off = 0;
  std::vector<size_t> o_con, o_start, o_fb, o_part, o_tick;
  size_t ticket_words = 0;
  for (Group& gr : p->groups) {
    const int C = (int)gr.cs.size();
    gr.start.assign((size_t)C + 1, 0);
    for (int i = 0; i < C; ++i) {
      if ((long long)gr.start[i] + gr.cs[i].items > 0x7fffffffLL) {
        delete p;
        return set_error(PCF_EINVAL, "batch has too many work items");
      }
      gr.start[i + 1] = gr.start[i] + gr.cs[i].items;
    }
    o_con.push_back(off);
    off = a256(off + sizeof(McContract) * C);
    o_start.push_back(off);
    off = a256(off + sizeof(int) * (C + 1));
    o_fb.push_back(off);
    off = a256(off + sizeof(float) * gr.fb.size());
  }
  const size_t upload = off;
  for (Group& gr : p->groups) {
    o_part.push_back(off);
    off = a256(off + sizeof(double) * kMoments * (size_t)gr.start[gr.cs.size()]);
    o_tick.push_back(ticket_words);
    ticket_words += gr.cs.size() + 1;
  }
  const size_t o_tickets = off;
  const size_t amer_flag_word = ticket_words;
  ticket_words += 2 * p->amer.size();
  p->tickets_bytes = sizeof(unsigned) * ticket_words;
  off = a256(off + p->tickets_bytes);
  const size_t o_out = off;
  off = a256(off + sizeof(double) * kMoments * (size_t)std::max(n, 1));
  const size_t host_out = sizeof(double) * kMoments * std::max(n, 1) +
                          sizeof(int) * 2 * (p->amer.size() + 1);
  char* d = nullptr;
  char* hup = nullptr;
  std::vector<char> hown;
  if (mem) {
    d = mem->dalloc(off);
    hup = mem->halloc(std::max(upload, (size_t)1));
    p->h_out = (double*)mem->halloc(host_out);
    if (!d || !hup || !p->h_out) {
      delete p;
      return set_error(PCF_ENOMEM, "batch needs %zu device bytes; the slot is full", off);
    }
  } else {
    if (c->budget_bytes && off > c->budget_bytes) {
      delete p;
      return set_error(PCF_ENOMEM, "plan needs %zu device bytes, over the context budget", off);
    }
    st = cuda_status(cudaMalloc(&p->d_mem, off), "cudaMalloc(plan)");
    if (!st) st = cuda_status(cudaMallocHost(&p->h_own, host_out), "cudaMallocHost(plan)");
    if (st) {
      pcf_plan_destroy(p);
      return st;
    }
    p->h_out = (double*)p->h_own;
    d = (char*)p->d_mem;
    hown.assign(std::max(upload, (size_t)1), 0);
    hup = hown.data();
  }
  p->d_tickets = (unsigned*)(d + o_tickets);
  p->d_out = (double*)(d + o_out);
  int row = 0;
  for (size_t gi = 0; gi < p->groups.size(); ++gi) {
    Group& gr = p->groups[gi];
    const int C = (int)gr.cs.size();
    memcpy(hup + o_con[gi], gr.cs.data(), sizeof(McContract) * C);
    memcpy(hup + o_start[gi], gr.start.data(), sizeof(int) * (C + 1));
    if (!gr.fb.empty()) memcpy(hup + o_fb[gi], gr.fb.data(), sizeof(float) * gr.fb.size());
    for (int i = 0; i < C; ++i) p->out_slot[gr.req[i]] = row + i;
    McLaunch& L = gr.L;
    L.contracts = (const McContract*)(d + o_con[gi]);
    L.item_start = (const int*)(d + o_start[gi]);
    L.basket_data = (const float*)(d + o_fb[gi]);
    L.ncontracts = C;
    L.total_items = gr.start[C];
    L.partial = (double*)(d + o_part[gi]);
    L.tickets = p->d_tickets + o_tick[gi];
    L.queue = L.tickets + C;
    L.out = p->d_out + (size_t)row * kMoments;
    L.persistent = 1;
    L.cv = 0;
    for (int i = 0; i < C; ++i) L.cv |= p->use_cv[gr.req[i]];
    gr.grid = std::min(L.total_items, c->sm_count * mc_max_active_blocks(gr.method, gr.max_d,
                                                                          gr.block, gr.tensor));
    row += C;
  }
  if (upload) {
    st = cuda_status(cudaMemcpyAsync(d, hup, upload, cudaMemcpyHostToDevice, s),
                     "H2D plan tables");
    if (!st && !mem) st = cuda_status(cudaStreamSynchronize(s), "plan upload");
    if (st) {
      pcf_plan_destroy(p);
      return st;
    }
  }
  if (!p->amer.empty()) {
    p->d_amer_flags = (int*)(p->d_tickets + amer_flag_word);
    p->h_amer_flags = (int*)(p->h_out + (size_t)kMoments * std::max(n, 1));
    std::vector<LsmRequest> lr;
    for (size_t a = 0; a < p->amer.size(); ++a) {
      const pcf_mc_request& q = p->amer_q[a];
      LsmRequest x;
      x.S0 = q.S0;
      x.E = q.E;
      x.r = q.r;
      x.sigma = q.sigma;
      x.T = q.T;
      x.N = q.N;
      x.M = q.M;
      x.pf = q.payoff_fun;
      x.ref_exercise = q.mode;
      x.seed = q.seed;
      x.stream = q.stream;
      x.d_out = p->d_out + (size_t)row * kMoments;
      x.d_flags = p->d_amer_flags + 2 * a;
      p->out_slot[p->amer[a]] = row++;
      lr.push_back(x);
    }
    st = lsm_batch_create(c, lr, s, mem, &p->lsm);
    if (st) {
      pcf_plan_destroy(p);
      return st;
    }
  }
  if (p->lsm && !p->groups.empty()) {
    // A failure here only leaves the plan without the fork (sequential launches).
    if (cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      if (p->side) cudaStreamDestroy(p->side);
      if (p->ev_fork) cudaEventDestroy(p->ev_fork);
      if (p->ev_join) cudaEventDestroy(p->ev_join);
      p->side = nullptr;
      p->ev_fork = p->ev_join = nullptr;
    }
  }
  *out = p;
  return PCF_OK;
}

// The plan's launch sequence: ticket reset, one persistent launch per Monte
// Carlo group, the LSM launches.
int plan_enqueue(pcf_plan* p) {
  pcf_ctx* c = p->ctx;
  if (p->tickets_bytes) {
    int st = cuda_status(cudaMemsetAsync(p->d_tickets, 0, p->tickets_bytes, p->stream),
                         "memset tickets");
    if (st) return st;
  }
  const bool fork = p->side && p->lsm && lsm_batch_cluster_kernels(p->lsm) > 0 &&
                    !p->groups.empty();
  if (fork) {
    int st = cuda_status(cudaEventRecord(p->ev_fork, p->stream), "plan fork");
    if (!st) st = cuda_status(cudaStreamWaitEvent(p->side, p->ev_fork, 0), "plan fork");
    if (!st) st = lsm_batch_launch_clusters(c, p->lsm, p->side);
    if (!st) st = cuda_status(cudaEventRecord(p->ev_join, p->side), "plan join");
    if (st) return st;
  }
  for (Group& gr : p->groups) {
    int st = cuda_status(launch_mc(gr.method, gr.L, gr.grid, gr.max_d, gr.block, gr.tensor,
                                   p->stream),
                         "batch kernel launch");
    if (st) return st;
    c->launches += 1;
  }
  if (fork) {
    const int st = cuda_status(cudaStreamWaitEvent(p->stream, p->ev_join, 0), "plan join");
    return st ? st : lsm_batch_launch_coop(c, p->lsm, p->stream);
  }
  if (p->lsm) return lsm_batch_launch(c, p->lsm, p->stream);
  return PCF_OK;
}

// Captures the launch sequence into a CUDA graph (every address in it is
// fixed for the plan's life). Returns false, leaving the stream out of
// capture, if the capture or the instantiation fails.
bool plan_capture(pcf_plan* p) {
  pcf_ctx* c = p->ctx;
  if (cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const long long before = c->launches;
  const int st = plan_enqueue(p);
  p->graph_kernels = c->launches - before;
  c->launches = before;
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(p->stream, &g);
  bool ok = st == PCF_OK && e == cudaSuccess && g != nullptr;
  if (ok) ok = cudaGraphInstantiate(&p->gexec, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    p->gexec = nullptr;
    cudaGetLastError();
  }
  return ok;
}

int plan_launch(pcf_plan* p) {
  pcf_ctx* c = p->ctx;
  if (!p->gexec && p->graph_mode && !p->graph_failed && p->launches_done >= 1)
    p->graph_failed = !plan_capture(p);
  int st;
  if (p->gexec) {
    st = cuda_status(cudaGraphLaunch(p->gexec, p->stream), "plan graph launch");
    if (!st) c->launches += p->graph_kernels;
  } else {
    st = plan_enqueue(p);
  }
  if (!st) p->launches_done += 1;
  return st;
}

int plan_fetch(pcf_plan* p) {
  if (p->n == 0) return PCF_OK;
  int st = cuda_status(cudaMemcpyAsync(p->h_out, p->d_out, sizeof(double) * kMoments * p->n,
                                       cudaMemcpyDeviceToHost, p->stream),
                       "D2H batch results");
  if (!st && !p->amer.empty())
    st = cuda_status(cudaMemcpyAsync(p->h_amer_flags, p->d_amer_flags,
                                     sizeof(int) * 2 * p->amer.size(), cudaMemcpyDeviceToHost,
                                     p->stream),
                     "D2H American flags");
  return st;
}

int plan_fill_results(pcf_plan* p, pcf_mc_result* results) {
  for (int i = 0; i < p->n; ++i)
    fill_result(p->h_out + (size_t)p->out_slot[i] * kMoments, p->npaths[i], p->mu_g[i],
                p->disc[i], p->use_cv[i] != 0, &results[i]);
  int status = PCF_OK;
  for (size_t a = 0; a < p->amer.size(); ++a) {
    const pcf_mc_request& q = p->amer_q[a];
    const int i = p->amer[a];
    fill_amer_result(p->h_out + (size_t)p->out_slot[i] * kMoments, q.N, q.S0, q.E, q.r, q.sigma,
                     q.T, q.payoff_fun, q.use_cv != 0, &results[i]);
    const int* fl = p->h_amer_flags + 2 * a;
    if (fl[0] || fl[1]) {
      // A request whose sweep failed gets NaN; the call reports the first failure.
      results[i].price = results[i].price_plain = results[i].price_cv = NAN;
      if (status == PCF_OK)
        status = fl[0] == 4 ? set_error(PCF_ECUDA, "request %d: LSM cluster launch ran without "
                                        "its cluster shape", i)
                 : set_error(fl[0] ? PCF_ETIMEOUT : PCF_ESINGULAR, "request %d: %s", i,
                             fl[0] ? "LSM device wait gave up" : "Detereminant is not > 0");
    }
  }
  return status;
}

}  // namespace pcf

extern "C" {

int pcf_plan_create(pcf_ctx* ctx, int n, const pcf_mc_request* reqs, pcf_plan** out) {
  return pcf::abi_guard([&]() -> int {
    if (!out || (n > 0 && !reqs) || n < 0) return set_error(PCF_EINVAL, "bad plan arguments");
    *out = nullptr;
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    return plan_build(c, n, reqs, c->stream, nullptr, out);
  });
}

int pcf_plan_launch(pcf_plan* p) {
  return pcf::abi_guard([&]() -> int {
    if (!p) return set_error(PCF_EINVAL, "plan is NULL");
    cudaSetDevice(p->ctx->device);
    return plan_launch(p);
  });
}

int pcf_plan_set_graph(pcf_plan* p, int mode) {
  return pcf::abi_guard([&]() -> int {
    if (!p || mode < 0 || mode > 1) return set_error(PCF_EINVAL, "bad arguments");
    cudaSetDevice(p->ctx->device);
    p->graph_mode = mode;
    if (!mode && p->gexec) {
      cudaStreamSynchronize(p->stream);
      cudaGraphExecDestroy(p->gexec);
      p->gexec = nullptr;
    }
    return PCF_OK;
  });
}

int pcf_plan_uses_graph(const pcf_plan* p) { return p && p->gexec ? 1 : 0; }

int pcf_plan_kernel_count(const pcf_plan* p) {
  return pcf::abi_guard([&]() -> int {
    return p ? (int)p->groups.size() + (p->lsm ? lsm_batch_kernels(p->lsm) : 0) : 0;
  });
}

int pcf_plan_results(pcf_plan* p, pcf_mc_result* results) {
  return pcf::abi_guard([&]() -> int {
    if (!p || (p->n && !results)) return set_error(PCF_EINVAL, "bad arguments");
    cudaSetDevice(p->ctx->device);
    int st = plan_fetch(p);
    if (!st) st = cuda_status(cudaStreamSynchronize(p->stream), "batch kernels");
    if (st) return st;
    return plan_fill_results(p, results);
  });
}

int pcf_plan_destroy(pcf_plan* p) {
  return pcf::abi_guard([&]() -> int {
    if (!p) return PCF_OK;
    cudaSetDevice(p->ctx->device);
    cudaStreamSynchronize(p->stream);
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->side) {
      cudaStreamSynchronize(p->side);
      cudaStreamDestroy(p->side);
    }
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->ev_join) cudaEventDestroy(p->ev_join);
    lsm_batch_destroy(p->lsm);
    if (p->d_mem) cudaFree(p->d_mem);
    if (p->h_own) cudaFreeHost(p->h_own);
    delete p;
    return PCF_OK;
  });
}

// The one-shot plan lives in the context's scratch arena (device and pinned
// host), which grows to the largest batch seen and is kept: after the first
// call of a given size a batch allocates nothing. A build that does not fit
// reports how far the arena must reach; the arena grows and the build runs
// again (at most a few times, only while the arena grows).
int pcf_price_batch(pcf_ctx* ctx, int n, const pcf_mc_request* reqs, pcf_mc_result* results) {
  return pcf::abi_guard([&]() -> int {
    if (n < 0 || (n > 0 && (!reqs || !results))) return set_error(PCF_EINVAL, "bad batch arguments");
    int st;
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    cudaSetDevice(c->device);
    size_t dneed = std::max(c->d_cap, (size_t)1 << 20), hneed = std::max(c->h_cap, (size_t)1 << 20);
    pcf_plan* p = nullptr;
    for (int attempt = 0;; ++attempt) {
      st = ctx_ensure(c, dneed, hneed);
      if (st) return st;
      ExtMem mem;
      mem.d = (char*)c->d_buf;
      mem.d_cap = c->d_cap;
      mem.h = (char*)c->h_buf;
      mem.h_cap = c->h_cap;
      st = plan_build(c, n, reqs, c->stream, &mem, &p);
      if (st != PCF_ENOMEM || (!mem.d_short && !mem.h_short) || attempt == 4) break;
      // Grow past the shortfall; later parts of the build may need more. A
      // failed build may have queued its table upload: let it land before the
      // arena is replaced.
      cudaStreamSynchronize(c->stream);
      dneed = std::max(dneed, mem.d_short + mem.d_short / 4);
      hneed = std::max(hneed, mem.h_short + mem.h_short / 4);
    }
    if (st) return st;
    st = plan_launch(p);
    if (!st) st = plan_fetch(p);
    if (!st) st = cuda_status(cudaStreamSynchronize(p->stream), "batch kernels");
    if (!st) st = plan_fill_results(p, results);
    pcf_plan_destroy(p);
    return st;
  });
}

}  // extern "C"
