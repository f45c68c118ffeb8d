// Binomial-lattice backward induction (the reference's binom_vanilla_eur and
// binom_vanilla_amer) on one GPU.
//
// Reference: binom() of src/binom_vanilla_eur.cpp:5-39 and
// src/binom_vanilla_amer.cpp:5-40, on the beta-lattice of
// src/binom_vanilla_eur.cpp:14-22. Level N holds payoff(S0 u^i d^{N-i}),
// i = 0..N; each level n < N replaces v[i] by (p v[i+1] + q v[i]) / R, and the
// American version by the larger of that and payoff(S0 u^i d^{n-i}). v[0] of
// level 0 is the price.
//
// The result is the reference's bit for bit: node prices are
// (S0 * u^i) * d^j with u^i and d^j from host tables made by the same libm
// pow the reference calls; the arithmetic is IEEE FP64 in the reference's
// order (explicit _rn operations, and the unit is compiled with -fmad=false);
// and every level is a pure function of the level above, so computing a
// level's nodes in parallel changes nothing.
//
// One cooperative launch, temporal blocking: a grid step advances K levels.
// The new level's nodes are split evenly over the blocks; a block loads its
// range of the current level plus the K nodes to its right (node i depends on
// i and i+1), advances K levels in shared memory, and writes its range of the
// new level into the other of two level arrays. One bounded grid barrier per
// step. The last levels (at most `tail + 1` nodes) are finished by block 0
// alone. Cost: (N+1)(N+2)/2 nodes, each a few FP64 operations and one
// division; the K(K-1)/2 halo nodes a block recomputes per step are a small
// fraction of its K x range.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "pcf_api_internal.h"
#include "pcf_device.cuh"

namespace pcf {

namespace {

constexpr int kLatBlock = 256;
constexpr int kLatSteps = 128;   // levels per grid step
constexpr int kLatTail = 2048;   // levels finished by block 0 alone
constexpr int kLatMaxN = 2000000;

struct LatticeParams {
  double S0, E, p, q, R;
  int N, pf, american;
  const double* up;  // pow(u, i), i = 0..N
  const double* dn;  // pow(d, j), j = 0..N
  double* A;         // two level arrays of N + 1 nodes
  double* B;
  unsigned* barrier;
  int* err;
  unsigned wait_limit;
  unsigned barrier_extra;  // test hook: arrivals the barrier expects beyond the grid
  double* out;
};

// include/common.h:56-60: std::max(payoff_fun * (St - E), 0.0).
__device__ __forceinline__ double lat_payoff(const LatticeParams& P, int n, int i) {
  const double S = __dmul_rn(__dmul_rn(P.S0, P.up[i]), P.dn[n - i]);
  const double a = __dmul_rn((double)P.pf, __dsub_rn(S, P.E));
  return a < 0.0 ? 0.0 : a;
}

// Node i of level n from nodes i, i+1 of level n+1
// (src/binom_vanilla_amer.cpp:33-35; the European version stops at jatk).
__device__ __forceinline__ double lat_node(const LatticeParams& P, double vi, double vi1, int n,
                                           int i) {
  const double jatk = __ddiv_rn(__dadd_rn(__dmul_rn(P.p, vi1), __dmul_rn(P.q, vi)), P.R);
  if (!P.american) return jatk;
  const double sij = lat_payoff(P, n, i);
  return jatk < sij ? sij : jatk;  // std::max(jatk, sij)
}

// Advances `cnt0` nodes of level `top` (starting at node `a`) by `k` levels
// in shared memory; on return cur holds the new level's first cnt0 - k nodes.
__device__ double* advance(const LatticeParams& P, double* cur, double* nxt, int cnt0, int top,
                           int k, int a) {
  for (int j = 1; j <= k; ++j) {
    const int n = top - j, cnt = cnt0 - j;
    for (int t = threadIdx.x; t < cnt; t += kLatBlock)
      nxt[t] = lat_node(P, cur[t], cur[t + 1], n, a + t);
    __syncthreads();
    double* x = cur;
    cur = nxt;
    nxt = x;
  }
  return cur;
}

__global__ void __launch_bounds__(kLatBlock) lattice_kernel(LatticeParams P, int seg_cap) {
  extern __shared__ double sm[];
  const int G = gridDim.x, b = blockIdx.x;
  // Level N (src/binom_vanilla_eur.cpp:27-28 writes max((S - E) pf, 0), the
  // same value as payoff()).
  for (int i = b * kLatBlock + threadIdx.x; i <= P.N; i += G * kLatBlock)
    P.A[i] = lat_payoff(P, P.N, i);
  if (!group_barrier(P.barrier, (unsigned)G + P.barrier_extra, P.err, P.wait_limit)) return;
  double* src = P.A;
  double* dst = P.B;
  int top = P.N;
  while (top > kLatTail) {
    const int k = min(kLatSteps, top - kLatTail);
    const int bot = top - k;  // the new level has bot + 1 nodes
    const int seg = (bot + 1 + G - 1) / G;
    const int a = b * seg, e = min(a + seg, bot + 1);
    if (a < e) {
      const int cnt0 = e - a + k;  // nodes [a, e + k) of level top; e + k <= top + 1
      double* cur = sm;
      double* nxt = sm + seg_cap + kLatSteps;
      for (int t = threadIdx.x; t < cnt0; t += kLatBlock) cur[t] = src[a + t];
      __syncthreads();
      cur = advance(P, cur, nxt, cnt0, top, k, a);
      for (int t = threadIdx.x; t < e - a; t += kLatBlock) dst[a + t] = cur[t];
    }
    if (!group_barrier(P.barrier, (unsigned)G + P.barrier_extra, P.err, P.wait_limit)) return;
    double* x = src;
    src = dst;
    dst = x;
    top = bot;
  }
  if (b != 0) return;
  double* cur = sm;
  double* nxt = sm + kLatTail + 1;
  for (int t = threadIdx.x; t <= top; t += kLatBlock) cur[t] = src[t];
  __syncthreads();
  cur = advance(P, cur, nxt, top + 1, top, top, 0);
  if (threadIdx.x == 0) *P.out = cur[0];
}

}  // namespace

}  // namespace pcf

using namespace pcf;

extern "C" int pcf_binom_vanilla(pcf_ctx* ctx, double S0, double E, double r, double sigma,
                                 double T, int N, int payoff_fun, int american, double* price) {
  return pcf::abi_guard([&]() -> int {
    if (!price) return set_error(PCF_EINVAL, "price is NULL");
    int st = check_common(S0, E, r, sigma, T, N, payoff_fun);
    if (st) return st;
    if (N > kLatMaxN) return set_error(PCF_EINVAL, "N must be <= %d", kLatMaxN);
    pcf_ctx* c = resolve_ctx(ctx, &st);
    if (!c) return st;
    double u, d, p, q, R;
    lattice(r, sigma, T, N, u, d, p, q, R);

    int G = N > kLatTail ? std::min(c->sm_count, (N + 1 + 511) / 512) : 1;
    G = std::max(G, 1);
    const int seg_cap = (N + 1 + G - 1) / G;
    const size_t smem = sizeof(double) * (size_t)std::max(2 * (seg_cap + kLatSteps),
                                                          2 * (kLatTail + 1));
    st = cuda_status(cudaFuncSetAttribute(lattice_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                     "lattice smem attribute");
    if (st) return st;
    int occ = 0;
    st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lattice_kernel, kLatBlock,
                                                                   smem),
                     "occupancy(lattice)");
    if (st) return st;
    if ((long long)occ * c->sm_count < G)
      return set_error(PCF_EINVAL, "lattice grid of %d blocks cannot be co-resident", G);

    // Scratch: up | dn | A | B | counters (barrier, err) | out.
    const size_t nodes = (size_t)N + 1;
    const size_t o_up = 0, o_dn = o_up + 8 * nodes, o_A = o_dn + 8 * nodes, o_B = o_A + 8 * nodes;
    const size_t o_cnt = (o_B + 8 * nodes + 255) & ~(size_t)255;
    const size_t o_out = o_cnt + 256;
    const size_t total = o_out + 256;
    st = ctx_ensure(c, total, 16 * nodes + 64);
    if (st) return st;
    char* dv = (char*)c->d_buf;
    double* h = (double*)c->h_buf;
    // The reference's pow(u, i) and pow(d, n - i) (src/binom_vanilla_amer.cpp:28,32).
    for (size_t i = 0; i < nodes; ++i) {
      h[i] = pow(u, (double)i);
      h[nodes + i] = pow(d, (double)i);
    }
    st = cuda_status(cudaMemcpyAsync(dv + o_up, h, 16 * nodes, cudaMemcpyHostToDevice, c->stream),
                     "H2D lattice tables");
    if (!st)
      st = cuda_status(cudaMemsetAsync(dv + o_cnt, 0, 256, c->stream), "memset lattice counters");
    if (st) return st;
    LatticeParams P;
    memset(&P, 0, sizeof P);
    P.S0 = S0;
    P.E = E;
    P.p = p;
    P.q = q;
    P.R = R;
    P.N = N;
    P.pf = payoff_fun;
    P.american = american ? 1 : 0;
    P.up = (const double*)(dv + o_up);
    P.dn = (const double*)(dv + o_dn);
    P.A = (double*)(dv + o_A);
    P.B = (double*)(dv + o_B);
    P.barrier = (unsigned*)(dv + o_cnt);
    P.err = (int*)(dv + o_cnt + 64);
    P.wait_limit = 1u << 22;
    if (c->test_barrier_extra) {  // test hook: a barrier that cannot complete
      P.barrier_extra = c->test_barrier_extra;
      P.wait_limit = c->test_poll_limit;
    }
    P.out = (double*)(dv + o_out);
    int cap = seg_cap;
    void* args[] = {&P, &cap};
    st = cuda_status(cudaLaunchCooperativeKernel((void*)lattice_kernel, dim3(G), dim3(kLatBlock),
                                                 args, smem, c->stream),
                     "lattice kernel launch");
    if (st) return st;
    c->launches += 1;
    st = cuda_status(cudaMemcpyAsync(h, dv + o_out, 8, cudaMemcpyDeviceToHost, c->stream),
                     "D2H lattice");
    if (!st)
      st = cuda_status(cudaMemcpyAsync(h + 1, dv + o_cnt + 64, sizeof(int), cudaMemcpyDeviceToHost,
                                       c->stream),
                       "D2H lattice flag");
    if (!st) st = cuda_status(cudaStreamSynchronize(c->stream), "lattice kernel");
    if (st) return st;
    if (*(const int*)(h + 1)) return set_error(PCF_ETIMEOUT, "lattice grid barrier gave up");
    *price = h[0];
    return PCF_OK;
  });
}
