// Longstaff-Schwartz American pricing (the reference's mc_amer) on one GPU.
//
// Reference: src/mc_amer.cpp:5-114 (serial), src/mc_amer_omp.cpp:5-117, with
// pathsfinder() of include/common.h:168-208 and the 3x3 solve of
// include/common.h:98-141. The MPI build reduces the seven regression sums
// and the in-the-money count to rank 0 and broadcasts three coefficients per
// date (src/mc_amer_mpi.cpp:82-131). Here the same exchange is a grid-wide
// FP64 reduction inside one persistent kernel.
//
// One cooperative launch per contract, at most one 512-thread block per SM:
//   forward   each thread generates its antithetic pairs (path p takes +z,
//             path p + H takes -z, as pathsfinder pairs them) and writes
//             S(date m), m = 1..M, to an FP32 time-major path matrix in HBM
//             (row m-1; plus half at columns [0, Hp), minus half at
//             [Hp, 2Hp), Hp = H rounded up to 4), coalesced across the warp;
//   backward  for m = M-1..1: the block's slice of row m-1 (two contiguous
//             runs) arrives in shared memory by TMA bulk copy. The copy for
//             date m-1 is issued as soon as date m's has landed, so HBM
//             latency hides behind the date's reduction and barrier. The
//             block accumulates the 8 regression sums of its in-the-money
//             paths, publishes one FP64 partial, waits at a bounded group
//             barrier, reduces all partials in block order (every block gets
//             the same bits), solves the normal equations by the adjugate
//             formula and updates the exercise decision of its paths from the
//             same shared-memory slice;
//   final     discounted cash flows and the martingale control variate are
//             averaged over antithetic pairs and reduced with the
//             deterministic last-block finaliser (cooperative launch) or
//             through distributed shared memory (cluster launch).
// Per-path state (cash flow, exercise date) stays in shared memory for the
// whole sweep. The regression basis is {1, x, x^2} with x = (S - E)/E: the
// reference's S - E rescaled, the same fitted values in exact arithmetic.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include <cooperative_groups.h>

#include "pcf_api_internal.h"
#include "pcf_device.cuh"
#include "pcf_math.h"

namespace cg = cooperative_groups;

namespace pcf {

namespace {

constexpr int kLsmBlock = 512;
constexpr int kRegSums = 8;  // n, x, x^2, x^3, x^4, y, y x, y x^2
constexpr size_t kLsmMaxSmem = 227 * 1024;

struct LsmParams {
  float pf, nK, E, invE;  // payoff = max(pf S + nK, 0); x = (S - E) * invE
  float a2, b2, l2S0;     // per-date log2 drift / vol, log2 S0
  float gdisc;            // exp(-rT)
  float rf, sigf, dtf;    // r, sigma, T/M: the European price of the control variate
  int M, ref_exercise;
  long long H;            // antithetic pairs = N / 2
  long long Hp;           // H rounded up to a multiple of 4
  int pairs_per_block;    // PB, a multiple of 4
  int nblocks;
  uint32_t seed_lo, seed_hi, stream;
  unsigned wait_limit;       // group-barrier polls before giving up
  unsigned copy_wait_limit;  // mbarrier polls before giving up on a bulk copy
  float* paths;           // M rows of 2*Hp floats
  const float* dtab;      // exp(-r dt k), k = 0..M
  double* partial;        // 2 x nblocks x kRegSums
  double* fpartial;       // nblocks x kMoments
  unsigned* barrier;
  unsigned* ticket;
  int* err;               // 1: a barrier wait gave up, 2: a bulk copy wait gave up
  int* singular;          // dates whose normal equations had det <= 0
  double* out;            // kMoments sums
};

__device__ __forceinline__ float lsm_payoff(const LsmParams& P, float S) {
  return fmaxf(fmaf(P.pf, S, P.nK), 0.f);
}

__device__ __forceinline__ float norm_cdf_f(float x) { return 0.5f * erfcf(-x * 0.70710678f); }

// Black-Scholes price of the European option with time `rem` to expiry, FP32.
__device__ float european_price(const LsmParams& P, float S, float rem) {
  const float sd = P.sigf * sqrtf(rem);
  const float dK = P.E * expf(-P.rf * rem);
  if (!(sd > 0.f)) return fmaxf(P.pf * (S - dK), 0.f);
  const float d1 = (logf(S * P.invE) + (P.rf + 0.5f * P.sigf * P.sigf) * rem) / sd;
  const float d2 = d1 - sd;
  if (P.pf > 0.f) return S * norm_cdf_f(d1) - dK * norm_cdf_f(d2);
  return dK * norm_cdf_f(-d2) - S * norm_cdf_f(-d1);
}

// include/common.h:98-141: the adjugate over the determinant, then the
// mat-vec product. The normal matrix of the basis {1, x, x^2} is the symmetric
// Hankel matrix [[a0,a1,a2],[a1,a2,a3],[a2,a3,a4]], so its adjugate has six
// distinct cofactors. They are formed with FMAs, and one reciprocal replaces
// nine divisions. In exact arithmetic this is the reference's solution; FP64
// is slow on GB300, so the short chain matters (it runs once per date on the
// critical path).
__device__ bool solve3(const double* a, double* coef) {
  const double c00 = fma(a[2], a[4], -a[3] * a[3]);
  const double c01 = fma(a[2], a[3], -a[1] * a[4]);
  const double c02 = fma(a[1], a[3], -a[2] * a[2]);
  const double c11 = fma(a[0], a[4], -a[2] * a[2]);
  const double c12 = fma(a[1], a[2], -a[0] * a[3]);
  const double c22 = fma(a[0], a[2], -a[1] * a[1]);
  const double det = fma(a[0], c00, fma(a[1], c01, a[2] * c02));
  if (!(det > 0)) return false;
  const double rd = 1.0 / det;
  const double y0 = a[5], y1 = a[6], y2 = a[7];
  coef[0] = fma(c00, y0, fma(c01, y1, c02 * y2)) * rd;
  coef[1] = fma(c01, y0, fma(c11, y1, c12 * y2)) * rd;
  coef[2] = fma(c02, y0, fma(c12, y1, c22 * y2)) * rd;
  return true;
}

struct LsmSmem {
  uint64_t* bar;           // 2 mbarriers
  float* dt;               // M+1
  float* cf;               // 2*PB
  unsigned short* tau;     // 2*PB
  float* buf[2];           // 2 x 2*PB path slices
};

__device__ __forceinline__ LsmSmem carve(unsigned char* base, int PB, int M) {
  LsmSmem s;
  size_t o = 0;
  s.bar = (uint64_t*)(base + o);
  o += 16;
  s.dt = (float*)(base + o);
  o += ((size_t)(M + 1) * 4 + 15) & ~(size_t)15;
  s.cf = (float*)(base + o);
  o += (size_t)2 * PB * 4;
  s.tau = (unsigned short*)(base + o);
  o += ((size_t)2 * PB * 2 + 15) & ~(size_t)15;
  s.buf[0] = (float*)(base + o);
  o += (size_t)2 * PB * 4;
  s.buf[1] = (float*)(base + o);
  return s;
}

// Bulk-copies the block's slice of row r (pairs [p0, p0 + nbr)) to dst:
// plus half to dst[0..nbr), minus half to dst[PB..PB + nbr).
__device__ __forceinline__ void issue_row(const LsmParams& P, const LsmSmem& S, int r,
                                          long long p0, int nbr, int PB, float* dst,
                                          uint64_t* bar) {
  const float* row = P.paths + (size_t)r * 2 * P.Hp;
  const uint32_t bytes = (uint32_t)nbr * 4u;
  mbar_arrive_expect_tx(bar, 2u * bytes);
  bulk_g2s(dst, row + p0, bytes, bar);
  bulk_g2s(dst + PB, row + P.Hp + p0, bytes, bar);
}

// Adds the regression sums of the in-the-money paths of one slice entry.
__device__ __forceinline__ void reg_accumulate(const LsmParams& P, float Sv, float y, float* acc) {
  const float x = (Sv - P.E) * P.invE;
  const float x2 = x * x;
  acc[0] += 1.f;
  acc[1] += x;
  acc[2] += x2;
  acc[3] = fmaf(x2, x, acc[3]);
  acc[4] = fmaf(x2, x2, acc[4]);
  acc[5] += y;
  acc[6] = fmaf(y, x, acc[6]);
  acc[7] = fmaf(y, x2, acc[7]);
}

// Block reduction of the regression sums for date m, the exchange of block
// partials, the 3x3 solve, and the issue of the next bulk copy.
//   cooperative launch (CLUSTER = false): each block publishes its partial in
//     global memory, waits at the bounded group barrier, then every block
//     sums all partials in block order (so all blocks get the same bits);
//   cluster launch (CLUSTER = true, one cluster per contract): each CTA keeps
//     its partial in shared memory; after a hardware cluster barrier every
//     CTA reads all CTAs' partials through distributed shared memory, in
//     rank order.
// Leaves the date's mode and coefficients in shared memory. When `next_row`
// >= 0, thread 0 issues the bulk copy of that row into `next_buf` once every
// thread is past the slice that buffer held. Returns false if a bounded wait
// gave up (cooperative launch only).
template <bool CLUSTER>
__device__ bool lsm_regress(const LsmParams& P, const LsmSmem& S, float (&acc)[kRegSums], int m,
                            int b, DF* sh, DF (*red)[kRegSums], double* s_coef, int* s_mode,
                            int next_row, long long p0, int nbr, int PB, float* next_buf,
                            uint64_t* next_bar) {
  DF v[kRegSums], tot[kRegSums];
#pragma unroll
  for (int q = 0; q < kRegSums; ++q) v[q] = DF{acc[q], 0.f};
  block_sum_df<kRegSums>(v, sh, tot);  // ends with __syncthreads: slices are free
  float2* slot = (float2*)P.partial + (size_t)(m & 1) * P.nblocks * kRegSums;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < kRegSums; ++q) {
      if (CLUSTER) red[m & 1][q] = tot[q];
      else slot[(size_t)b * kRegSums + q] = make_float2(tot[q].hi, tot[q].lo);
    }
    if (next_row >= 0 && nbr > 0) issue_row(P, S, next_row, p0, nbr, PB, next_buf, next_bar);
  }
  if (CLUSTER) {
    cg::this_cluster().sync();
  } else {
    if (!group_barrier(P.barrier, (unsigned)P.nblocks, P.err, P.wait_limit)) return false;
  }
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    DF g[kRegSums];
#pragma unroll
    for (int q = 0; q < kRegSums; ++q) g[q] = DF{0.f, 0.f};
    if (CLUSTER) {
      if (lane < P.nblocks) {
        const DF* rr = cg::this_cluster().map_shared_rank(&red[m & 1][0], lane);
#pragma unroll
        for (int q = 0; q < kRegSums; ++q) g[q] = rr[q];
      }
    } else {
      for (int bb = lane; bb < P.nblocks; bb += 32) {
        const float4* r4 = (const float4*)(slot + (size_t)bb * kRegSums);
        float4 a[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) a[u] = __ldcg(r4 + u);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          g[2 * u] = df_add(g[2 * u], DF{a[u].x, a[u].y});
          g[2 * u + 1] = df_add(g[2 * u + 1], DF{a[u].z, a[u].w});
        }
      }
    }
    double t[kRegSums];
#pragma unroll
    for (int q = 0; q < kRegSums; ++q) t[q] = df_value(warp_sum_df(g[q]));
    if (lane == 0) {
      if (t[0] == 0.0) {
        *s_mode = 0;
      } else if (t[0] <= 2.0) {
        *s_mode = 1;
      } else {
        double c[3];
        if (solve3(t, c)) {
          *s_mode = 2;
          s_coef[0] = c[0];
          s_coef[1] = c[1];
          s_coef[2] = c[2];
        } else {
          *s_mode = 0;
          if (b == 0) atomicAdd(P.singular, 1);
        }
      }
    }
  }
  __syncthreads();
  return true;
}

// Exercise decision of one path at date m (src/mc_amer.cpp:73-106).
__device__ __forceinline__ void lsm_update(const LsmParams& P, const LsmSmem& S, int s, float Sv,
                                           int m, int mode, float c0, float c1, float c2) {
  const float pv = lsm_payoff(P, Sv);
  if (pv > 0.f) {
    float cont, ex = pv;
    if (mode == 1) {
      cont = S.cf[s] * S.dt[S.tau[s] - m];
    } else {
      const float x = (Sv - P.E) * P.invE;
      cont = fmaf(fmaf(c2, x, c1), x, c0);
      // src/mc_amer.cpp:100: the reference exercises at payoff(S - E, E).
      if (P.ref_exercise) ex = fmaxf(P.pf * (Sv - 2.f * P.E), 0.f);
    }
    if (ex > cont) {
      S.cf[s] = ex;
      S.tau[s] = (unsigned short)m;
    }
  }
}

// One contract's forward pass, backward sweep and final moments, executed by
// block `b` of the contract's `P.nblocks` blocks. In a cluster launch a
// failed copy wait is recorded and the CTA keeps taking part in every cluster
// barrier (a hardware barrier has no timeout), so no CTA leaves early.
template <bool CLUSTER>
__device__ void lsm_body(const LsmParams& P, int b) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int PB = P.pairs_per_block;
  const int M = P.M;
  const LsmSmem S = carve(smem_raw, PB, M);
  __shared__ DF sh[32 * kRegSums];
  __shared__ DF red[2][kRegSums];
  __shared__ DF fin[kMoments];
  __shared__ double s_coef[3];
  __shared__ int s_mode;  // 0 skip date, 1 few ITM paths, 2 regression
  __shared__ int s_ok;

  const long long p0 = (long long)b * PB;
  const int nb = (int)max(0LL, min((long long)PB, P.H - p0));  // pairs in this block
  const int nbr = (nb + 3) & ~3;                                // bulk-copy width
  for (int k = threadIdx.x; k <= M; k += kLsmBlock) S.dt[k] = P.dtab[k];
  if (threadIdx.x == 0) {
    mbar_init(&S.bar[0], 1);
    mbar_init(&S.bar[1], 1);
    fence_mbar_init();
  }

  // ---- forward: generate and store paths ----
  const RngKey key{P.seed_lo, P.seed_hi, P.stream, TAG_AMER};
  for (int i = threadIdx.x; i < nb; i += kLsmBlock) {
    const long long p = p0 + i;
    float Lp = 0.f, Lm = 0.f, Sp = 0.f, Sm = 0.f;
    float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int m = 1; m <= M; ++m) {
      if (((m - 1) & 3) == 0) z4 = normals4(draw_words(key, (uint64_t)p, (uint32_t)((m - 1) >> 2)));
      const float z = lane4(z4, (m - 1) & 3);
      Lp += fmaf(P.b2, z, P.a2);
      Lm += fmaf(-P.b2, z, P.a2);
      Sp = ex2_approx(P.l2S0 + Lp);
      Sm = ex2_approx(P.l2S0 + Lm);
      float* row = P.paths + (size_t)(m - 1) * 2 * P.Hp;
      row[p] = Sp;
      row[P.Hp + p] = Sm;
    }
    S.cf[i] = lsm_payoff(P, Sp);
    S.cf[PB + i] = lsm_payoff(P, Sm);
    S.tau[i] = (unsigned short)M;
    S.tau[PB + i] = (unsigned short)M;
  }
  // The bulk copies below read what this block's threads just stored.
  fence_proxy_async_global();
  __syncthreads();

  // Buffer schedule: date d's slice sits in buf[(M - 1 - d) & 1]. Thread 0
  // owns the copies; pending[k] says a copy into buf[k] is in flight.
  bool pending[2] = {false, false};
  uint32_t parity[2] = {0u, 0u};
  bool alive = true;
  auto wait_buf = [&](int k) {  // thread 0 only
    if (!pending[k]) return true;
    if (!mbar_wait(&S.bar[k], parity[k], P.copy_wait_limit)) return false;
    parity[k] ^= 1u;
    pending[k] = false;
    return true;
  };
  if (threadIdx.x == 0) {
    s_ok = 1;
    if (nbr > 0) {
      issue_row(P, S, M - 2, p0, nbr, PB, S.buf[0], &S.bar[0]);  // date M-1
      pending[0] = true;
      if (!wait_buf(0)) {
        atomicExch(P.err, 2);
        s_ok = 0;
      }
    }
  }
  __syncthreads();
  if (!CLUSTER) alive = s_ok != 0;

  // Sums for date M-1 (the only date without a preceding update pass).
  if (alive) {
    float acc[kRegSums];
#pragma unroll
    for (int q = 0; q < kRegSums; ++q) acc[q] = 0.f;
    const float* sl = S.buf[0];
    for (int i = threadIdx.x; i < nb; i += kLsmBlock) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int s = h * PB + i;
        const float Sv = sl[s];
        if (lsm_payoff(P, Sv) > 0.f) reg_accumulate(P, Sv, S.cf[s] * S.dt[S.tau[s] - (M - 1)], acc);
      }
    }
    if (threadIdx.x == 0 && M - 2 >= 1 && nbr > 0) pending[1] = true;  // issued in lsm_regress
    alive = lsm_regress<CLUSTER>(P, S, acc, M - 1, b, sh, red, s_coef, &s_mode,
                                 M - 2 >= 1 ? M - 3 : -1, p0, nbr, PB, S.buf[1], &S.bar[1]);
  }

  // Date m: update with date m's coefficients, fused with the sums of date m-1.
  for (int m = M - 1; m >= 1 && alive; --m) {
    const int k = (M - 1 - m) & 1;
    const bool has_next = m > 1;
    if (has_next) {
      if (threadIdx.x == 0) {
        s_ok = 1;
        if (nbr > 0 && !wait_buf(k ^ 1)) {
          atomicExch(P.err, 2);
          s_ok = 0;
        }
      }
      __syncthreads();
      if (!s_ok && !CLUSTER) {
        alive = false;
        break;
      }
    }
    const int mode = s_mode;
    const float c0 = (float)s_coef[0], c1 = (float)s_coef[1], c2 = (float)s_coef[2];
    const float* cur = S.buf[k];
    const float* nxt = S.buf[k ^ 1];
    float acc[kRegSums];
#pragma unroll
    for (int q = 0; q < kRegSums; ++q) acc[q] = 0.f;
    for (int i = threadIdx.x; i < nb; i += kLsmBlock) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int s = h * PB + i;
        if (mode != 0) lsm_update(P, S, s, cur[s], m, mode, c0, c1, c2);
        if (has_next) {
          const float Sv = nxt[s];
          if (lsm_payoff(P, Sv) > 0.f) reg_accumulate(P, Sv, S.cf[s] * S.dt[S.tau[s] - (m - 1)], acc);
        }
      }
    }
    if (!has_next) break;
    // buf[k] (date m) is free once lsm_regress's block reduction has synced;
    // date m-2 goes there.
    const int next_row = m - 2 >= 1 ? m - 3 : -1;
    if (threadIdx.x == 0 && next_row >= 0 && nbr > 0) pending[k] = true;
    alive = lsm_regress<CLUSTER>(P, S, acc, m - 1, b, sh, red, s_coef, &s_mode, next_row, p0,
                                 nbr, PB, S.buf[k], &S.bar[k]);
  }
  __syncthreads();
  if (!alive) {
    // Let any bulk copy this block issued land before the block exits.
    if (threadIdx.x == 0)
      for (int k = 0; k < 2; ++k)
        if (pending[k]) mbar_wait(&S.bar[k], parity[k], P.copy_wait_limit);
    return;
  }

  // ---- discounted cash flows and the control variate, per antithetic pair ----
  // Moments are taken over pair means: the two paths of a pair share their
  // draws, so the pair, not the path, is the independent sample.
  // Control variate (martingale CV): g = e^{-r tau} P_E(S_tau, T - tau), the
  // discounted European price at the path's exercise time. The discounted
  // European price is a martingale, so E[g] = P_E(S0, T) for any stopping
  // time. S_tau is E + pf*cf where the path exercised (or finished in the
  // money) and S_M from the last row otherwise.
  const float* last = P.paths + (size_t)(M - 1) * 2 * P.Hp;
  KSum sy, syy, sg, sgg, syg;
  for (int i = threadIdx.x; i < nb; i += kLsmBlock) {
    float y2 = 0.f, g2 = 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int s = h * PB + i;
      const int tau = S.tau[s];
      const float cf = S.cf[s];
      y2 += cf * S.dt[tau];
      float g;
      if (P.ref_exercise) {
        // The reference's exercise value does not identify S_tau: use the
        // discounted European payoff at T (mean: the same P_E(S0, T)).
        g = S.dt[M] * lsm_payoff(P, last[h * P.Hp + p0 + i]);
      } else if (tau == M) {
        g = cf * S.dt[M];  // European payoff at T (cf is payoff(S_M)), discounted
      } else {
        const float St = P.E + P.pf * cf;
        g = S.dt[tau] * european_price(P, St, (float)(M - tau) * P.dtf);
      }
      g2 += g;
    }
    const float y = 0.5f * y2, g = 0.5f * g2;
    sy.add(y);
    syy.add(y * y);
    sg.add(g);
    sgg.add(g * g);
    syg.add(y * g);
  }
  DF v[kMoments] = {df_of(sy), df_of(syy), df_of(sg), df_of(sgg), df_of(syg)};
  DF tot[kMoments];
  block_sum_df<kMoments>(v, sh, tot);
  if (CLUSTER) {
    if (threadIdx.x == 0)
      for (int q = 0; q < kMoments; ++q) fin[q] = tot[q];
    cg::this_cluster().sync();
    if (b == 0 && threadIdx.x == 0) {
      DF t[kMoments];
      for (int q = 0; q < kMoments; ++q) t[q] = DF{0.f, 0.f};
      for (int r = 0; r < P.nblocks; ++r) {
        const DF* rf = cg::this_cluster().map_shared_rank(&fin[0], r);
        for (int q = 0; q < kMoments; ++q) t[q] = df_add(t[q], rf[q]);
      }
      for (int q = 0; q < kMoments; ++q) P.out[q] = df_value(t[q]);
    }
    cg::this_cluster().sync();  // rank 0 has read every CTA's shared memory
  } else {
    grid_finalize_df<kMoments>(tot, (float2*)P.fpartial, P.ticket, P.out, P.nblocks, b);
  }
}

__global__ void __launch_bounds__(kLsmBlock) lsm_kernel(LsmParams P) {
  lsm_body<false>(P, blockIdx.x);
}

// Many contracts in one launch, one thread-block cluster per contract
// (cluster size = the contracts' common block count).
__global__ void __launch_bounds__(kLsmBlock) lsm_cluster_kernel(const LsmParams* __restrict__ cs) {
  __shared__ LsmParams sP;  // the contract's parameters, read from shared memory
  const unsigned rank = cg::this_cluster().block_rank();
  const int c = (int)(blockIdx.x / cg::this_cluster().num_blocks());
  if (threadIdx.x == 0) sP = cs[c];
  __syncthreads();
  lsm_body<true>(sP, (int)rank);
}

size_t lsm_smem(int PB, int M) {
  return 16 + ((((size_t)M + 1) * 4 + 15) & ~(size_t)15) + (size_t)2 * PB * 4 +
         (((size_t)2 * PB * 2 + 15) & ~(size_t)15) + (size_t)2 * 2 * PB * 4;
}

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

// Parameters of one contract that do not depend on where its buffers live.
void lsm_fill(LsmParams& P, double S0, double E, double r, double sigma, double T, long long N,
              int M, int pf, int ref_exercise, unsigned long long seed, unsigned stream) {
  const double log2e = 1.4426950408889634;
  const double dtd = T / M;
  memset(&P, 0, sizeof P);
  P.pf = (float)pf;
  P.nK = (float)(-pf * E);
  P.E = (float)E;
  P.invE = (float)(1.0 / E);
  P.a2 = (float)((r - 0.5 * sigma * sigma) * dtd * log2e);
  P.b2 = (float)(sigma * sqrt(dtd) * log2e);
  P.l2S0 = (float)(log(S0) * log2e);
  P.gdisc = (float)exp(-r * T);
  P.rf = (float)r;
  P.sigf = (float)sigma;
  P.dtf = (float)dtd;
  P.M = M;
  P.ref_exercise = ref_exercise ? 1 : 0;
  P.H = N / 2;
  P.Hp = (P.H + 3) & ~3LL;
  P.seed_lo = (uint32_t)seed;
  P.seed_hi = (uint32_t)(seed >> 32);
  P.stream = stream;
  P.wait_limit = 1u << 22;       // ~64 ns sleep + an L2 round trip per poll: seconds
  P.copy_wait_limit = 1u << 20;  // try_wait polls: far beyond a microsecond-scale copy
}

void dtab_fill(float* dst, double r, double T, int M) {
  const double dtd = T / M;
  for (int k = 0; k <= M; ++k) dst[k] = (float)exp(-r * dtd * k);
}

constexpr size_t kStaticSmemReserve = 4096;  // lsm_body's static shared arrays

// Cooperative-launch grid for one contract: at most one block per SM, at
// least one pair per thread. Returns false if it cannot be co-resident.
bool coop_shape(const pcf_ctx* c, long long H, int M, int& G, int& PB, size_t& smem) {
  const long long G0 = std::max(1LL, std::min((H + kLsmBlock - 1) / kLsmBlock,
                                              (long long)c->sm_count));
  PB = (int)((((H + G0 - 1) / G0) + 3) & ~3LL);
  G = (int)((H + PB - 1) / PB);
  smem = lsm_smem(PB, M);
  return smem + kStaticSmemReserve <= kLsmMaxSmem;
}

}  // namespace

int check_lsm_request(double S0, double E, double r, double sigma, double T, long long N, int M,
                      int pf) {
  int st = check_common(S0, E, r, sigma, T, N, pf);
  if (st) return st;
  if (N % 2 != 0)  // include/common.h:180
    return set_error(PCF_EINVAL, "N needs to be divisible by 2 for finding paths");
  if (M < 2 || M > 4096) return set_error(PCF_EINVAL, "M must be in [2, 4096]");
  if (!(E > 0)) return set_error(PCF_EINVAL, "E must be > 0 for the LSM regression basis");
  return PCF_OK;
}

void fill_amer_result(const double* s, long long N, double S0, double E, double r, double sigma,
                      double T, int pf, bool use_cv, pcf_mc_result* out) {
  // The sums run over N/2 antithetic pair means (the independent samples).
  fill_result(s, N / 2, bs_price(S0, E, r, sigma, T, pf), 1.0, use_cv, out);
  out->n_paths = N;
  // src/mc_amer.cpp:113: the price is at least the immediate exercise value.
  const double intrinsic = std::max(pf * (S0 - E), 0.0);
  out->price = std::max(out->price, intrinsic);
  out->price_plain = std::max(out->price_plain, intrinsic);
  if (use_cv) out->price_cv = std::max(out->price_cv, intrinsic);
}

// ---- batches of American contracts (used by pcf_plan_*) ----

struct LsmCluster {  // one cluster launch: every contract with the same shape
  int CL = 0, PB = 0, C = 0;
  size_t smem = 0;
  LsmParams* d_params = nullptr;
};

struct LsmBatch {
  std::vector<LsmCluster> clusters;
  std::vector<LsmParams> coop;  // contracts too large for one cluster
  std::vector<int> coop_grid;
  std::vector<size_t> coop_smem;
  void* d_mem = nullptr;
  size_t bytes = 0;
};

int lsm_cluster_size(pcf_ctx* c) {
  // 16 CTAs per cluster where the device can co-schedule them, else 8.
  static int cached = 0;
  if (cached) return cached;
  cudaFuncSetAttribute(lsm_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  const size_t smem = lsm_smem(8192, 64);
  cudaFuncSetAttribute(lsm_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 16;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(16);
  cfg.blockDim = dim3(kLsmBlock);
  cfg.dynamicSmemBytes = smem;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, lsm_cluster_kernel, &cfg) == cudaSuccess && n > 0)
    cached = 16;
  else
    cached = 8;
  cudaGetLastError();
  (void)c;
  return cached;
}

// Shapes and device layout of a batch: params tables | discount tables (the
// uploaded prefix) | cooperative scratch | path matrices.
struct LsmLayout {
  std::vector<int> cls;  // index into kLsmPB, or -1 for the cooperative kernel
  std::vector<int> cl;   // CTAs per contract (cluster size)
  std::vector<std::vector<int>> members;
  std::vector<size_t> o_params, o_dt, o_paths, o_coop;
  std::vector<int> coop_G, coop_PB;
  std::vector<size_t> coop_sm;
  size_t upload = 0, total = 0;
};

constexpr int kLsmPB[] = {512, 1024, 2048, 4096, 8192};

int lsm_layout(pcf_ctx* c, const std::vector<LsmRequest>& reqs, LsmLayout& L) {
  const size_t n = reqs.size();
  // Shape of each contract: a cluster of the device's full size (16 CTAs
  // where allowed), with the smallest slice class that covers the contract.
  // Small slices keep each CTA's shared memory low, so two CTAs share an SM
  // and more contracts are in flight; a contract too large for a cluster
  // runs the cooperative kernel.
  const int CLmax = lsm_cluster_size(c);
  L.cls.assign(n, -1);
  L.cl.assign(n, 0);
  for (size_t i = 0; i < n; ++i) {
    const long long H = reqs[i].N / 2;
    const int cl = CLmax;
    for (int k = 0; k < 5; ++k)
      if ((long long)cl * kLsmPB[k] >= H &&
          lsm_smem(kLsmPB[k], reqs[i].M) + kStaticSmemReserve <= kLsmMaxSmem) {
        L.cls[i] = k;
        L.cl[i] = cl;
        break;
      }
  }
  // Launch groups: one per (cluster size, slice class).
  L.members.assign(5 * 5, {});
  for (size_t i = 0; i < n; ++i)
    if (L.cls[i] >= 0) {
      int lg = 0;
      while ((1 << lg) < L.cl[i]) ++lg;
      L.members[lg * 5 + L.cls[i]].push_back((int)i);
    }
  size_t off = 0;
  L.o_params.assign(L.members.size(), 0);
  for (size_t k = 0; k < L.members.size(); ++k) {
    L.o_params[k] = off;
    off = a256(off + sizeof(LsmParams) * L.members[k].size());
  }
  L.o_dt.assign(n, 0);
  for (size_t i = 0; i < n; ++i) {
    L.o_dt[i] = off;
    off = a256(off + sizeof(float) * (reqs[i].M + 1));
  }
  L.upload = off;
  L.coop_G.assign(n, 0);
  L.coop_PB.assign(n, 0);
  L.coop_sm.assign(n, 0);
  L.o_coop.assign(n, 0);
  for (size_t i = 0; i < n; ++i) {
    if (L.cls[i] >= 0) continue;
    if (!coop_shape(c, reqs[i].N / 2, reqs[i].M, L.coop_G[i], L.coop_PB[i], L.coop_sm[i]))
      return set_error(PCF_EINVAL, "American request with N = %lld is too large", reqs[i].N);
    L.o_coop[i] = off;  // partial (2 G 8 float2) | fpartial (G 5 float2) | 2 counters
    off = a256(off + 8 * (2 * (size_t)L.coop_G[i] * kRegSums + (size_t)L.coop_G[i] * kMoments) +
               16);
  }
  L.o_paths.assign(n, 0);
  for (size_t i = 0; i < n; ++i) {
    L.o_paths[i] = off;
    const long long Hp = ((reqs[i].N / 2) + 3) & ~3LL;
    off = a256(off + sizeof(float) * (size_t)reqs[i].M * 2 * (size_t)Hp);
  }
  L.total = std::max(off, (size_t)256);
  return PCF_OK;
}

int lsm_batch_bytes(pcf_ctx* c, const std::vector<LsmRequest>& reqs, size_t* dev,
                    size_t* host) {
  LsmLayout L;
  const int st = lsm_layout(c, reqs, L);
  if (st) return st;
  *dev = L.total;
  *host = L.upload;
  return PCF_OK;
}

int lsm_batch_create(pcf_ctx* c, const std::vector<LsmRequest>& reqs, cudaStream_t s,
                     ExtMem* mem, LsmBatch** out) {
  *out = nullptr;
  LsmLayout Lo;
  int st = lsm_layout(c, reqs, Lo);
  if (st) return st;
  LsmBatch* B = new LsmBatch();
  char* d = nullptr;
  char* h = nullptr;
  std::vector<char> hown;
  if (mem) {
    d = mem->dalloc(Lo.total);
    h = mem->halloc(Lo.upload);
    if (!d || !h) {
      delete B;
      return set_error(PCF_ENOMEM, "American batch needs %zu device bytes; the slot is full",
                       Lo.total);
    }
  } else {
    if (c->budget_bytes && Lo.total > c->budget_bytes) {
      delete B;
      return set_error(PCF_ENOMEM, "American batch needs %zu device bytes, over the budget",
                       Lo.total);
    }
    st = cuda_status(cudaMalloc(&B->d_mem, Lo.total), "cudaMalloc(LSM batch)");
    if (st) {
      delete B;
      return st;
    }
    d = (char*)B->d_mem;
    hown.assign(Lo.upload, 0);
    h = hown.data();
  }
  B->bytes = Lo.total;
  auto fill = [&](size_t i, LsmParams& P) {
    const LsmRequest& q = reqs[i];
    lsm_fill(P, q.S0, q.E, q.r, q.sigma, q.T, q.N, q.M, q.pf, q.ref_exercise, q.seed, q.stream);
    dtab_fill((float*)(h + Lo.o_dt[i]), q.r, q.T, q.M);
    P.dtab = (const float*)(d + Lo.o_dt[i]);
    P.paths = (float*)(d + Lo.o_paths[i]);
    P.out = q.d_out;
    P.err = q.d_flags;
    P.singular = q.d_flags + 1;
  };
  for (size_t k = 0; k < Lo.members.size(); ++k) {
    if (Lo.members[k].empty()) continue;
    LsmCluster L;
    L.CL = 1 << (k / 5);
    L.PB = kLsmPB[k % 5];
    L.C = (int)Lo.members[k].size();
    int Mmax = 2;
    LsmParams* tab = (LsmParams*)(h + Lo.o_params[k]);
    for (int j = 0; j < L.C; ++j) {
      const int i = Lo.members[k][j];
      fill(i, tab[j]);
      tab[j].pairs_per_block = L.PB;
      tab[j].nblocks = L.CL;
      Mmax = std::max(Mmax, reqs[i].M);
    }
    L.smem = lsm_smem(L.PB, Mmax);
    L.d_params = (LsmParams*)(d + Lo.o_params[k]);
    B->clusters.push_back(L);
  }
  for (size_t i = 0; i < reqs.size(); ++i) {
    if (Lo.cls[i] >= 0) continue;
    LsmParams P;
    fill(i, P);
    P.pairs_per_block = Lo.coop_PB[i];
    P.nblocks = Lo.coop_G[i];
    char* base = d + Lo.o_coop[i];
    P.partial = (double*)base;
    P.fpartial = (double*)(base + 8 * 2 * (size_t)Lo.coop_G[i] * kRegSums);
    unsigned* cnt = (unsigned*)(base + 8 * (2 * (size_t)Lo.coop_G[i] * kRegSums +
                                            (size_t)Lo.coop_G[i] * kMoments));
    P.barrier = cnt;
    P.ticket = cnt + 1;
    B->coop.push_back(P);
    B->coop_grid.push_back(Lo.coop_G[i]);
    B->coop_smem.push_back(Lo.coop_sm[i]);
  }
  st = cuda_status(cudaMemcpyAsync(d, h, Lo.upload, cudaMemcpyHostToDevice, s), "H2D LSM batch");
  if (!st && !mem) st = cuda_status(cudaStreamSynchronize(s), "LSM batch upload");
  if (st) {
    lsm_batch_destroy(B);
    return st;
  }
  *out = B;
  return PCF_OK;
}

int lsm_batch_launch(pcf_ctx* c, LsmBatch* B, cudaStream_t s) {
  int st;
  for (const LsmCluster& L : B->clusters) {
    st = cuda_status(cudaFuncSetAttribute(lsm_cluster_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)L.smem),
                     "lsm cluster smem attribute");
    if (st) return st;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = L.CL;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(L.C * L.CL);
    cfg.blockDim = dim3(kLsmBlock);
    cfg.dynamicSmemBytes = L.smem;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    st = cuda_status(cudaLaunchKernelEx(&cfg, lsm_cluster_kernel,
                                        (const LsmParams*)L.d_params),
                     "lsm cluster launch");
    if (st) return st;
    c->launches += 1;
  }
  for (size_t i = 0; i < B->coop.size(); ++i) {
    LsmParams& P = B->coop[i];
    st = cuda_status(cudaMemsetAsync(P.barrier, 0, 2 * sizeof(unsigned), s), "memset LSM counters");
    if (st) return st;
    st = cuda_status(cudaFuncSetAttribute(lsm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)B->coop_smem[i]),
                     "lsm smem attribute");
    if (st) return st;
    void* args[] = {&P};
    st = cuda_status(cudaLaunchCooperativeKernel((void*)lsm_kernel, dim3(B->coop_grid[i]),
                                                 dim3(kLsmBlock), args, B->coop_smem[i], s),
                     "lsm cooperative launch");
    if (st) return st;
    c->launches += 1;
  }
  return PCF_OK;
}

int lsm_batch_kernels(const LsmBatch* B) { return (int)(B->clusters.size() + B->coop.size()); }

void lsm_batch_destroy(LsmBatch* B) {
  if (!B) return;
  if (B->d_mem) cudaFree(B->d_mem);
  delete B;
}

}  // namespace pcf

using namespace pcf;

extern "C" int pcf_mc_amer(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T,
                           long long N, int M, int payoff_fun, int ref_exercise,
                           unsigned long long seed, int use_cv, pcf_mc_result* out) {
  if (!out) return set_error(PCF_EINVAL, "out is NULL");
  int st = check_lsm_request(S0, E, r, sigma, T, N, M, payoff_fun);
  if (st) return st;
  pcf_ctx* c = resolve_ctx(ctx, &st);
  if (!c) return st;
  int G = 0, PB = 0;
  size_t smem = 0;
  if (!coop_shape(c, N / 2, M, G, PB, smem))
    return set_error(PCF_EINVAL, "N = %lld is too large for one device sweep", N);
  st = cuda_status(cudaFuncSetAttribute(lsm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem),
                   "lsm smem attribute");
  if (st) return st;
  int occ = 0;
  st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lsm_kernel, kLsmBlock, smem),
                   "occupancy(lsm)");
  if (st) return st;
  if ((long long)occ * c->sm_count < G)
    return set_error(PCF_EINVAL, "LSM grid of %d blocks cannot be co-resident", G);

  LsmParams P;
  lsm_fill(P, S0, E, r, sigma, T, N, M, payoff_fun, ref_exercise, seed, 0);
  P.pairs_per_block = PB;
  P.nblocks = G;
  // Resident path matrix: M rows x 2*Hp floats.
  const size_t paths_bytes = sizeof(float) * (size_t)M * 2 * (size_t)P.Hp;
  if (paths_bytes > c->paths_cap) {
    if (c->d_paths) cudaFree(c->d_paths);
    c->d_paths = nullptr;
    c->paths_cap = 0;
    if (c->budget_bytes && paths_bytes > c->budget_bytes)
      return set_error(PCF_ENOMEM, "path matrix of %zu bytes exceeds the context budget",
                       paths_bytes);
    st = cuda_status(cudaMalloc(&c->d_paths, paths_bytes), "cudaMalloc(path matrix)");
    if (st) return st;
    c->paths_cap = paths_bytes;
  }
  // Scratch: dtab | partial | fpartial | counters | out.
  const size_t o_dt = 0;
  const size_t o_part = a256(o_dt + sizeof(float) * (M + 1));
  const size_t o_fpart = a256(o_part + sizeof(double) * 2 * G * kRegSums);
  const size_t o_cnt = a256(o_fpart + sizeof(double) * G * kMoments);
  const size_t o_out = a256(o_cnt + sizeof(unsigned) * 4);
  const size_t total = a256(o_out + sizeof(double) * kMoments);
  st = ctx_ensure(c, total, total);
  if (st) return st;
  char* d = (char*)c->d_buf;
  char* h = (char*)c->h_buf;
  dtab_fill((float*)(h + o_dt), r, T, M);
  st = cuda_status(cudaMemcpyAsync(d + o_dt, h + o_dt, sizeof(float) * (M + 1),
                                   cudaMemcpyHostToDevice, c->stream), "H2D dtab");
  if (!st) st = cuda_status(cudaMemsetAsync(d + o_cnt, 0, sizeof(unsigned) * 4, c->stream),
                            "memset counters");
  if (st) return st;
  P.paths = (float*)c->d_paths;
  P.dtab = (const float*)(d + o_dt);
  P.partial = (double*)(d + o_part);
  P.fpartial = (double*)(d + o_fpart);
  unsigned* cnt = (unsigned*)(d + o_cnt);
  P.barrier = cnt;
  P.ticket = cnt + 1;
  P.err = (int*)(cnt + 2);
  P.singular = (int*)(cnt + 3);
  P.out = (double*)(d + o_out);
  void* args[] = {&P};
  st = cuda_status(cudaLaunchCooperativeKernel((void*)lsm_kernel, dim3(G), dim3(kLsmBlock), args,
                                               smem, c->stream),
                   "lsm kernel launch");
  if (st) return st;
  c->launches += 1;
  st = cuda_status(cudaMemcpyAsync(h + o_cnt, d + o_cnt, o_out - o_cnt + sizeof(double) * kMoments,
                                   cudaMemcpyDeviceToHost, c->stream),
                   "D2H lsm");
  if (!st) st = cuda_status(cudaStreamSynchronize(c->stream), "lsm kernel");
  if (st) return st;
  const int* flags = (const int*)(h + o_cnt);
  if (flags[2]) return set_error(PCF_ETIMEOUT, "LSM device wait gave up (code %d)", flags[2]);
  if (flags[3])
    return set_error(PCF_ESINGULAR, "Detereminant is not > 0 at %d exercise date(s)", flags[3]);
  const double* s = (const double*)(h + o_out);
  fill_amer_result(s, N, S0, E, r, sigma, T, payoff_fun, use_cv != 0, out);
  return PCF_OK;
}
