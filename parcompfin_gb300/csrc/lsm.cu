// Longstaff-Schwartz American pricing (the reference's mc_amer) on one GPU.
//
// Reference: src/mc_amer.cpp:5-114 (serial), src/mc_amer_omp.cpp:5-117, with
// pathsfinder() of include/common.h:168-208 and the 3x3 solve of
// include/common.h:98-141. The MPI build reduces the seven regression sums
// and the in-the-money count to rank 0 and broadcasts three coefficients per
// date (src/mc_amer_mpi.cpp:82-131). Here the same exchange runs between the
// CTAs of one launch, once per exercise date.
//
// Launch forms (the first three share one body, lsm_body):
//   cooperative  one contract per launch, at most one 512-thread block per
//                SM (pcf_mc_amer, and batch contracts too large for a
//                cluster). Blocks exchange their partial sums through global
//                memory and a bounded group barrier;
//   cluster      many contracts per launch, one thread-block cluster per
//                contract (pcf_plan_*). CTAs write their partial sums into
//                every peer's shared memory and signal the peer's mbarrier;
//   cooperative grid of clusters  one large contract: the cluster exchange,
//                then only the cluster leaders meet in global memory;
//   streaming    one contract whose per-block slice exceeds shared memory
//                (lsm_stream_kernel): per-path state in device memory.
// Phases:
//   forward   each thread generates its antithetic pairs (path p takes +z,
//             path p + H takes -z, as pathsfinder pairs them) and writes the
//             positive part of the signed moneyness, max(pf (S/E - 1), 0) at
//             dates m = 1..M, to an FP32 time-major path matrix in HBM
//             (row m-1; plus half at columns [0, Hp), minus half at
//             [Hp, 2Hp), Hp = H rounded up to 4), coalesced across the warp;
//   backward  for m = M-1..1 the block's slice of row m-1 (two contiguous
//             runs) arrives in shared memory by TMA bulk copy, issued two
//             dates ahead. Each thread updates the exercise decision of its
//             paths at date m and, in the same pass, adds date m-1's
//             regression sums in FP32, four consecutive paths per 16-byte
//             shared-memory load. A warp reduce-scatter leaves the
//             warp's eight sums in eight lanes; after one block barrier a
//             single warp adds the warp partials and then all CTAs' partials
//             in double-float, in a fixed order (every CTA gets the same
//             bits), solves the normal equations in double-float and
//             publishes the coefficients before a second block barrier;
//   final     discounted cash flows and the martingale control variate are
//             averaged over antithetic pairs and reduced with the
//             deterministic last-block finaliser (cooperative launch) or
//             through distributed shared memory (cluster launch).
// Per-path state stays in shared memory for the whole sweep: the cash flow
// discounted to time 0 (a date's regression target is that times the date's
// growth factor, which multiplies the date's three y sums once) and the
// exercise date (8 bits where M <= 255). The
// regression basis is {1, u, u^2} with u = pf (S - E)/E: the reference's S - E
// rescaled (and negated for a put), the same fitted values in exact
// arithmetic. Only paths in the money enter a regression or exercise, so the
// path matrix holds x = max(u, 0): a path is in the money where x > 0, its
// payoff is E x, and an out-of-the-money path adds exact zeros to the sums
// in x.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <vector>

#include <cooperative_groups.h>

#include "pcf_api_internal.h"
#include "pcf_device.cuh"
#include "pcf_math.h"

namespace cg = cooperative_groups;

namespace pcf {

namespace {

constexpr int kLsmBlock = 512;     // cooperative kernel: one block per SM
constexpr int kLsmCBlock = 512;    // cluster kernel: two CTAs per SM
constexpr int kRegSums = 8;      // n, u, u^2, u^3, u^4, y, y u, y u^2
constexpr int kMaxCluster = 16;  // CTAs per contract in a cluster launch

// How the CTAs of one contract exchange their per-date sums.
enum LsmMode : int {
  kCoop = 0,         // cooperative grid: global memory and a group barrier
  kCluster = 1,      // one thread-block cluster: distributed shared memory
  kCoopCluster = 2,  // cooperative grid of clusters: both, in two levels
};

struct LsmParams {
  float pf, nK, E, invE;  // payoff = max(pf S + nK, 0) = E max(u, 0)
  float a2, b2, l2SE;     // per-date log2 drift / vol, log2(S0 / E)
  float rf, sigf, dtf;    // r, sigma, T/M: the European price of the control variate
  int M, ref_exercise;
  long long H;            // antithetic pairs = N / 2
  long long Hp;           // H rounded up to a multiple of 4
  int pairs_per_block;    // PB, a multiple of 4
  int nblocks;            // blocks (cooperative) or CTAs of the cluster
  int cluster;            // hybrid launch: CTAs per cluster (nblocks is a multiple)
  uint32_t seed_lo, seed_hi, stream;
  unsigned wait_limit;       // group-barrier polls before giving up
  unsigned copy_wait_limit;  // mbarrier polls before giving up
  unsigned barrier_extra;    // test hook: arrivals the cooperative group barrier expects
                             // beyond the grid (it can then never complete); 0 otherwise
  float* paths;           // M rows of 2*Hp floats
  const float* dtab;      // exp(-r dt k), k = 0..M, then exp(+r dt k), k = 0..M
  double* partial;        // 2 x nblocks x kRegSums (cooperative)
  double* fpartial;       // nblocks x kMoments (cooperative)
  unsigned* barrier;
  unsigned* ticket;
  int* err;               // 1: a barrier wait gave up, 2: a bulk copy wait gave up,
                          // 4: the launch lacked its cluster shape (nothing computed)
  int* singular;          // dates whose normal equations had det <= 0
  double* out;            // kMoments sums
  float* gcf;             // streaming sweep: 2*Hp discounted cash flows (device memory)
  unsigned short* gtau;   // streaming sweep: 2*Hp exercise dates
  // Audit record (pcf_mc_amer_audit; NULL otherwise), written by block 0 /
  // every block for its own paths: per date d, {mode, c0, c1, c2} and the
  // eight regression sums as the solve saw them; per path its exercise date.
  float* dbg_coef;        // M x 4
  double* dbg_sums;       // M x kRegSums
  unsigned short* dbg_tau;  // N: plus half [0, H), minus half [H, 2H)
};

// Four consecutive floats of shared memory (16-byte aligned).
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

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

// Dynamic shared memory of one block: two copy mbarriers, the discount and
// growth tables, per-path state, and two path-slice buffers.
template <typename TauT>
struct LsmSmem {
  uint64_t* bar;  // 2 mbarriers, one per slice buffer
  float* dt;      // exp(-r dt k), k = 0..M
  float* edt;     // exp(+r dt k), k = 0..M
  float* cf;      // 2*PB cash flows, discounted to time 0
  TauT* tau;      // 2*PB exercise dates
  float* buf;     // 2 x 2*PB path slices, back to back
  int PB;
  __device__ __forceinline__ float* slice(int k) const { return buf + (size_t)k * 2 * PB; }
};

__host__ __device__ __forceinline__ size_t r16(size_t x) { return (x + 15) & ~(size_t)15; }

template <typename TauT>
__device__ __forceinline__ LsmSmem<TauT> carve(unsigned char* base, int PB, int M) {
  LsmSmem<TauT> s;
  size_t o = 0;
  s.bar = (uint64_t*)(base + o);
  o += 16;
  s.dt = (float*)(base + o);
  o += r16((size_t)(M + 1) * 4);
  s.edt = (float*)(base + o);
  o += r16((size_t)(M + 1) * 4);
  s.cf = (float*)(base + o);
  o += (size_t)2 * PB * 4;
  s.tau = (TauT*)(base + o);
  o += r16((size_t)2 * PB * sizeof(TauT));
  s.buf = (float*)(base + o);
  s.PB = PB;
  return s;
}

// Static shared memory of one block of NW warps: the exchange of regression
// sums.
template <int NW>
struct LsmShared {
  float wpart[NW][kRegSums];                     // per-warp FP32 sums
  alignas(16) DF xin[2][kMaxCluster][kRegSums];  // cluster: every CTA's totals, by date parity
  alignas(16) DF ctot[kRegSums];                 // this CTA's totals
  uint64_t xbar[2];                              // cluster: bytes of the CTAs' totals
  DF tdf[kRegSums];                              // the contract's sums, scaled
  DF cof[8];                                     // adjugate of the normal matrix
  float coef[3];
  int mode;  // 0 skip the date, 1 few in-the-money paths, 2 regression
  int fail;  // a wait gave up
  DF sh[NW * kMoments];
  DF fin[kMoments];
};

// Bulk-copies the block's slice of row r (pairs [p0, p0 + nbr)) to dst:
// plus half to dst[0..nbr), minus half to dst[PB..PB + nbr).
__device__ __forceinline__ void issue_row(const LsmParams& P, int r, long long p0, int nbr, int PB,
                                          float* dst, uint64_t* bar) {
  const float* row = P.paths + (size_t)r * 2 * P.Hp;
  const uint32_t bytes = (uint32_t)nbr * 4u;
  mbar_arrive_expect_tx(bar, 2u * bytes);
  bulk_g2s(dst, row + p0, bytes, bar);
  bulk_g2s(dst + PB, row + P.Hp + p0, bytes, bar);
}

// Adds one path's terms to the regression sums of a date if the path is in
// the money there (src/mc_amer.cpp:57-66 regresses on in-the-money paths
// only): x = max(u, 0) with u = pf (S - E)/E, as the path matrix holds it,
// and the cash flow discounted to time 0, y = cfd. The regression target is
// y times the date's growth factor; the factor is common to every path, so
// regress_date applies it once to the three y sums. A path out of the money
// has x = 0, so the terms in x add exact zeros without a select; only the
// count and the y sum test it.
__device__ __forceinline__ void reg_accumulate(float x, float cfd, float (&acc)[kRegSums]) {
  const bool itm = x > 0.f;
  const float x2 = x * x;
  acc[0] += itm ? 1.f : 0.f;
  acc[1] += x;
  acc[2] += x2;
  acc[3] = fmaf(x2, x, acc[3]);
  acc[4] = fmaf(x2, x2, acc[4]);
  acc[5] += itm ? cfd : 0.f;
  acc[6] = fmaf(cfd, x, acc[6]);
  acc[7] = fmaf(cfd, x2, acc[7]);
}

// Reduce-scatter of eight FP32 sums over a warp: each step sends half of the
// lane's values to the partner lane and keeps the half the partner sends.
// Afterwards the four lanes l with ((l >> 2) & 7) == q hold the warp total of
// sum q. FP32 addition is commutative, so those lanes hold the same bits.
__device__ __forceinline__ float warp_scatter8(const float (&a)[kRegSums]) {
  const int lane = threadIdx.x & 31;
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  float v4[4], v2[2];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float send = b4 ? a[i] : a[i + 4];
    const float keep = b4 ? a[i + 4] : a[i];
    v4[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const float send = b3 ? v4[i] : v4[i + 2];
    const float keep = b3 ? v4[i + 2] : v4[i];
    v2[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  float v = (b2 ? v2[1] : v2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? v2[0] : v2[1], 4);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

// Cooperative launch: arrival at the group barrier by one thread, after the
// block's partials were stored and fenced. `counter` only grows: arrival
// number a (0-based) waits until the count reaches (a/G + 1)*G. Bounded: after
// `limit` polls (or once another block reported a failure) it raises *err and
// returns false.
__device__ __forceinline__ bool group_arrive_wait(unsigned* counter, unsigned G, int* err,
                                                  unsigned limit) {
  const unsigned a = atomicAdd(counter, 1u);
  const unsigned target = (a / G + 1u) * G;
  for (unsigned polls = 0;; ++polls) {
    const unsigned c = *((volatile unsigned*)counter);
    if ((int)(c - target) >= 0) break;
    if (*((volatile int*)err) != 0 || polls > limit) {
      atomicExch(err, 1);
      return false;
    }
    __nanosleep(32);
  }
  __threadfence();
  return true;
}

// Date d's regression, run by warp 0 between the two block barriers: the
// block's total of each sum, the exchange of block totals, the contract's
// sums in FP64 and the solve. Leaves the mode and coefficients in X.
template <int MODE, int NW>
__device__ __forceinline__ void regress_date(const LsmParams& P, LsmShared<NW>& X, int d, int b,
                                             int rank, uint32_t& xph, uint32_t& xcount,
                                             float growth) {
  const int lane = threadIdx.x & 31;
  const int q = lane & 7;
  // Block total of sum q: lane groups l>>3 = 0..3 each add four warps' sums,
  // then two shuffle steps combine the groups. Lanes 0..7 hold the totals.
  DF v = DF{X.wpart[lane >> 3][q], 0.f};
#pragma unroll
  for (int w = (lane >> 3) + 4; w < NW; w += 4) v = df_add_f(v, X.wpart[w][q]);
  v = df_add(v, shfl_xor_df(v, 8));
  v = df_add(v, shfl_xor_df(v, 16));
  const int slot = d & 1;
  const int G = P.nblocks;
  DF g{0.f, 0.f};
  if (MODE != kCoop) {
    // Every CTA stores its eight totals into xin[slot][rank] of every CTA with
    // st.async; each store counts its bytes against that CTA's xbar[slot],
    // which the CTA's own lane 0 arms for G x 64 bytes (a store may land
    // before the arming: the phase cannot complete before the arming's
    // arrival). Slot reuse is safe: a CTA sends date d-2 only after its wait
    // for date d-1, which needs every peer's date d-1 totals, which each peer
    // sends after it has read its date d slot.
    const int CL = MODE == kCluster ? G : P.cluster;
    if (lane == 0) mbar_arrive_expect_tx(&X.xbar[slot], (uint32_t)(CL * kRegSums * sizeof(DF)));
    if (lane < kRegSums) X.ctot[lane] = v;
    __syncwarp();
    if (lane < CL) {
      const float4* src = reinterpret_cast<const float4*>(X.ctot);
      const uint32_t dst = cluster_map(&X.xin[slot][rank][0], (uint32_t)lane);
      const uint32_t bar = cluster_map(&X.xbar[slot], (uint32_t)lane);
#pragma unroll
      for (int j = 0; j < kRegSums * 2 / 4; ++j) st_async_v4(dst + 16u * j, src[j], bar);
    }
    if (!mbar_wait(&X.xbar[slot], (xph >> slot) & 1u, P.copy_wait_limit)) {
      X.fail = 1;
      atomicExch(P.err, 1);
    }
    xph ^= 1u << slot;
    for (int r = lane >> 3; r < CL; r += 4) g = df_add(g, X.xin[slot][r][q]);
    if (MODE == kCoopCluster) {
      // Second level: every cluster now holds its total (the same bits in each
      // of its CTAs); rank 0 publishes it, the clusters meet at a counter that
      // grows by one arrival per cluster and date, and every CTA sums the
      // cluster totals in cluster order.
      g = df_add(g, shfl_xor_df(g, 8));
      g = df_add(g, shfl_xor_df(g, 16));
      const int ncl = G / CL, cid = b / CL;
      float2* part = (float2*)P.partial + (size_t)slot * ncl * kRegSums;
      if (rank == 0 && lane < kRegSums) {
        part[(size_t)cid * kRegSums + lane] = make_float2(g.hi, g.lo);
        __threadfence();
      }
      __syncwarp();
      xcount += 1;
      int ok = 1;
      if (lane == 0) {
        if (rank == 0) atomicAdd(P.barrier, 1u);
        const unsigned target = xcount * (unsigned)ncl;
        for (unsigned polls = 0;; ++polls) {
          const unsigned cnt = *((volatile unsigned*)P.barrier);
          if ((int)(cnt - target) >= 0) break;
          if (*((volatile int*)P.err) != 0 || polls > P.wait_limit) {
            atomicExch(P.err, 1);
            ok = 0;
            break;
          }
          __nanosleep(32);
        }
        __threadfence();
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok && lane == 0) X.fail = 1;
      g = DF{0.f, 0.f};
#pragma unroll 4
      for (int cc = lane >> 3; cc < ncl; cc += 4) {
        const float2 p = __ldcg(part + (size_t)cc * kRegSums + q);
        g = df_add(g, DF{p.x, p.y});
      }
    }
  } else {
    float2* part = (float2*)P.partial + (size_t)slot * G * kRegSums;
    if (lane < kRegSums) {
      part[(size_t)b * kRegSums + lane] = make_float2(v.hi, v.lo);
      __threadfence();
    }
    __syncwarp();
    int ok = 1;
    if (lane == 0)
      ok = group_arrive_wait(P.barrier, (unsigned)G + P.barrier_extra, P.err, P.wait_limit);
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok && lane == 0) X.fail = 1;
#pragma unroll 4
    for (int bb = lane >> 3; bb < G; bb += 4) {
      const float2 p = __ldcg(part + (size_t)bb * kRegSums + q);
      g = df_add(g, DF{p.x, p.y});
    }
  }
  g = df_add(g, shfl_xor_df(g, 8));
  g = df_add(g, shfl_xor_df(g, 16));  // lanes 0..7: the contract's sum q = lane
  if (q >= 5) g = df_mul(g, DF{growth, 0.f});  // y sums: cash flows grown to date d
  if (P.dbg_sums && b == 0 && lane < kRegSums) P.dbg_sums[(size_t)d * kRegSums + lane] = df_value(g);
  // include/common.h:98-141 solves the normal equations by the adjugate over
  // the determinant, then a mat-vec product. The normal matrix of the basis
  // {1, u, u^2} is the symmetric Hankel matrix [[a0,a1,a2],[a1,a2,a3],
  // [a2,a3,a4]], so its adjugate has six distinct cofactors:
  //   c00 = a2 a4 - a3 a3   c01 = a2 a3 - a1 a4   c02 = a1 a3 - a2 a2
  //   c11 = a0 a4 - a2 a2   c12 = a1 a2 - a0 a3   c22 = a0 a2 - a1 a1
  // one per lane. Lanes 0..2 then form the numerators adj (a5, a6, a7) and
  // lane 3 the determinant a0 c00 + a1 c01 + a2 c02, each a three-term dot
  // product. The arithmetic is double-float (~48 significant bits, enough for
  // the cancellation in the cofactors) instead of FP64, which is slow on
  // GB300 and sits on every date's critical path; the sums are first scaled
  // by a power of two near 1/a0 (exact, and it leaves the solution
  // unchanged) to keep every product well inside the FP32 exponent range.
  // The coefficients are used in FP32, so the final division is FP32.
  const float n = __shfl_sync(0xffffffffu, g.hi, 0);  // in-the-money paths (an exact integer)
  if (n >= 1.f) {
    const int e = (__float_as_int(n) >> 23) & 255;  // biased exponent of n, in [127, 254]
    const float s = __int_as_float((254 - e) << 23);  // 2^-(e - 127), exact
    g = DF{g.hi * s, g.lo * s};
  }
  if (lane < kRegSums) X.tdf[lane] = g;
  __syncwarp();
  const DF* a = X.tdf;
  DF cof{0.f, 0.f};
  if (lane < 6) {
    const int sh = 4 * lane;  // operand indices of cofactor `lane`, one nibble per lane
    cof = df_add(df_mul(a[(0x010122 >> sh) & 15], a[(0x224334 >> sh) & 15]),
                 df_neg(df_mul(a[(0x102213 >> sh) & 15], a[(0x132243 >> sh) & 15])));
    X.cof[lane] = cof;
  }
  __syncwarp();
  DF dot{0.f, 0.f};
  if (lane < 4) {
    const int sh = 4 * lane;  // adjugate row `lane` (row 0 again for lane 3)
    const DF* y = lane < 3 ? a + 5 : a;
    dot = df_add(df_add(df_mul(X.cof[(0x0210 >> sh) & 15], y[0]),
                        df_mul(X.cof[(0x1431 >> sh) & 15], y[1])),
                 df_mul(X.cof[(0x2542 >> sh) & 15], y[2]));
  }
  const DF n1 = shfl_df(dot, 1), n2 = shfl_df(dot, 2), det = shfl_df(dot, 3);
  if (lane == 0) {
    int mode = 2;
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
    if (n == 0.f) {
      mode = 0;
    } else if (n <= 2.f) {
      mode = 1;
    } else if (!(det.hi > 0.f) || !(det.hi < INFINITY)) {  // include/common.h:115-117
      mode = 0;
      if (b == 0) atomicAdd(P.singular, 1);
    } else {
      const float r = 1.f / det.hi;
      c0 = (dot.hi + dot.lo) * r;
      c1 = (n1.hi + n1.lo) * r;
      c2 = (n2.hi + n2.lo) * r;
    }
    X.mode = mode;
    X.coef[0] = c0;
    X.coef[1] = c1;
    X.coef[2] = c2;
    if (P.dbg_coef && b == 0) {
      float* o = P.dbg_coef + (size_t)d * 4;
      o[0] = (float)mode;
      o[1] = c0;
      o[2] = c1;
      o[3] = c2;
    }
  }
}

// Antithetic pair p over the contract's M dates (path p takes +z, path p + H
// takes -z, as pathsfinder pairs them): writes the positive part of the
// signed moneyness, x = max(u, 0) with u = pf (S/E - 1), of both paths to the
// path matrix, one row per date, and returns x at date M of the plus and the
// minus path. Only x enters the sweep: a path is in the money where x > 0,
// and its payoff is E x. Date m0 + l + 1 takes
// lane l of Philox block m0 / 4: whole blocks first, without per-date checks,
// then the last 1..3 dates.
__device__ __forceinline__ float2 forward_pair(const LsmParams& P, const RngKey& key,
                                               long long p) {
  // The parameters in registers: the stores below go through generic
  // pointers, which the compiler cannot tell apart from P.
  const long long Hp = P.Hp;
  const size_t stride = (size_t)2 * Hp;  // floats per row
  const float b2 = P.b2, nb2 = -P.b2, a2 = P.a2, pf = P.pf;
  const int M = P.M;
  float Lp = P.l2SE, Lm = P.l2SE, Up = 0.f, Um = 0.f;  // log2(S/E)
  float* row = P.paths + p;
  auto step = [&](float z) {
    Lp += fmaf(b2, z, a2);
    Lm += fmaf(nb2, z, a2);
    Up = fmaxf(fmaf(pf, ex2_approx(Lp), -pf), 0.f);  // max(pf (S/E - 1), 0)
    Um = fmaxf(fmaf(pf, ex2_approx(Lm), -pf), 0.f);
    row[0] = Up;
    row[Hp] = Um;
    row += stride;
  };
  const int Mfull = M & ~3;
  for (int m0 = 0; m0 < Mfull; m0 += 4) {
    const float4 z4 = normals4(draw_words(key, (uint64_t)p, (uint32_t)(m0 >> 2)));
    step(z4.x);
    step(z4.y);
    step(z4.z);
    step(z4.w);
  }
  if (Mfull < M) {
    const float4 z4 = normals4(draw_words(key, (uint64_t)p, (uint32_t)(Mfull >> 2)));
    step(z4.x);
    if (Mfull + 1 < M) step(z4.y);
    if (Mfull + 2 < M) step(z4.z);
  }
  return make_float2(Up, Um);
}

// The control-variate sample of one path with exercise date tau, cash flow
// cfd (discounted to 0) and moneyness uM at date M. Martingale control
// variate: g = e^{-r tau} P_E(S_tau, T - tau), the discounted European price
// at the path's exercise time; the discounted European price is a martingale,
// so E[g] = P_E(S0, T) for any stopping time. S_tau is E + pf*cf where the
// path exercised before T; a path held to T (tau = M) contributes its
// discounted payoff at T, which is cfd.
__device__ __forceinline__ float cv_sample(const LsmParams& P, const float* dt, const float* edt,
                                           int tau, float cfd, float uM) {
  const int M = P.M;
  if (P.ref_exercise) {
    // The reference's exercise value does not identify S_tau: use the
    // discounted European payoff at T (mean: the same P_E(S0, T)).
    return dt[M] * (P.E * fmaxf(uM, 0.f));
  }
  if (tau == M) return cfd;  // the discounted European payoff at T
  const float St = P.E + P.pf * (cfd * edt[tau]);
  return dt[tau] * european_price(P, St, (float)(M - tau) * P.dtf);
}

// One contract's forward pass, backward sweep and final moments, executed by
// block `b` of the contract's `P.nblocks` blocks. Every wait is bounded. A
// cooperative block that gave up leaves after its in-flight copies landed; a
// cluster CTA records the failure and keeps taking part in every exchange and
// cluster barrier (a hardware barrier has no timeout), so no CTA leaves early.
template <int MODE, typename TauT, int BS>
__device__ void lsm_body(const LsmParams& P, int b, int rank) {
  constexpr bool CLUSTER = MODE == kCluster;  // one cluster per contract
  constexpr bool DSMEM = MODE != kCoop;       // CTAs exchange through cluster shared memory
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int PB = P.pairs_per_block;
  const int M = P.M;
  const LsmSmem<TauT> S = carve<TauT>(smem_raw, PB, M);
  __shared__ LsmShared<BS / 32> X;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

  const long long p0 = (long long)b * PB;
  const int nb = (int)max(0LL, min((long long)PB, P.H - p0));  // pairs in this block
  const int nbr = (nb + 3) & ~3;                                // bulk-copy width
  const int nq = nbr >> 2;                                      // four-path groups
  for (int k = threadIdx.x; k <= M; k += BS) {
    S.dt[k] = P.dtab[k];
    S.edt[k] = P.dtab[M + 1 + k];
  }
  if (threadIdx.x == 0) {
    mbar_init(&S.bar[0], 1);
    mbar_init(&S.bar[1], 1);
    if (DSMEM) {
      mbar_init(&X.xbar[0], 1);  // armed by this CTA's lane 0 once per date
      mbar_init(&X.xbar[1], 1);
    }
    fence_mbar_init();
    X.fail = 0;
  }

  // ---- forward: generate and store paths ----
  const RngKey key{P.seed_lo, P.seed_hi, P.stream, TAG_AMER};
  const float EdM = P.E * P.dtab[M];  // payoff at T = E max(u, 0), discounted
  const size_t stride = (size_t)2 * P.Hp;  // floats per row
#pragma unroll 2
  for (int i = threadIdx.x; i < nb; i += BS) {
    const float2 uM = forward_pair(P, key, p0 + i);
    S.cf[i] = fmaxf(uM.x, 0.f) * EdM;
    S.cf[PB + i] = fmaxf(uM.y, 0.f) * EdM;
    S.tau[i] = (TauT)M;
    S.tau[PB + i] = (TauT)M;
  }
  // Columns [nb, nbr) pad the last block's bulk copies to 16 bytes: u = 0 and
  // cf = 0 there, so the four-path steps below see paths out of the money
  // that never exercise and add nothing.
  for (int i = nb + threadIdx.x; i < nbr; i += BS) {
    for (int m = 0; m < M; ++m) {
      P.paths[(size_t)m * stride + p0 + i] = 0.f;
      P.paths[(size_t)m * stride + P.Hp + p0 + i] = 0.f;
    }
    S.cf[i] = 0.f;
    S.cf[PB + i] = 0.f;
  }
  // The bulk copies below read what this block's threads just stored; the
  // cluster barrier also publishes the exchange mbarriers to the peers.
  fence_proxy_async_global();
  if (DSMEM) cg::this_cluster().sync();
  else __syncthreads();

  // Buffer schedule: date d's slice sits in buf[(M - 1 - d) & 1]. Thread 32
  // issues every copy; every thread waits on the copy it is about to read.
  // `pend` (copies issued, not yet waited) and `ph` (mbarrier parities) evolve
  // the same way in every thread.
  uint32_t ph = 0, pend = 0, xph = 0, xcount = 0;
  if (nbr > 0) {
    if (threadIdx.x == 32) {
      issue_row(P, M - 2, p0, nbr, PB, S.slice(0), &S.bar[0]);                 // date M-1
      if (M >= 3) issue_row(P, M - 3, p0, nbr, PB, S.slice(1), &S.bar[1]);  // date M-2
    }
    pend = M >= 3 ? 3u : 1u;
  }
  auto wait_copy = [&](int k) {
    if (!((pend >> k) & 1u)) return;
    if (!mbar_wait(&S.bar[k], (ph >> k) & 1u, P.copy_wait_limit)) {
      X.fail = 1;
      atomicExch(P.err, 2);
    }
    ph ^= 1u << k;
    pend &= ~(1u << k);
  };
  // Regression for date d from each thread's sums; then thread 32 issues the
  // copy of `next_row` into buf[next_k] (free: every thread has passed the
  // first barrier, so it is done reading that buffer).
  auto regress = [&](const float (&acc)[kRegSums], int d, int next_row, int next_k) {
    const float v = warp_scatter8(acc);
    if ((lane & 3) == 0) X.wpart[wid][lane >> 2] = v;
    __syncthreads();
    if (next_row >= 0 && nbr > 0) {
      if (threadIdx.x == 32) issue_row(P, next_row, p0, nbr, PB, S.slice(next_k), &S.bar[next_k]);
      pend |= 1u << next_k;
    }
    if (wid == 0) regress_date<MODE, BS / 32>(P, X, d, b, rank, xph, xcount, S.edt[d]);
    __syncthreads();
  };

  // Sums for date M-1 (the only date without a preceding update pass).
  {
    wait_copy(0);
    float acc[kRegSums];
#pragma unroll
    for (int q = 0; q < kRegSums; ++q) acc[q] = 0.f;
    const float* sl = S.slice(0);
    for (int j = threadIdx.x; j < nq; j += BS) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int s = h * PB + 4 * j;
        const float4 u = ld4(sl + s), c = ld4(S.cf + s);
        reg_accumulate(u.x, c.x, acc);
        reg_accumulate(u.y, c.y, acc);
        reg_accumulate(u.z, c.z, acc);
        reg_accumulate(u.w, c.w, acc);
      }
    }
    regress(acc, M - 1, -1, 0);
  }

  // Date m: update with date m's coefficients, fused with the sums of date m-1.
  bool failed = !DSMEM && X.fail;
  for (int m = M - 1; m >= 1 && !failed; --m) {
    const int k = (M - 1 - m) & 1;
    const bool has_next = m > 1;
    if (has_next) wait_copy(k ^ 1);
    const int mode = X.mode;
    const float c0 = X.coef[0], c1 = X.coef[1], c2 = X.coef[2];
    const float dm = S.dt[m], em = S.edt[m];
    const float* cur = S.slice(k);
    const float* nxt = S.slice(k ^ 1);
    float acc[kRegSums];
#pragma unroll
    for (int q = 0; q < kRegSums; ++q) acc[q] = 0.f;
    const float E = P.E, nK = P.nK;
    // One pass over the block's paths, compiled once per case (the date's
    // mode MD, the reference's exercise rule RX, a following date NX), so
    // the loop carries no per-path test of them.
    auto sweep = [&](auto md_c, auto rx_c, auto nx_c) {
      constexpr int MD = decltype(md_c)::value;
      constexpr bool RX = decltype(rx_c)::value;
      constexpr bool NX = decltype(nx_c)::value;
      // Exercise decision at date m (src/mc_amer.cpp:73-106) for one path:
      // exercise where the path is in the money and the payoff beats the
      // continuation value; the cash flow becomes the payoff discounted to 0.
      auto decide = [&](float u, float& cfd, int s) {  // u: the stored max(u, 0)
        float cont, ex = u * E;  // the payoff E max(u, 0)
        if (MD == 1) {
          cont = cfd * em;
        } else {
          cont = fmaf(fmaf(c2, u, c1), u, c0);
          // src/mc_amer.cpp:100: the reference exercises at payoff(S - E, E),
          // max(pf (S - 2E), 0) = max(E u - pf E, 0).
          if (RX) ex = fmaxf(fmaf(E, u, nK), 0.f);
        }
        if (u > 0.f && ex > cont) {
          cfd = ex * dm;
          S.tau[s] = (TauT)m;
        }
      };
#pragma unroll 2
      for (int j = threadIdx.x; j < nq; j += BS) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int s = h * PB + 4 * j;
          float4 c = ld4(S.cf + s);
          // Date m-1's slice is not written by this pass: load it before the
          // exercise update's stores, so its latency overlaps the update.
          const float4 un = NX ? ld4(nxt + s) : make_float4(0.f, 0.f, 0.f, 0.f);
          if (MD != 0) {
            const float4 u = ld4(cur + s);
            decide(u.x, c.x, s);
            decide(u.y, c.y, s + 1);
            decide(u.z, c.z, s + 2);
            decide(u.w, c.w, s + 3);
            st4(S.cf + s, c);
          }
          if (NX) {
            const float4 u = un;
            reg_accumulate(u.x, c.x, acc);
            reg_accumulate(u.y, c.y, acc);
            reg_accumulate(u.z, c.z, acc);
            reg_accumulate(u.w, c.w, acc);
          }
        }
      }
    };
    using Md0 = std::integral_constant<int, 0>;
    using Md1 = std::integral_constant<int, 1>;
    using Md2 = std::integral_constant<int, 2>;
    using Yes = std::true_type;
    using No = std::false_type;
    const bool refx = P.ref_exercise != 0;
    if (has_next) {
      if (mode == 0) sweep(Md0{}, No{}, Yes{});
      else if (mode == 1) sweep(Md1{}, No{}, Yes{});
      else if (refx) sweep(Md2{}, Yes{}, Yes{});
      else sweep(Md2{}, No{}, Yes{});
    } else {
      if (mode == 1) sweep(Md1{}, No{}, No{});
      else if (mode == 2 && refx) sweep(Md2{}, Yes{}, No{});
      else if (mode == 2) sweep(Md2{}, No{}, No{});
    }
    if (!has_next) break;
    regress(acc, m - 1, m - 2 >= 1 ? m - 3 : -1, k);
    failed = !DSMEM && X.fail;
  }
  __syncthreads();
  if (failed) {
    // Let any bulk copy this block issued land before the block exits.
    if (threadIdx.x == 32)
      for (int k = 0; k < 2; ++k)
        if ((pend >> k) & 1u) mbar_wait(&S.bar[k], (ph >> k) & 1u, P.copy_wait_limit);
    return;
  }
  if (P.dbg_tau)
    for (int i = threadIdx.x; i < nb; i += BS) {
      P.dbg_tau[p0 + i] = (unsigned short)S.tau[i];
      P.dbg_tau[P.H + p0 + i] = (unsigned short)S.tau[PB + i];
    }

  // ---- discounted cash flows and the control variate, per antithetic pair ----
  // Moments are taken over pair means: the two paths of a pair share their
  // draws, so the pair, not the path, is the independent sample.
  const float* last = P.paths + (size_t)(M - 1) * 2 * P.Hp;
  KSum sy, syy, sg, sgg, syg;
  for (int i = threadIdx.x; i < nb; i += BS) {
    float y2 = 0.f, g2 = 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int s = h * PB + i;
      const float cfd = S.cf[s];  // cash flow discounted to time 0
      y2 += cfd;
      g2 += cv_sample(P, S.dt, S.edt, S.tau[s], cfd,
                      P.ref_exercise ? last[h * P.Hp + p0 + i] : 0.f);
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
  block_sum_df<kMoments>(v, X.sh, tot);
  if (CLUSTER) {
    if (threadIdx.x == 0)
      for (int q = 0; q < kMoments; ++q) X.fin[q] = tot[q];
    cg::this_cluster().sync();
    if (b == 0 && threadIdx.x == 0) {
      DF t[kMoments];
      for (int q = 0; q < kMoments; ++q) t[q] = DF{0.f, 0.f};
      for (int r = 0; r < P.nblocks; ++r) {
        const DF* rf = cg::this_cluster().map_shared_rank(&X.fin[0], r);
        for (int q = 0; q < kMoments; ++q) t[q] = df_add(t[q], rf[q]);
      }
      for (int q = 0; q < kMoments; ++q) P.out[q] = df_value(t[q]);
    }
    cg::this_cluster().sync();  // rank 0 has read every CTA's shared memory
  } else {
    grid_finalize_df<kMoments>(tot, (float2*)P.fpartial, P.ticket, P.out, P.nblocks, b);
    if (DSMEM) cg::this_cluster().sync();  // no CTA leaves while a peer may address it
  }
}

__global__ void __launch_bounds__(kLsmBlock, 1) lsm_kernel(LsmParams P) {
  lsm_body<kCoop, unsigned short, kLsmBlock>(P, blockIdx.x, 0);
}

// One large contract on a cooperative grid of clusters (P.cluster CTAs each):
// per date the CTAs of a cluster exchange through distributed shared memory,
// and only the clusters' leaders meet in global memory.
__global__ void __launch_bounds__(kLsmBlock, 1) lsm_coop_cluster_kernel(LsmParams P) {
  // The exchange addresses P.cluster peers: a launch without that cluster
  // shape stops here with an error instead of addressing absent CTAs.
  if (cg::this_cluster().num_blocks() != (unsigned)P.cluster) {
    if (threadIdx.x == 0) atomicExch(P.err, 4);
    return;
  }
  lsm_body<kCoopCluster, unsigned short, kLsmBlock>(P, blockIdx.x,
                                                    (int)cg::this_cluster().block_rank());
}

// Streaming sweep for a contract whose per-block slice does not fit in
// shared memory (about 2.8e6 paths and more on 152 SMs): the same algorithm
// as lsm_body's cooperative form, with the cash flows and exercise dates in
// device memory (P.gcf, P.gtau, laid out like a path-matrix row) and the
// path rows read straight from it, four paths per 16-byte load. A date then
// moves 16 bytes per path (date m and m-1, the cash flow in and out) instead
// of 4; the sweep stays bandwidth-bound at any N.
__global__ void __launch_bounds__(kLsmBlock, 1) lsm_stream_kernel(LsmParams P) {
  constexpr int BS = kLsmBlock, NW = BS / 32;
  __shared__ LsmShared<NW> X;
  extern __shared__ __align__(16) float stab[];  // dt[M+1] | edt[M+1]
  const int b = blockIdx.x, M = P.M;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float* dt = stab;
  float* edt = stab + (M + 1);
  const long long PB = P.pairs_per_block, Hp = P.Hp;
  const long long p0 = (long long)b * PB;
  const long long nb = max(0LL, min(PB, P.H - p0));
  const long long nbr = (nb + 3) & ~3LL;
  const long long nq = nbr >> 2;
  for (int k = threadIdx.x; k <= M; k += BS) {
    dt[k] = P.dtab[k];
    edt[k] = P.dtab[M + 1 + k];
  }
  if (threadIdx.x == 0) X.fail = 0;

  // ---- forward: the whole-path loop of lsm_body ----
  const RngKey key{P.seed_lo, P.seed_hi, P.stream, TAG_AMER};
  const float EdM = P.E * P.dtab[M];
  const size_t stride = (size_t)2 * Hp;
  for (long long i = threadIdx.x; i < nb; i += BS) {
    const long long p = p0 + i;
    const float2 uM = forward_pair(P, key, p);
    P.gcf[p] = fmaxf(uM.x, 0.f) * EdM;
    P.gcf[Hp + p] = fmaxf(uM.y, 0.f) * EdM;
    P.gtau[p] = (unsigned short)M;
    P.gtau[Hp + p] = (unsigned short)M;
  }
  for (long long i = nb + threadIdx.x; i < nbr; i += BS) {  // padding: out of the money
    for (int m = 0; m < M; ++m) {
      P.paths[(size_t)m * stride + p0 + i] = 0.f;
      P.paths[(size_t)m * stride + Hp + p0 + i] = 0.f;
    }
    P.gcf[p0 + i] = 0.f;
    P.gcf[Hp + p0 + i] = 0.f;
  }
  __syncthreads();  // every path of the block is read below by another thread

  uint32_t xph = 0, xcount = 0;
  auto regress = [&](const float (&acc)[kRegSums], int d) {
    const float v = warp_scatter8(acc);
    if ((lane & 3) == 0) X.wpart[wid][lane >> 2] = v;
    __syncthreads();
    if (wid == 0) regress_date<kCoop, NW>(P, X, d, b, 0, xph, xcount, edt[d]);
    __syncthreads();
  };
  {
    float acc[kRegSums];
#pragma unroll
    for (int q = 0; q < kRegSums; ++q) acc[q] = 0.f;
    const float* rowd = P.paths + (size_t)(M - 2) * stride + p0;  // date M-1
    for (long long j = threadIdx.x; j < nq; j += BS) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const long long s = h * Hp + 4 * j;
        const float4 u = __ldcs(reinterpret_cast<const float4*>(rowd + s));
        const float4 c = *reinterpret_cast<const float4*>(P.gcf + p0 + s);
        reg_accumulate(u.x, c.x, acc);
        reg_accumulate(u.y, c.y, acc);
        reg_accumulate(u.z, c.z, acc);
        reg_accumulate(u.w, c.w, acc);
      }
    }
    regress(acc, M - 1);
  }
  bool failed = X.fail;
  for (int m = M - 1; m >= 1 && !failed; --m) {
    const bool has_next = m > 1;
    const int mode = X.mode;
    const float c0 = X.coef[0], c1 = X.coef[1], c2 = X.coef[2];
    const float dm = dt[m], em = edt[m];
    const float* cur = P.paths + (size_t)(m - 1) * stride + p0;  // date m is row m-1
    const float* nxt = has_next ? cur - stride : cur;
    float acc[kRegSums];
#pragma unroll
    for (int q = 0; q < kRegSums; ++q) acc[q] = 0.f;
    auto decide = [&](float u, float& cfd, long long s) {
      float cont, ex = u * P.E;
      if (mode == 1) {
        cont = cfd * em;
      } else {
        cont = fmaf(fmaf(c2, u, c1), u, c0);
        if (P.ref_exercise) ex = fmaxf(fmaf(P.E, u, P.nK), 0.f);  // src/mc_amer.cpp:100
      }
      if (u > 0.f && ex > cont) {
        cfd = ex * dm;
        P.gtau[p0 + s] = (unsigned short)m;
      }
    };
#pragma unroll 2
    for (long long j = threadIdx.x; j < nq; j += BS) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const long long s = h * Hp + 4 * j;
        float4* cp = reinterpret_cast<float4*>(P.gcf + p0 + s);
        float4 c = *cp;
        if (mode != 0) {
          const float4 u = __ldcs(reinterpret_cast<const float4*>(cur + s));
          decide(u.x, c.x, s);
          decide(u.y, c.y, s + 1);
          decide(u.z, c.z, s + 2);
          decide(u.w, c.w, s + 3);
          *cp = c;
        }
        if (has_next) {
          const float4 u = *reinterpret_cast<const float4*>(nxt + s);
          reg_accumulate(u.x, c.x, acc);
          reg_accumulate(u.y, c.y, acc);
          reg_accumulate(u.z, c.z, acc);
          reg_accumulate(u.w, c.w, acc);
        }
      }
    }
    if (!has_next) break;
    regress(acc, m - 1);
    failed = X.fail;
  }
  __syncthreads();
  if (failed) return;
  if (P.dbg_tau)
    for (long long i = threadIdx.x; i < nb; i += BS) {
      P.dbg_tau[p0 + i] = P.gtau[p0 + i];
      P.dbg_tau[P.H + p0 + i] = P.gtau[Hp + p0 + i];
    }

  // ---- final moments over pair means (as lsm_body) ----
  const float* last = P.paths + (size_t)(M - 1) * stride;
  KSum sy, syy, sg, sgg, syg;
  for (long long i = threadIdx.x; i < nb; i += BS) {
    float y2 = 0.f, g2 = 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long s = h * Hp + p0 + i;
      const float cfd = P.gcf[s];
      y2 += cfd;
      g2 += cv_sample(P, dt, edt, P.gtau[s], cfd, P.ref_exercise ? last[s] : 0.f);
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
  block_sum_df<kMoments>(v, X.sh, tot);
  grid_finalize_df<kMoments>(tot, (float2*)P.fpartial, P.ticket, P.out, P.nblocks, b);
}

// Many contracts in one launch, one thread-block cluster per contract
// (cluster size = the contracts' common CTA count). Two CTAs per SM: while
// one runs its per-date exchange and solve, the other's paths keep the SM
// busy.
template <typename TauT>
__global__ void __launch_bounds__(kLsmCBlock, 2)
    lsm_cluster_kernel(const LsmParams* __restrict__ cs, int C) {
  __shared__ LsmParams sP;  // the contract's parameters, read from shared memory
  const unsigned rank = cg::this_cluster().block_rank();
  const unsigned CL = cg::this_cluster().num_blocks();
  // Every contract of the launch has cs[0].nblocks CTAs, one cluster each; a
  // launch of another shape stops with an error instead of mixing contracts.
  if (CL != (unsigned)cs[0].nblocks || gridDim.x != (unsigned)C * CL) {
    if (threadIdx.x == 0 && blockIdx.x < (unsigned)C) atomicExch(cs[blockIdx.x].err, 4);
    return;
  }
  const int c = (int)(blockIdx.x / CL);
  if (threadIdx.x == 0) sP = cs[c];
  __syncthreads();
  lsm_body<kCluster, TauT, kLsmCBlock>(sP, (int)rank, (int)rank);
}

// Dynamic shared memory of one block (the carve above).
size_t lsm_smem(int PB, int M, size_t tau_bytes) {
  return 16 + 2 * r16((size_t)(M + 1) * 4) + (size_t)2 * PB * 4 +
         r16((size_t)2 * PB * tau_bytes) + (size_t)2 * 2 * PB * 4;
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
  P.l2SE = (float)(log(S0 / E) * log2e);
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
  P.wait_limit = 1u << 22;       // ~32 ns sleep + an L2 round trip per poll: seconds
  P.copy_wait_limit = 1u << 20;  // try_wait polls: far beyond a microsecond-scale wait
}

// Discount factors exp(-r dt k) then growth factors exp(+r dt k), k = 0..M.
size_t dtab_bytes(int M) { return sizeof(float) * 2 * ((size_t)M + 1); }
void dtab_fill(float* dst, double r, double T, int M) {
  const double dtd = T / M;
  for (int k = 0; k <= M; ++k) {
    dst[k] = (float)exp(-r * dtd * k);
    dst[M + 1 + k] = (float)exp(r * dtd * k);
  }
}

// Shared-memory limits of the device and of the three kernels, queried once
// per device; the kernels' dynamic shared-memory ceilings are raised to the
// device maximum at the same time.
struct LsmLimits {
  size_t per_block = 0;  // opt-in maximum per block
  size_t per_sm = 0;
  size_t reserved = 0;   // per block, taken by the system
  size_t stat_coop = 0, stat8 = 0, stat16 = 0;  // static shared memory of each kernel
  int cl_max = 8;        // CTAs per cluster the device co-schedules (8 or 16)
  int status = PCF_OK;
};

template <typename K>
int lsm_kernel_setup(K kernel, size_t per_block, size_t* stat, bool cluster) {
  cudaFuncAttributes fa;
  int st = cuda_status(cudaFuncGetAttributes(&fa, kernel), "lsm kernel attributes");
  if (st) return st;
  *stat = fa.sharedSizeBytes;
  st = cuda_status(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(per_block - fa.sharedSizeBytes)),
                   "lsm smem attribute");
  if (!st)
    st = cuda_status(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                          (int)cudaSharedmemCarveoutMaxShared),
                     "lsm carveout attribute");
  if (!st && cluster)
    st = cuda_status(cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed,
                                          1),
                     "lsm cluster attribute");
  return st;
}

const LsmLimits& lsm_limits(const pcf_ctx* c) {
  static std::mutex mu;
  static LsmLimits cache[64];
  static bool have[64] = {};
  std::lock_guard<std::mutex> lock(mu);
  const int dev = c->device & 63;
  LsmLimits& L = cache[dev];
  if (have[dev]) return L;
  int v = 0;
  L.status = cuda_status(
      cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device), "attr");
  L.per_block = (size_t)v;
  if (!L.status)
    L.status = cuda_status(
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device),
        "attr");
  L.per_sm = (size_t)v;
  if (!L.status)
    L.status = cuda_status(
        cudaDeviceGetAttribute(&v, cudaDevAttrReservedSharedMemoryPerBlock, c->device), "attr");
  L.reserved = (size_t)v;
  if (!L.status) L.status = lsm_kernel_setup(lsm_kernel, L.per_block, &L.stat_coop, false);
  if (!L.status) {
    size_t stat = 0;
    L.status = lsm_kernel_setup(lsm_coop_cluster_kernel, L.per_block, &stat, false);
    L.stat_coop = std::max(L.stat_coop, stat);
  }
  if (!L.status)
    L.status = lsm_kernel_setup(lsm_cluster_kernel<unsigned char>, L.per_block, &L.stat8, true);
  if (!L.status)
    L.status = lsm_kernel_setup(lsm_cluster_kernel<unsigned short>, L.per_block, &L.stat16, true);
  if (!L.status) {
    // 16-CTA clusters where the device can co-schedule them at two CTAs per
    // SM with 4096-pair slices; otherwise the portable 8.
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 16;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(kLsmCBlock);
    cfg.dynamicSmemBytes = lsm_smem(4096, 64, 1);
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    L.cl_max = cudaOccupancyMaxActiveClusters(&n, lsm_cluster_kernel<unsigned char>, &cfg) ==
                           cudaSuccess &&
                       n > 0
                   ? 16
                   : 8;
    cudaGetLastError();
  }
  have[dev] = L.status == PCF_OK;
  return L;
}

bool lsm_fits(const LsmLimits& Lm, int PB, int M, size_t tau_bytes, size_t stat, int per_sm) {
  const size_t need = lsm_smem(PB, M, tau_bytes) + stat;
  return need <= Lm.per_block && (size_t)per_sm * (need + Lm.reserved) <= Lm.per_sm;
}

// Cooperative-launch grid for one contract: at most one block per SM, at
// least one pair per thread. Returns false if a block's slice does not fit.
bool coop_shape(const pcf_ctx* c, const LsmLimits& Lm, long long H, int M, int& G, int& PB,
                size_t& smem) {
  const long long G0 = std::max(1LL, std::min((H + kLsmBlock - 1) / kLsmBlock,
                                              (long long)c->sm_count));
  PB = (int)((((H + G0 - 1) / G0) + 3) & ~3LL);
  G = (int)((H + PB - 1) / PB);
  smem = lsm_smem(PB, M, 2);
  return lsm_fits(Lm, PB, M, 2, Lm.stat_coop, 1);
}

// Grid of the streaming sweep (lsm_stream_kernel) for a contract of H pairs:
// one block per SM (cooperative), the pairs split evenly in multiples of 4.
int stream_shape(const pcf_ctx* c, long long H, int M, int& G, int& PB, size_t& smem) {
  smem = sizeof(float) * 2 * (size_t)(M + 1);
  int occ = 0;
  const int st = cuda_status(
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lsm_stream_kernel, kLsmBlock, smem),
      "occupancy(lsm stream)");
  if (st) return st;
  if (occ < 1) return set_error(PCF_EINVAL, "the streaming LSM block does not fit on an SM");
  const long long G0 = std::min((long long)c->sm_count, (H + 3) / 4);
  PB = (int)((((H + G0 - 1) / G0) + 3) & ~3LL);
  G = (int)((H + PB - 1) / PB);
  return PCF_OK;
}

// Bytes after a contract's path matrix that the streaming sweep keeps its
// per-path state in: 2*Hp cash flows, then 2*Hp exercise dates.
size_t stream_state_bytes(long long Hp) { return a256(8 * (size_t)Hp) + a256(4 * (size_t)Hp); }

// A grid of whole clusters for the two-level exchange
// (lsm_coop_cluster_kernel) of one contract of H pairs whose plain
// cooperative grid is G blocks of `smem` bytes: as many clusters of 8 (else 4)
// CTAs as the device co-schedules, which cluster placement can make fewer
// than the SMs. hcl = 0 when the plain cooperative kernel should run. Measured
// on one put, 50 dates: 2^19 paths 0.40 -> 0.33 ms, 2^20 0.46 -> 0.39, 2^21
// 0.62 -> 0.53.
void hybrid_shape(const LsmLimits& Lm, long long H, int M, int G, size_t smem, int& hcl, int& Gh,
                  int& PBh) {
  hcl = Gh = PBh = 0;
  for (int cl : {8, 4}) {
    if (G < 2 * cl) continue;
    cudaLaunchConfig_t q = {};
    cudaLaunchAttribute qa[1];
    qa[0].id = cudaLaunchAttributeClusterDimension;
    qa[0].val.clusterDim.x = cl;
    qa[0].val.clusterDim.y = 1;
    qa[0].val.clusterDim.z = 1;
    q.gridDim = dim3(cl);
    q.blockDim = dim3(kLsmBlock);
    q.dynamicSmemBytes = smem;
    q.attrs = qa;
    q.numAttrs = 1;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, lsm_coop_cluster_kernel, &q) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    const int g = std::min((G + cl - 1) / cl, ncl) * cl;
    if (g < 2 * cl || g * 5 < G * 4) continue;  // keep at least 80 % of the grid
    const int pb = (int)(((H + g - 1) / g + 3) & ~3LL);
    // Below ~1024 pairs per CTA the in-cluster exchange costs more than the
    // global barrier it spares (measured: 2^17 paths 0.32 -> 0.38 ms).
    if (pb < 1024 || !lsm_fits(Lm, pb, M, 2, Lm.stat_coop, 1)) continue;
    hcl = cl;
    Gh = g;
    PBh = pb;
    break;
  }
}

// Launches one contract's sweep on the hybrid grid if hcl > 0, else (or if
// the device refuses that launch) on the plain cooperative grid.
int launch_coop(const LsmParams& P0, int G, int PB, size_t smem, int hcl, int Gh, int PBh,
                cudaStream_t s, bool* used_hybrid) {
  LsmParams P = P0;
  *used_hybrid = false;
  if (hcl > 0) {
    P.pairs_per_block = PBh;
    P.nblocks = Gh;
    P.cluster = hcl;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = hcl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeCooperative;
    at[1].val.cooperative = 1;
    cfg.gridDim = dim3(Gh);
    cfg.blockDim = dim3(kLsmBlock);
    cfg.dynamicSmemBytes = lsm_smem(PBh, P.M, 2);
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 2;
    if (cudaLaunchKernelEx(&cfg, lsm_coop_cluster_kernel, P) == cudaSuccess) {
      *used_hybrid = true;
      return PCF_OK;
    }
    cudaGetLastError();
  }
  P.pairs_per_block = PB;
  P.nblocks = G;
  P.cluster = 0;
  void* args[] = {&P};
  return cuda_status(cudaLaunchCooperativeKernel((void*)lsm_kernel, dim3(G), dim3(kLsmBlock), args,
                                                 smem, s),
                     "lsm cooperative launch");
}

constexpr int kLsmPB[] = {512, 1024, 2048, 4096, 8192};
constexpr int kNumPB = 5;

// Shape of a contract in a cluster launch: the smallest power-of-two cluster
// that covers the contract with slices that let two CTAs share an SM (the
// smallest such slice at that cluster size); beyond that, the largest cluster
// with one CTA per SM. Few CTAs per contract leave room for more contracts in
// flight, and each CTA pays the per-date exchange once for more paths.
// (Measured: one 1024-thread CTA per SM holding the same 8192 pairs ran the
// 64-put batch no faster and the mixed stream 4 % slower.)
// `shift` (the tuning table's, by class of N) moves off that choice: +1
// doubles the cluster and halves the slice, -1 halves the cluster and
// doubles the slice (one CTA per SM where two no longer fit), when the
// device allows the result; the CTAs still cover the contract.
bool cluster_shape(const LsmLimits& Lm, long long H, int M, int shift, int& cl, int& k,
                   bool& t8) {
  t8 = M <= 255;
  const size_t tb = t8 ? 1 : 2, stat = t8 ? Lm.stat8 : Lm.stat16;
  bool found = false;
  for (cl = 1; cl <= Lm.cl_max && !found; cl *= 2)
    for (k = 0; k < kNumPB; ++k)
      if ((long long)cl * kLsmPB[k] >= H && lsm_fits(Lm, kLsmPB[k], M, tb, stat, 2)) {
        found = true;
        break;
      }
  if (found) {
    cl /= 2;  // undo the loop's last doubling
  } else {
    cl = Lm.cl_max;
    for (k = 0; k < kNumPB && !found; ++k)
      if ((long long)cl * kLsmPB[k] >= H && lsm_fits(Lm, kLsmPB[k], M, tb, stat, 1)) found = true;
    if (!found) return false;
    --k;  // undo the loop's last increment
  }
  if (shift > 0 && k > 0 && 2 * cl <= Lm.cl_max && lsm_fits(Lm, kLsmPB[k - 1], M, tb, stat, 2)) {
    cl *= 2;
    --k;
  } else if (shift < 0 && cl > 1 && k + 1 < kNumPB &&
             lsm_fits(Lm, kLsmPB[k + 1], M, tb, stat, 1)) {
    cl /= 2;
    ++k;
  }
  return true;
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
  bool t8 = true;
  size_t smem = 0;
  LsmParams* d_params = nullptr;
};

struct LsmBatch {
  std::vector<LsmCluster> clusters;
  std::vector<LsmParams> coop;  // contracts too large for one cluster
  std::vector<int> coop_grid, coop_pb, coop_hcl, coop_gh, coop_pbh;
  std::vector<char> coop_stream;  // runs the streaming sweep
  std::vector<size_t> coop_smem;
  void* d_mem = nullptr;
  size_t bytes = 0;
};

// Shapes and device layout of a batch: params tables | discount tables (the
// uploaded prefix) | cooperative scratch | path matrices.
struct LsmLayout {
  std::vector<int> group;  // launch group of each contract, -1: cooperative kernel
  std::vector<std::vector<int>> members;
  std::vector<size_t> o_params, o_dt, o_paths, o_coop;
  std::vector<char> stream;  // cooperative contract that runs the streaming sweep
  std::vector<int> coop_G, coop_PB, coop_hcl, coop_Gh, coop_PBh;
  std::vector<size_t> coop_sm;
  size_t upload = 0, total = 0;
};

// Launch group of a cluster shape: (log2 cluster size, slice class, tau width).
constexpr int kLsmGroups = 5 * kNumPB * 2;
int group_of(int cl, int k, bool t8) {
  int lg = 0;
  while ((1 << lg) < cl) ++lg;
  return (lg * kNumPB + k) * 2 + (t8 ? 1 : 0);
}

int lsm_layout(pcf_ctx* c, const std::vector<LsmRequest>& reqs, LsmLayout& L) {
  const LsmLimits& Lm = lsm_limits(c);
  if (Lm.status) return Lm.status;
  const TuneTable tt = tune_table(c->device);
  const size_t n = reqs.size();
  L.group.assign(n, -1);
  L.members.assign(kLsmGroups, {});
  for (size_t i = 0; i < n; ++i) {
    int cl, k;
    bool t8;
    if (cluster_shape(Lm, reqs[i].N / 2, reqs[i].M, tt.lsm_shift[lsm_class(reqs[i].N)], cl, k,
                      t8)) {
      L.group[i] = group_of(cl, k, t8);
      L.members[L.group[i]].push_back((int)i);
    }
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
    off = a256(off + dtab_bytes(reqs[i].M));
  }
  L.upload = off;
  L.coop_G.assign(n, 0);
  L.coop_PB.assign(n, 0);
  L.coop_hcl.assign(n, 0);
  L.coop_Gh.assign(n, 0);
  L.coop_PBh.assign(n, 0);
  L.coop_sm.assign(n, 0);
  L.o_coop.assign(n, 0);
  L.stream.assign(n, 0);
  for (size_t i = 0; i < n; ++i) {
    if (L.group[i] >= 0) continue;
    if (coop_shape(c, Lm, reqs[i].N / 2, reqs[i].M, L.coop_G[i], L.coop_PB[i], L.coop_sm[i])) {
      hybrid_shape(Lm, reqs[i].N / 2, reqs[i].M, L.coop_G[i], L.coop_sm[i], L.coop_hcl[i],
                   L.coop_Gh[i], L.coop_PBh[i]);
    } else {
      const int st = stream_shape(c, reqs[i].N / 2, reqs[i].M, L.coop_G[i], L.coop_PB[i],
                                  L.coop_sm[i]);
      if (st) return st;
      L.stream[i] = 1;
    }
    const size_t gm = (size_t)std::max(L.coop_G[i], L.coop_Gh[i]);
    L.o_coop[i] = off;  // partial (2 G 8 float2) | fpartial (G 5 float2) | 2 counters
    off = a256(off + 8 * (2 * gm * kRegSums + gm * kMoments) + 16);
  }
  L.o_paths.assign(n, 0);
  for (size_t i = 0; i < n; ++i) {
    L.o_paths[i] = off;
    const long long Hp = ((reqs[i].N / 2) + 3) & ~3LL;
    off = a256(off + sizeof(float) * (size_t)reqs[i].M * 2 * (size_t)Hp);
    if (L.stream[i]) off += stream_state_bytes(Hp);
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
  for (size_t g = 0; g < Lo.members.size(); ++g) {
    if (Lo.members[g].empty()) continue;
    LsmCluster L;
    L.t8 = (g & 1) != 0;
    L.PB = kLsmPB[(g / 2) % kNumPB];
    L.CL = 1 << (g / 2 / kNumPB);
    L.C = (int)Lo.members[g].size();
    int Mmax = 2;
    LsmParams* tab = (LsmParams*)(h + Lo.o_params[g]);
    for (int j = 0; j < L.C; ++j) {
      const int i = Lo.members[g][j];
      fill(i, tab[j]);
      tab[j].pairs_per_block = L.PB;
      tab[j].nblocks = L.CL;
      Mmax = std::max(Mmax, reqs[i].M);
    }
    L.smem = lsm_smem(L.PB, Mmax, L.t8 ? 1 : 2);
    L.d_params = (LsmParams*)(d + Lo.o_params[g]);
    B->clusters.push_back(L);
  }
  for (size_t i = 0; i < reqs.size(); ++i) {
    if (Lo.group[i] >= 0) continue;
    LsmParams P;
    fill(i, P);
    P.pairs_per_block = Lo.coop_PB[i];
    P.nblocks = Lo.coop_G[i];
    const size_t gm = (size_t)std::max(Lo.coop_G[i], Lo.coop_Gh[i]);
    char* base = d + Lo.o_coop[i];
    P.partial = (double*)base;
    P.fpartial = (double*)(base + 8 * 2 * gm * kRegSums);
    unsigned* cnt = (unsigned*)(base + 8 * (2 * gm * kRegSums + gm * kMoments));
    P.barrier = cnt;
    P.ticket = cnt + 1;
    if (Lo.stream[i]) {
      const size_t mb = a256(sizeof(float) * (size_t)P.M * 2 * (size_t)P.Hp);
      P.gcf = (float*)(d + Lo.o_paths[i] + mb);
      P.gtau = (unsigned short*)(d + Lo.o_paths[i] + mb + a256(8 * (size_t)P.Hp));
    }
    B->coop_stream.push_back(Lo.stream[i]);
    B->coop.push_back(P);
    B->coop_grid.push_back(Lo.coop_G[i]);
    B->coop_pb.push_back(Lo.coop_PB[i]);
    B->coop_hcl.push_back(Lo.coop_hcl[i]);
    B->coop_gh.push_back(Lo.coop_Gh[i]);
    B->coop_pbh.push_back(Lo.coop_PBh[i]);
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
  const int st = lsm_batch_launch_clusters(c, B, s);
  return st ? st : lsm_batch_launch_coop(c, B, s);
}

int lsm_batch_launch_clusters(pcf_ctx* c, LsmBatch* B, cudaStream_t s) {
  int st;
  for (const LsmCluster& L : B->clusters) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = L.CL;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(L.C * L.CL);
    cfg.blockDim = dim3(kLsmCBlock);
    cfg.dynamicSmemBytes = L.smem;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const LsmParams* prm = L.d_params;
    const int C = L.C;
    st = cuda_status(L.t8 ? cudaLaunchKernelEx(&cfg, lsm_cluster_kernel<unsigned char>, prm, C)
                          : cudaLaunchKernelEx(&cfg, lsm_cluster_kernel<unsigned short>, prm, C),
                     "lsm cluster launch");
    if (st) return st;
    c->launches += 1;
  }
  return PCF_OK;
}

int lsm_batch_launch_coop(pcf_ctx* c, LsmBatch* B, cudaStream_t s) {
  int st;
  for (size_t i = 0; i < B->coop.size(); ++i) {
    LsmParams& P = B->coop[i];
    st = cuda_status(cudaMemsetAsync(P.barrier, 0, 2 * sizeof(unsigned), s), "memset LSM counters");
    if (st) return st;
    if (B->coop_stream[i]) {
      P.pairs_per_block = B->coop_pb[i];
      P.nblocks = B->coop_grid[i];
      void* args[] = {&P};
      st = cuda_status(cudaLaunchCooperativeKernel((void*)lsm_stream_kernel,
                                                   dim3(B->coop_grid[i]), dim3(kLsmBlock), args,
                                                   B->coop_smem[i], s),
                       "lsm streaming launch");
    } else {
      bool used = false;
      st = launch_coop(P, B->coop_grid[i], B->coop_pb[i], B->coop_smem[i], B->coop_hcl[i],
                       B->coop_gh[i], B->coop_pbh[i], s, &used);
    }
    if (st) return st;
    c->launches += 1;
  }
  return PCF_OK;
}

int lsm_batch_kernels(const LsmBatch* B) { return (int)(B->clusters.size() + B->coop.size()); }
int lsm_batch_cluster_kernels(const LsmBatch* B) { return (int)B->clusters.size(); }

void lsm_batch_destroy(LsmBatch* B) {
  if (!B) return;
  if (B->d_mem) cudaFree(B->d_mem);
  delete B;
}

}  // namespace pcf

using namespace pcf;

namespace {

// Optional audit record of one pcf_mc_amer call (host buffers; any may be NULL).
struct AmerAudit {
  float* coef;            // M x 4: per date d (index d), {mode, c0, c1, c2}
  double* sums;           // M x 8: the regression sums the solve saw at date d
  unsigned short* tau;    // N: exercise date per path (plus half, then minus half)
  float* u;               // M x N: the path matrix, row m-1 = date m
};

int amer_run(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T, long long N,
             int M, int payoff_fun, int ref_exercise, unsigned long long seed, int use_cv,
             pcf_mc_result* out, const AmerAudit* au) {
  if (!out) return set_error(PCF_EINVAL, "out is NULL");
  int st = check_lsm_request(S0, E, r, sigma, T, N, M, payoff_fun);
  if (st) return st;
  pcf_ctx* c = resolve_ctx(ctx, &st);
  if (!c) return st;
  const LsmLimits& Lm = lsm_limits(c);
  if (Lm.status) return Lm.status;
  int G = 0, PB = 0;
  size_t smem = 0;
  // A contract whose per-block slice does not fit in shared memory runs the
  // streaming sweep (per-path state in device memory), one block per SM.
  const bool streaming = !coop_shape(c, Lm, N / 2, M, G, PB, smem);
  int hcl = 0, Gh = 0, PBh = 0;
  if (streaming) {
    st = stream_shape(c, N / 2, M, G, PB, smem);
    if (st) return st;
  } else {
    int occ = 0;
    st = cuda_status(
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, lsm_kernel, kLsmBlock, smem),
        "occupancy(lsm)");
    if (st) return st;
    if ((long long)occ * c->sm_count < G)
      return set_error(PCF_EINVAL, "LSM grid of %d blocks cannot be co-resident", G);
    // The barrier test hook runs on the plain cooperative grid only.
    if (!c->test_barrier_extra) hybrid_shape(Lm, N / 2, M, G, smem, hcl, Gh, PBh);
  }
  const int Gmax = std::max(G, Gh);

  LsmParams P;
  lsm_fill(P, S0, E, r, sigma, T, N, M, payoff_fun, ref_exercise, seed, 0);
  P.pairs_per_block = PB;
  P.nblocks = G;
  if (c->test_barrier_extra) {
    P.barrier_extra = c->test_barrier_extra;
    P.wait_limit = c->test_poll_limit;
  }
  // Resident path matrix: M rows x 2*Hp floats (the streaming sweep adds
  // 2*Hp cash flows and 2*Hp exercise dates).
  const size_t matrix_bytes = a256(sizeof(float) * (size_t)M * 2 * (size_t)P.Hp);
  const size_t paths_bytes = matrix_bytes + (streaming ? stream_state_bytes(P.Hp) : 0);
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
  // Scratch: dtab | partial | fpartial | counters | out [| audit coef | sums | tau].
  const size_t o_dt = 0;
  const size_t o_part = a256(o_dt + dtab_bytes(M));
  const size_t o_fpart = a256(o_part + sizeof(double) * 2 * Gmax * kRegSums);
  const size_t o_cnt = a256(o_fpart + sizeof(double) * Gmax * kMoments);
  const size_t o_out = a256(o_cnt + sizeof(unsigned) * 4);
  const size_t o_acoef = a256(o_out + sizeof(double) * kMoments);
  const size_t o_asums = a256(o_acoef + (au ? sizeof(float) * 4 * (size_t)M : 0));
  const size_t o_atau = a256(o_asums + (au ? sizeof(double) * kRegSums * (size_t)M : 0));
  const size_t total = a256(o_atau + (au ? sizeof(unsigned short) * (size_t)N : 0));
  st = ctx_ensure(c, total, total);
  if (st) return st;
  char* d = (char*)c->d_buf;
  char* h = (char*)c->h_buf;
  dtab_fill((float*)(h + o_dt), r, T, M);
  st = cuda_status(cudaMemcpyAsync(d + o_dt, h + o_dt, dtab_bytes(M), cudaMemcpyHostToDevice,
                                   c->stream), "H2D dtab");
  if (!st) st = cuda_status(cudaMemsetAsync(d + o_cnt, 0, sizeof(unsigned) * 4, c->stream),
                            "memset counters");
  if (!st && au)  // dates without a regression (date 0, skipped dates) read as mode 0
    st = cuda_status(cudaMemsetAsync(d + o_acoef, 0, total - o_acoef, c->stream), "memset audit");
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
  if (au) {
    P.dbg_coef = (float*)(d + o_acoef);
    P.dbg_sums = (double*)(d + o_asums);
    P.dbg_tau = (unsigned short*)(d + o_atau);
  }
  if (streaming) {
    P.gcf = (float*)((char*)c->d_paths + matrix_bytes);
    P.gtau = (unsigned short*)((char*)c->d_paths + matrix_bytes + a256(8 * (size_t)P.Hp));
    void* args[] = {&P};
    st = cuda_status(cudaLaunchCooperativeKernel((void*)lsm_stream_kernel, dim3(G),
                                                 dim3(kLsmBlock), args, smem, c->stream),
                     "lsm streaming launch");
  } else {
    bool used = false;
    st = launch_coop(P, G, PB, smem, hcl, Gh, PBh, c->stream, &used);
  }
  if (st) return st;
  c->launches += 1;
  st = cuda_status(cudaMemcpyAsync(h + o_cnt, d + o_cnt, total - o_cnt, cudaMemcpyDeviceToHost,
                                   c->stream),
                   "D2H lsm");
  if (!st && au && au->u) {
    // Row m-1 (date m): plus half [0, H) then minus half [Hp, Hp + H) of each
    // 2*Hp-float row, into M rows of N floats.
    const size_t pitch = sizeof(float) * 2 * (size_t)P.Hp, w = sizeof(float) * (size_t)P.H;
    st = cuda_status(cudaMemcpy2DAsync(au->u, sizeof(float) * (size_t)N, c->d_paths, pitch, w,
                                       (size_t)M, cudaMemcpyDeviceToHost, c->stream),
                     "D2H audit paths (plus half)");
    if (!st)
      st = cuda_status(cudaMemcpy2DAsync(au->u + P.H, sizeof(float) * (size_t)N,
                                         (const float*)c->d_paths + P.Hp, pitch, w, (size_t)M,
                                         cudaMemcpyDeviceToHost, c->stream),
                       "D2H audit paths (minus half)");
  }
  if (!st) st = cuda_status(cudaStreamSynchronize(c->stream), "lsm kernel");
  if (st) return st;
  if (au) {
    if (au->coef) memcpy(au->coef, h + o_acoef, sizeof(float) * 4 * (size_t)M);
    if (au->sums) memcpy(au->sums, h + o_asums, sizeof(double) * kRegSums * (size_t)M);
    if (au->tau) memcpy(au->tau, h + o_atau, sizeof(unsigned short) * (size_t)N);
  }
  const int* flags = (const int*)(h + o_cnt);
  if (flags[2] == 4) return set_error(PCF_ECUDA, "LSM cluster launch ran without its cluster shape");
  if (flags[2]) return set_error(PCF_ETIMEOUT, "LSM device wait gave up (code %d)", flags[2]);
  if (flags[3])
    return set_error(PCF_ESINGULAR, "Determinant is not > 0 at %d exercise date(s)", flags[3]);
  const double* s = (const double*)(h + o_out);
  fill_amer_result(s, N, S0, E, r, sigma, T, payoff_fun, use_cv != 0, out);
  return PCF_OK;
}

}  // namespace

extern "C" int pcf_mc_amer(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T,
                           long long N, int M, int payoff_fun, int ref_exercise,
                           unsigned long long seed, int use_cv, pcf_mc_result* out) {
  return pcf::abi_guard([&]() -> int {
    return amer_run(ctx, S0, E, r, sigma, T, N, M, payoff_fun, ref_exercise, seed, use_cv, out,
                    nullptr);
  });
}

extern "C" int pcf_mc_amer_audit(pcf_ctx* ctx, double S0, double E, double r, double sigma,
                                 double T, long long N, int M, int payoff_fun, int ref_exercise,
                                 unsigned long long seed, pcf_mc_result* out, float* coef,
                                 double* sums, unsigned short* tau, float* u) {
  return pcf::abi_guard([&]() -> int {
    const AmerAudit au{coef, sums, tau, u};
    return amer_run(ctx, S0, E, r, sigma, T, N, M, payoff_fun, ref_exercise, seed, 1, out, &au);
  });
}
