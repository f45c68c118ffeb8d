// Monte Carlo pricing kernels for the European (mc_eur), Asian (mc_asia) and
// basket (mc_eur_multi) paths of moledoc/parcompfin.
//
// One kernel template serves the one-contract drop-in call and batched
// launches. Work is cut into items (one 256-thread block of paths of one
// contract). A block either takes item = blockIdx.x, or, when launched
// persistently, pulls items from a device queue until it is empty. Per-path
// arithmetic is FP32: Philox4x32-10 -> Box-Muller -> GBM in the log2 domain
// (one FMA + one ex2 per step) -> payoff. Each thread accumulates Kahan-
// compensated FP32 moment sums. Blocks reduce them as double-floats (FP32
// hi/lo pairs; the FP64 pipe is slow on GB300) and write one partial per
// item. The last item of a contract to finish sums that contract's partials
// in item order and widens to FP64, so results do not depend on scheduling.
//
// The kernels are issue-bound (a European path is ~31 FP32/INT instructions,
// two thirds of them Philox and Box-Muller, against 3 SFU operations), so the
// control-variate sums are compiled in only when a launch asks for them (CV
// template flag). Baskets of more than 16 assets run mc_basket_tc_kernel,
// which multiplies the normals by the correlation factor on the tensor
// cores, from the basket size the tuning table routes there (24 built in,
// where the tensor cores start to win; below it, up to 32 assets, the
// CUDA-core kernel runs; above 32 the tensor cores always do).
//
// Reference loops these kernels replace:
//   European  src/mc_eur.cpp:22-26,  src/mc_eur_omp.cpp:24-27
//   Asian     src/mc_asia.cpp:26-39, src/mc_asia_omp.cpp:33-44
//   basket    src/mc_eur_multi.cpp:19-34 with include/mvn.h:42-82
#include <algorithm>

#include "pcf_device.cuh"
#include "pcf_internal.h"

namespace pcf {

namespace {

// Per-thread moment accumulators. Values are first summed in plain FP32 over
// a short chunk (a few paths), then each chunk sum is added with Kahan
// compensation, so the thread total is accurate to a few FP32 ulps.
template <bool CV>
struct Moments {
  KSum y, yy, g, gg, yg;
  __device__ __forceinline__ void flush(float cy, float cyy, float cg, float cgg, float cyg) {
    y.add(cy);
    yy.add(cyy);
    if (CV) {
      g.add(cg);
      gg.add(cgg);
      yg.add(cyg);
    }
  }
  __device__ __forceinline__ void add(float Y, float G) {
    flush(Y, Y * Y, G, G * G, Y * G);
  }
};

__device__ __forceinline__ float payoff(const McContract& C, float S) {
  return fmaxf(fmaf(C.pf, S, C.nK), 0.f);  // max(pf (S - K), 0)
}

// European: item j covers path quads [j*U, (j+1)*U), U = units_per_item.
// Quad q's four paths take the four normals of Philox block (x=q, y=0).
// S_T = 2^(log2 S0 + a2 + b2 z); y = payoff(S_T), g = S_T.
template <bool CV, int BS>
__device__ __forceinline__ void eur_item(const McContract& C, int j, Moments<CV>& mo) {
  const long long nq = (C.N + 3) >> 2;
  const long long nfull = C.N >> 2;  // quads whose four paths are all < N
  const long long q0 = (long long)j * C.units_per_item + threadIdx.x;
  const int qpt = C.units_per_item / BS;
  const RngKey key{C.seed_lo, C.seed_hi, C.stream, TAG_EUR};
  const float a2 = C.a2 + C.l2S0;
  for (int k0 = 0; k0 < qpt; k0 += 4) {
    float cy = 0.f, cyy = 0.f, cg = 0.f, cgg = 0.f, cyg = 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const long long q = q0 + (long long)(k0 + kk) * BS;
      if (k0 + kk < qpt && q < nq) {
        const float4 z = normals4_x2(draw_words(key, (uint64_t)(C.x0 + q), 0u));
        // Paths (0, 2) and (1, 3) side by side in packed FP32x2 arithmetic
        // (each lane rounds exactly as the scalar operation).
        const float2 b2 = make_float2(C.b2, C.b2), a22 = make_float2(a2, a2);
        const float2 e02 = __ffma2_rn(b2, make_float2(z.x, z.z), a22);
        const float2 e13 = __ffma2_rn(b2, make_float2(z.y, z.w), a22);
        const float2 s02 = make_float2(ex2_approx(e02.x), ex2_approx(e02.y));
        const float2 s13 = make_float2(ex2_approx(e13.x), ex2_approx(e13.y));
        const float2 pf = make_float2(C.pf, C.pf), nK = make_float2(C.nK, C.nK);
        const float2 v02 = __ffma2_rn(pf, s02, nK), v13 = __ffma2_rn(pf, s13, nK);
        float s[4] = {s02.x, s13.x, s02.y, s13.y};
        float y[4] = {fmaxf(v02.x, 0.f), fmaxf(v13.x, 0.f), fmaxf(v02.y, 0.f),
                      fmaxf(v13.y, 0.f)};  // payoff
        if (q >= nfull) {  // the one partial quad at the end of the contract
          const long long left = C.N - 4 * q;
#pragma unroll
          for (int l = 0; l < 4; ++l)
            if (l >= left) y[l] = s[l] = 0.f;
        }
        cy += (y[0] + y[1]) + (y[2] + y[3]);
        cyy = fmaf(y[0], y[0], fmaf(y[1], y[1], fmaf(y[2], y[2], fmaf(y[3], y[3], cyy))));
        if (CV) {
          cg += (s[0] + s[1]) + (s[2] + s[3]);
          cgg = fmaf(s[0], s[0], fmaf(s[1], s[1], fmaf(s[2], s[2], fmaf(s[3], s[3], cgg))));
          cyg = fmaf(y[0], s[0], fmaf(y[1], s[1], fmaf(y[2], s[2], fmaf(y[3], s[3], cyg))));
        }
      }
    }
    mo.flush(cy, cyy, cg, cgg, cyg);
  }
}

// Asian: item j covers paths [j*U, (j+1)*U), U = units_per_item, U/BS per
// thread (path j*U + k*BS + thread); increment m uses lane m%4 of Philox block
// (x=path, y=m/4). log2(S/S0) is accumulated, S = S0 * 2^L.
// mode 0 (reference, src/mc_asia.cpp:31-35): I += S_m (c1 + c2 z_m) with S_m
//   the level before the step; A = I/M.
// mode 1: I += S_{m+1}; A = I/M (discrete mean of S_1..S_M).
// g = payoff of the geometric mean exp(sum_m w_m log S_m): mode 0 uses the
// trapezoid weights (w_M = 1/(2M), S_0's weight multiplies log S0/S0 = 0),
// mode 1 equal weights 1/M on S_1..S_M.
// One monitoring step of an Asian path (see asia_item). I accumulates the
// running sum in units of S0 (S/S0 = 2^L); the path multiplies by S0 once.
template <int MODE, bool CV>
__device__ __forceinline__ void asia_step(const McContract& C, float w, float z, float& L,
                                          float& I, float& lg) {
  if (MODE == 0) {
    I = fmaf(ex2_approx(L), fmaf(C.c2, z, C.c1), I);
    L += fmaf(C.b2, z, C.a2);
  } else {
    L += fmaf(C.b2, z, C.a2);
    I += ex2_approx(L);
  }
  if (CV) lg = fmaf(w, L, lg);
}

// One Asian path: the full groups of four steps (one Philox block each) run
// without per-step checks; the last 1..3 steps, if any, follow.
template <int MODE, bool CV>
__device__ __forceinline__ void asia_path(const McContract& C, const RngKey& key, long long n,
                                          float w, Moments<CV>& mo) {
  const int M = C.M, Mfull = M & ~3;
  float L = 0.f, I = 0.f, lg = 0.f;
  for (int m0 = 0; m0 < Mfull; m0 += 4) {
    const float4 z = normals4_x2(draw_words(key, (uint64_t)(C.x0 + n), (uint32_t)(m0 >> 2)));
    asia_step<MODE, CV>(C, w, z.x, L, I, lg);
    asia_step<MODE, CV>(C, w, z.y, L, I, lg);
    asia_step<MODE, CV>(C, w, z.z, L, I, lg);
    asia_step<MODE, CV>(C, w, z.w, L, I, lg);
  }
  if (Mfull < M) {
    const float4 z = normals4_x2(draw_words(key, (uint64_t)(C.x0 + n), (uint32_t)(Mfull >> 2)));
    asia_step<MODE, CV>(C, w, z.x, L, I, lg);
    if (Mfull + 1 < M) asia_step<MODE, CV>(C, w, z.y, L, I, lg);
    if (Mfull + 2 < M) asia_step<MODE, CV>(C, w, z.z, L, I, lg);
  }
  // Mode 0's trapezoid weight on the last level is w_last, not w.
  if (CV && MODE == 0) lg = fmaf(C.w_last - w, L, lg);
  const float Y = payoff(C, I * (C.S0 * w));
  const float G = CV ? payoff(C, C.S0 * ex2_approx(lg)) : 0.f;
  mo.add(Y, G);
}

// asia_step for two paths side by side (lanes .x and .y) in packed FP32x2
// arithmetic: each lane rounds exactly as the scalar step.
template <int MODE, bool CV>
__device__ __forceinline__ void asia_step2(const McContract& C, float2 w2, float2 z, float2& L,
                                           float2& I, float2& lg) {
  const float2 a2 = make_float2(C.a2, C.a2), b2 = make_float2(C.b2, C.b2);
  if (MODE == 0) {
    const float2 c = __ffma2_rn(make_float2(C.c2, C.c2), z, make_float2(C.c1, C.c1));
    I = __ffma2_rn(make_float2(ex2_approx(L.x), ex2_approx(L.y)), c, I);
    L = __fadd2_rn(L, __ffma2_rn(b2, z, a2));
  } else {
    L = __fadd2_rn(L, __ffma2_rn(b2, z, a2));
    I = __fadd2_rn(I, make_float2(ex2_approx(L.x), ex2_approx(L.y)));
  }
  if (CV) lg = __ffma2_rn(w2, L, lg);
}

// Two Asian paths at once (asia_path for paths n0 and n1, the same bits),
// their moments added in path order.
template <int MODE, bool CV>
__device__ __forceinline__ void asia_path2(const McContract& C, const RngKey& key, long long n0,
                                           long long n1, float w, Moments<CV>& mo) {
  const int M = C.M, Mfull = M & ~3;
  const float2 w2 = make_float2(w, w);
  float2 L = make_float2(0.f, 0.f), I = L, lg = L;
  for (int m0 = 0; m0 < Mfull; m0 += 4) {
    const float4 z0 = normals4_x2(draw_words(key, (uint64_t)(C.x0 + n0), (uint32_t)(m0 >> 2)));
    const float4 z1 = normals4_x2(draw_words(key, (uint64_t)(C.x0 + n1), (uint32_t)(m0 >> 2)));
    asia_step2<MODE, CV>(C, w2, make_float2(z0.x, z1.x), L, I, lg);
    asia_step2<MODE, CV>(C, w2, make_float2(z0.y, z1.y), L, I, lg);
    asia_step2<MODE, CV>(C, w2, make_float2(z0.z, z1.z), L, I, lg);
    asia_step2<MODE, CV>(C, w2, make_float2(z0.w, z1.w), L, I, lg);
  }
  if (Mfull < M) {
    const float4 z0 = normals4_x2(draw_words(key, (uint64_t)(C.x0 + n0), (uint32_t)(Mfull >> 2)));
    const float4 z1 = normals4_x2(draw_words(key, (uint64_t)(C.x0 + n1), (uint32_t)(Mfull >> 2)));
    asia_step2<MODE, CV>(C, w2, make_float2(z0.x, z1.x), L, I, lg);
    if (Mfull + 1 < M) asia_step2<MODE, CV>(C, w2, make_float2(z0.y, z1.y), L, I, lg);
    if (Mfull + 2 < M) asia_step2<MODE, CV>(C, w2, make_float2(z0.z, z1.z), L, I, lg);
  }
  if (CV && MODE == 0) lg = __ffma2_rn(make_float2(C.w_last - w, C.w_last - w), L, lg);
  const float sw = C.S0 * w;
  mo.add(payoff(C, I.x * sw), CV ? payoff(C, C.S0 * ex2_approx(lg.x)) : 0.f);
  mo.add(payoff(C, I.y * sw), CV ? payoff(C, C.S0 * ex2_approx(lg.y)) : 0.f);
}

template <bool CV, int BS>
__device__ __forceinline__ void asia_item(const McContract& C, int j, Moments<CV>& mo) {
  const RngKey key{C.seed_lo, C.seed_hi, C.stream, TAG_ASIA};
  const float w = 1.f / (float)C.M;
  const int ppt = C.units_per_item / BS;
  // Paths k and k + 1 of the thread side by side, then the odd one out.
#pragma unroll 1
  for (int k = 0; k < ppt; k += 2) {
    const long long n = (long long)j * C.units_per_item + (long long)k * BS + threadIdx.x;
    if (n >= C.N) break;
    const long long n1 = n + BS;
    if (k + 1 < ppt && n1 < C.N) {
      if (C.mode == 0) asia_path2<0, CV>(C, key, n, n1, w, mo);
      else asia_path2<1, CV>(C, key, n, n1, w, mo);
    } else {
      if (C.mode == 0) asia_path<0, CV>(C, key, n, w, mo);
      else asia_path<1, CV>(C, key, n, w, mo);
      break;
    }
  }
}

// Basket of d <= DMAX assets, one path. Asset a's normal is lane a%4 of
// Philox block (x=path, y=a/4). x = Lz with the correlation factor staged in
// shared memory; log2 S_a = l0_a + v_a x_a; y = payoff(mean_a S_a),
// g = payoff(2^(mean_a log2 S_a)). mode 0: the factor is lower triangular
// (Cholesky); mode 1: a full factor (eigen-decomposition fallback).
// The staged block is fb = [l0 | v | L], each row of L padded to DMAX floats
// with zeros beyond the factor, 16-byte aligned. The product runs column
// group by column group: the four normals of group b are drawn and folded
// into every row accumulator x_a that group touches (a >= 4b for the
// triangular factor), one 16-byte load of L per row and group. So the normals
// are never held as an array, the row accumulators are independent FMA
// chains, and the triangle costs exactly its FMAs (groups beyond d are
// skipped by uniform branches). Each x_a is the sum over b = 0, 1, ... in
// order, and the padding adds exact zeros.
template <int DMAX, bool CV>
__device__ __forceinline__ void basket_path(const McContract& C, const float* fb, long long n,
                                            Moments<CV>& mo) {
  const RngKey key{C.seed_lo, C.seed_hi, C.stream, TAG_BASKET};
  const int d = C.M;
  const float* l0 = fb;
  const float* vol = fb + DMAX;
  const float* Lf = fb + 2 * DMAX;
  const bool tri = C.mode == 0;
  // Rows 2p and 2p + 1 side by side (x2[p].x, x2[p].y) in packed FP32x2
  // FMAs: each lane accumulates its row in the scalar order.
  float2 x2[DMAX / 2];
#pragma unroll
  for (int p = 0; p < DMAX / 2; ++p) x2[p] = make_float2(0.f, 0.f);
#pragma unroll
  for (int b4 = 0; b4 < DMAX / 4; ++b4) {
    if (4 * b4 < d) {
      const float4 z = normals4_x2(draw_words(key, (uint64_t)(C.x0 + n), (uint32_t)b4));
      const float2 zx = make_float2(z.x, z.x), zy = make_float2(z.y, z.y);
      const float2 zz = make_float2(z.z, z.z), zw = make_float2(z.w, z.w);
#pragma unroll
      for (int a4 = 0; a4 < DMAX / 4; ++a4) {
        if (4 * a4 < d && (a4 >= b4 || !tri)) {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int p = 2 * a4 + h;  // rows 2p, 2p + 1
            // staged as (L[2p][k], L[2p+1][k]) pairs along k
            const float4 q0 = *reinterpret_cast<const float4*>(Lf + p * 2 * DMAX + 8 * b4);
            const float4 q1 = *reinterpret_cast<const float4*>(Lf + p * 2 * DMAX + 8 * b4 + 4);
            x2[p] = __ffma2_rn(make_float2(q0.x, q0.y), zx, x2[p]);
            x2[p] = __ffma2_rn(make_float2(q0.z, q0.w), zy, x2[p]);
            x2[p] = __ffma2_rn(make_float2(q1.x, q1.y), zz, x2[p]);
            x2[p] = __ffma2_rn(make_float2(q1.z, q1.w), zw, x2[p]);
          }
        }
      }
    }
  }
  float bsk = 0.f, geo = 0.f;
#pragma unroll
  for (int p = 0; p < DMAX / 2; ++p) {
    if (2 * p < d) {
      const float2 l2 = __ffma2_rn(*reinterpret_cast<const float2*>(vol + 2 * p), x2[p],
                                   *reinterpret_cast<const float2*>(l0 + 2 * p));
      bsk += ex2_approx(l2.x);
      geo += l2.x;
      if (2 * p + 1 < d) {
        bsk += ex2_approx(l2.y);
        geo += l2.y;
      }
    }
  }
  const float inv_d = 1.f / (float)d;
  const float Y = payoff(C, bsk * inv_d);
  const float G = CV ? payoff(C, ex2_approx(geo * inv_d)) : 0.f;
  mo.add(Y, G);
}

// Basket item j covers paths [j*U, (j+1)*U), U = units_per_item: U/BS paths
// per thread (path j*U + k*BS + thread), one after the other (the loop is
// not unrolled, so a path's unrolled factor product keeps its registers).
template <int DMAX, bool CV, int BS>
__device__ __forceinline__ void basket_item(const McContract& C, int j, const float* fb,
                                            Moments<CV>& mo) {
  const long long n0 = (long long)j * C.units_per_item + threadIdx.x;
  const int ppt = C.units_per_item / BS;
#pragma unroll 1
  for (int k = 0; k < ppt; ++k) {
    const long long n = n0 + (long long)k * BS;
    if (n >= C.N) break;
    basket_path<DMAX, CV>(C, fb, n, mo);
  }
}

__device__ __forceinline__ int find_contract(const int* start, int n, int item) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(start + mid) <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Threads resident per SM that a block size's launch bound keeps (the
// register budget per thread is the same for every block size).
template <int METHOD, int DMAX, int BS>
constexpr int mc_min_blocks() {
  return (DMAX >= 64 ? 2 : (METHOD == MC_EUR ? 5 : 4)) * 256 / BS > 0
             ? (DMAX >= 64 ? 2 : (METHOD == MC_EUR ? 5 : 4)) * 256 / BS
             : 1;
}

// Persistent launch: blocks of BS threads take work items from a queue in
// increasing order. The next ticket is taken while the current item runs, and
// the item's contract is found in one round: the contract is the block's
// previous one or one of the next BS - 1, so each thread tests one candidate
// (a binary search covers longer jumps). A work item is one block's worth of
// paths: units_per_item = BS x (paths or quads per thread).
template <int METHOD, int DMAX, bool CV, int BS>
__global__ void __launch_bounds__(BS, (mc_min_blocks<METHOD, DMAX, BS>()))
mc_kernel(McLaunch L) {
  __shared__ DF sh[32 * kMoments];
  __shared__ int s_item[2];
  __shared__ int s_c;
  extern __shared__ __align__(16) float s_fb[];
  if (threadIdx.x == 0) {
    s_c = -1;
    if (L.persistent) s_item[0] = (int)atomicAdd(L.queue, 1u);
  }
  __syncthreads();
  int c = 0;        // contract of the block's previous item
  int loaded = -1;  // basket whose factor block sits in s_fb
  for (int iter = 0;; ++iter) {
    int item;
    if (L.persistent) {
      item = s_item[iter & 1];
      // Read by every thread after this item's barriers; the slot it
      // overwrites was last read before the previous item's final barrier.
      if (threadIdx.x == 0 && item < L.total_items)
        s_item[(iter + 1) & 1] = (int)atomicAdd(L.queue, 1u);
    } else {
      if (iter > 0) break;
      item = blockIdx.x;
    }
    if (item >= L.total_items) break;
    {
      const int t = c + (int)threadIdx.x;
      if (t < L.ncontracts && __ldg(L.item_start + t) <= item &&
          (t + 1 == L.ncontracts || item < __ldg(L.item_start + t + 1)))
        s_c = t;
      __syncthreads();
      const int found = s_c;
      c = found >= 0 ? found : find_contract(L.item_start, L.ncontracts, item);
    }
    const McContract C = L.contracts[c];
    const int base = __ldg(L.item_start + c);
    const int j = item - base;
    Moments<CV> mo;
    if (METHOD == MC_EUR) {
      eur_item<CV, BS>(C, j, mo);
    } else if (METHOD == MC_ASIA) {
      asia_item<CV, BS>(C, j, mo);
    } else {
      if (loaded != c) {  // the previous item's readers are past the final barrier
        // Host layout [l0 (d) | v (d) | L (d x d)] -> padded [l0 | v | L]: L's
        // rows 2p and 2p + 1 interleaved, L[2p][k] at 2 DMAX p + 2k and
        // L[2p+1][k] next to it, zero beyond the factor.
        const int d = C.M;
        const float* src = L.basket_data + C.basket_off;
        for (int i = threadIdx.x; i < (2 + DMAX) * DMAX; i += BS) {
          float v = 0.f;
          if (i < 2 * DMAX) {
            const int row = i / DMAX, col = i % DMAX;
            if (col < d) v = src[row * d + col];
          } else {
            const int e = i - 2 * DMAX;
            const int row = 2 * (e / (2 * DMAX)) + (e & 1), col = (e % (2 * DMAX)) >> 1;
            if (row < d && col < d) v = src[2 * d + row * d + col];
          }
          s_fb[i] = v;
        }
        __syncthreads();
        loaded = c;
      }
      basket_item<DMAX, CV, BS>(C, j, s_fb, mo);
    }
    DF v[kMoments] = {df_of(mo.y), df_of(mo.yy), df_of(mo.g), df_of(mo.gg), df_of(mo.yg)};
    DF tot[kMoments];
    block_sum_df<kMoments>(v, sh, tot);
    grid_finalize_df<kMoments>(tot, (float2*)L.partial + (size_t)base * kMoments, L.tickets + c,
                               L.out + (size_t)c * kMoments, C.items, j);
    if (threadIdx.x == 0) s_c = -1;  // every thread read s_c before block_sum_df's barriers
    __syncthreads();
  }
}

// ---- baskets of more than 16 assets: the L z product on the tensor cores ----
//
// A tile is 128 paths (one per thread); the product X = Z L^T of a tile runs
// on the tensor cores, K (the assets) in chunks of 8. For each chunk every
// thread draws its path's next 8 normals and stores them, split into two
// TF32 parts z = z_hi + z_lo, as row `tid` of a 128 x 8 K-major chunk in
// shared memory (double-buffered); one thread then issues three
// tcgen05.mma kind::tf32 (M = 128, N = d rounded up to 16, K = 8)
// accumulating X += Z_hi L_hi^T + Z_lo L_hi^T + Z_hi L_lo^T in tensor memory
// and commits them to the chunk buffer's mbarrier, so drawing chunk c + 1
// overlaps the MMAs of chunk c. The dropped Z_lo L_lo^T term is below 2^-22
// of the product: X carries FP32-level accuracy. The factor is staged once
// per contract, split the same way. After the last chunk each warp reads its
// 32 rows of X (tcgen05.ld 32x32b) and finishes its paths on the CUDA cores.
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, adjacent along K 128 bytes apart (leading
// offset) and along M/N (K/4) x 128 bytes apart (stride offset). A chunk
// buffer is 16 KB, so four CTAs share an SM.
constexpr int kTcBlock = 128;

__device__ __forceinline__ uint32_t kmajor_off(int row, int k, int ktot) {
  return (uint32_t)((row >> 3) * (ktot >> 2) * 128 + (k >> 2) * 128 + (row & 7) * 16 +
                    (k & 3) * 4);
}

// Shared-memory matrix descriptor (no swizzle, descriptor version 1).
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar)));
}

// 32 consecutive accumulator columns of this thread's row (its warp's lanes).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

constexpr int kTcChunk = kTcBlock * 8;  // floats in one 128 x 8 chunk

template <int DMAX>
constexpr size_t tc_basket_smem() {  // l0, v | L_hi, L_lo | 2 x (Z_hi, Z_lo) chunks (floats)
  return (size_t)(2 * DMAX + 2 * DMAX * DMAX + 4 * kTcChunk) * sizeof(float);
}

template <int DMAX, bool CV>
__global__ void __launch_bounds__(kTcBlock, 4) mc_basket_tc_kernel(McLaunch L) {
  static_assert(DMAX == 32 || DMAX == 64, "tensor-core baskets: 17..64 assets");
  extern __shared__ __align__(128) float s_tc[];
  __shared__ DF sh[32 * kMoments];
  __shared__ int s_item[2];
  __shared__ int s_c;
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t s_tmem;
  float* l0 = s_tc;
  float* vol = s_tc + DMAX;
  float* Lhi = s_tc + 2 * DMAX;
  float* Llo = Lhi + DMAX * DMAX;
  float* Zc = Llo + DMAX * DMAX;  // buffer b: Z_hi at Zc + 2 b chunk, Z_lo next to it
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&s_tmem)),
                 "r"(DMAX));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    s_c = -1;
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
    if (L.persistent) s_item[0] = (int)atomicAdd(L.queue, 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;
  const uint32_t row_tmem = tmem + ((uint32_t)(warp * 32) << 16);
  const uint32_t sbo_l = (DMAX / 4) * 128;
  const uint32_t z_off = kmajor_off(tid, 0, 8) >> 2;  // this thread's row in a chunk
  uint32_t phase = 0;   // bit b: parity of the next wait on mbar[b]
  uint32_t pending = 0; // bit b: a commit on mbar[b] not yet waited
  bool failed = false;
  auto wait_buf = [&](int b) {
    if (!((pending >> b) & 1u)) return;
    if (!mbar_poll(&mbar[b], (phase >> b) & 1u, 1u << 24)) failed = true;
    phase ^= 1u << b;
    pending &= ~(1u << b);
  };
  int c = 0, loaded = -1;
  for (int iter = 0;; ++iter) {
    int item;
    if (L.persistent) {
      item = s_item[iter & 1];
      if (tid == 0 && item < L.total_items) s_item[(iter + 1) & 1] = (int)atomicAdd(L.queue, 1u);
    } else {
      if (iter > 0) break;
      item = blockIdx.x;
    }
    if (item >= L.total_items) break;
    {
      const int t = c + tid;
      if (t < L.ncontracts && __ldg(L.item_start + t) <= item &&
          (t + 1 == L.ncontracts || item < __ldg(L.item_start + t + 1)))
        s_c = t;
      __syncthreads();
      const int found = s_c;
      c = found >= 0 ? found : find_contract(L.item_start, L.ncontracts, item);
    }
    const McContract C = L.contracts[c];
    const int base = __ldg(L.item_start + c);
    const int j = item - base;
    const int d = C.M;
    if (loaded != c) {
      // Every MMA has completed (the last tile waited for all of them).
      // Host layout [l0 (d) | v (d) | L (d x d)]; L rows are the MMA's N rows.
      const float* src = L.basket_data + C.basket_off;
      for (int i = tid; i < DMAX; i += kTcBlock) {
        l0[i] = i < d ? src[i] : 0.f;
        vol[i] = i < d ? src[d + i] : 0.f;
      }
      for (int i = tid; i < DMAX * DMAX; i += kTcBlock) {
        const int n = i / DMAX, k = i % DMAX;
        const float v = (n < d && k < d) ? src[2 * d + n * d + k] : 0.f;
        const float hi = tf32_round(v);
        const uint32_t o = kmajor_off(n, k, DMAX) >> 2;
        Lhi[o] = hi;
        Llo[o] = tf32_round(v - hi);
      }
      loaded = c;
    }
    const int nchunks = (d + 7) >> 3, np = (d + 15) & ~15;
    // D f32, A and B tf32, both K-major; N >> 3 at bit 17, M >> 4 at bit 24.
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(np >> 3) << 17) |
                           ((uint32_t)(kTcBlock >> 4) << 24);
    const RngKey key{C.seed_lo, C.seed_hi, C.stream, TAG_BASKET};
    Moments<CV> mo;
    for (int tile = 0; tile < C.units_per_item / kTcBlock; ++tile) {
      const long long n = (long long)j * C.units_per_item + (long long)tile * kTcBlock + tid;
      for (int ch = 0; ch < nchunks; ++ch) {
        const int b = ch & 1;
        wait_buf(b);  // the MMAs that read buffer b two chunks ago are done
        float* zh = Zc + 2 * b * kTcChunk;
        float* zl = zh + kTcChunk;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int k4 = 2 * ch + h;
          float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
          if (4 * k4 < d) z = normals4_x2(draw_words(key, (uint64_t)(C.x0 + n), (uint32_t)k4));
          const float4 hi = make_float4(tf32_round(z.x), tf32_round(z.y), tf32_round(z.z),
                                        tf32_round(z.w));
          const float4 lo = make_float4(tf32_round(z.x - hi.x), tf32_round(z.y - hi.y),
                                        tf32_round(z.z - hi.z), tf32_round(z.w - hi.w));
          *reinterpret_cast<float4*>(zh + z_off + 32 * h) = hi;  // +128 bytes: next core matrix
          *reinterpret_cast<float4*>(zl + z_off + 32 * h) = lo;
        }
        // The chunk (and a newly staged factor) is visible to the tensor core;
        // at ch = 0 every thread has also read the previous tile's X.
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
          const uint32_t ah = smem_u32(zh), al = smem_u32(zl);
          const uint32_t bo = (uint32_t)ch * 256;  // chunk ch: two core matrices along K
          const uint32_t bh = smem_u32(Lhi) + bo, bl = smem_u32(Llo) + bo;
          umma_tf32(tmem, umma_desc(ah, 128, 256), umma_desc(bh, 128, sbo_l), idesc, ch > 0);
          umma_tf32(tmem, umma_desc(al, 128, 256), umma_desc(bh, 128, sbo_l), idesc, 1);
          umma_tf32(tmem, umma_desc(ah, 128, 256), umma_desc(bl, 128, sbo_l), idesc, 1);
          umma_commit(&mbar[b]);
        }
        pending |= 1u << b;
      }
      wait_buf(0);
      wait_buf(1);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      float bsk = 0.f, geo = 0.f;
#pragma unroll
      for (int half = 0; half < DMAX / 32; ++half) {
        if (32 * half < np) {
          float x[32];
          tmem_ld32(row_tmem + 32 * half, x);
#pragma unroll
          for (int a = 0; a < 32; ++a) {
            if (32 * half + a < d) {
              const float l2 = fmaf(vol[32 * half + a], x[a], l0[32 * half + a]);
              bsk += ex2_approx(l2);
              geo += l2;
            }
          }
        }
      }
      if (n < C.N) {
        const float inv_d = 1.f / (float)d;
        float Y = payoff(C, bsk * inv_d);
        float G = CV ? payoff(C, ex2_approx(geo * inv_d)) : 0.f;
        if (failed) Y = G = __int_as_float(0x7fc00000);  // a wait gave up: the result is NaN
        mo.add(Y, G);
      }
    }
    DF v[kMoments] = {df_of(mo.y), df_of(mo.yy), df_of(mo.g), df_of(mo.gg), df_of(mo.yg)};
    DF tot[kMoments];
    block_sum_df<kMoments>(v, sh, tot);
    grid_finalize_df<kMoments>(tot, (float2*)L.partial + (size_t)base * kMoments, L.tickets + c,
                               L.out + (size_t)c * kMoments, C.items, j);
    if (tid == 0) s_c = -1;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(DMAX));
  }
}

// Dynamic shared memory above 48 KB and the largest shared-memory carveout,
// so that four CTAs share an SM. Function attributes belong to the current
// device, so they are set on every launch (two host calls, no device work).
template <int DMAX, bool CV>
void tc_setup() {
  cudaFuncSetAttribute(mc_basket_tc_kernel<DMAX, CV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)tc_basket_smem<DMAX>());
  cudaFuncSetAttribute(mc_basket_tc_kernel<DMAX, CV>,
                       cudaFuncAttributePreferredSharedMemoryCarveout,
                       (int)cudaSharedmemCarveoutMaxShared);
}

template <int DMAX, bool CV>
cudaError_t launch_tc(const McLaunch& L, int grid, cudaStream_t s) {
  tc_setup<DMAX, CV>();
  mc_basket_tc_kernel<DMAX, CV><<<grid, kTcBlock, tc_basket_smem<DMAX>(), s>>>(L);
  return cudaGetLastError();
}

// CTAs per SM: the launch bound (4) caps the registers; shared memory
// decides the rest. (The occupancy query reports one CTA per SM for this
// kernel, which leaves three quarters of each SM idle; a persistent launch
// of more CTAs than fit would only queue them.)
template <int DMAX>
int tc_max_active(void) {
  tc_setup<DMAX, true>();
  tc_setup<DMAX, false>();
  int dev = 0, smem_sm = 0, reserved = 0;
  cudaFuncAttributes fa;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) !=
          cudaSuccess ||
      cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) !=
          cudaSuccess ||
      cudaFuncGetAttributes(&fa, mc_basket_tc_kernel<DMAX, true>) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  const size_t per = tc_basket_smem<DMAX>() + fa.sharedSizeBytes + (size_t)reserved;
  return std::max(1, std::min(4, (int)((size_t)smem_sm / per)));
}

constexpr size_t basket_smem(int dmax) { return (size_t)(2 + dmax) * dmax * sizeof(float); }

template <int METHOD, int DMAX, bool CV, int BS>
cudaError_t launch_one(const McLaunch& L, int grid, cudaStream_t s) {
  const size_t smem = METHOD == MC_BASKET ? basket_smem(DMAX) : 0;
  mc_kernel<METHOD, DMAX, CV, BS><<<grid, BS, smem, s>>>(L);
  return cudaGetLastError();
}

template <int METHOD, int DMAX, int BS>
cudaError_t launch_cv(const McLaunch& L, int grid, cudaStream_t s) {
  return L.cv ? launch_one<METHOD, DMAX, true, BS>(L, grid, s)
              : launch_one<METHOD, DMAX, false, BS>(L, grid, s);
}

template <int METHOD, int DMAX>
cudaError_t launch_bs(const McLaunch& L, int grid, int block, cudaStream_t s) {
  switch (block) {
    case 128: return launch_cv<METHOD, DMAX, 128>(L, grid, s);
    case 256: return launch_cv<METHOD, DMAX, 256>(L, grid, s);
    case 512: return launch_cv<METHOD, DMAX, 512>(L, grid, s);
  }
  return cudaErrorInvalidValue;
}

template <int METHOD, int DMAX, int BS>
int max_active_bs(void) {
  int n = 0;
  const size_t smem = METHOD == MC_BASKET ? basket_smem(DMAX) : 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mc_kernel<METHOD, DMAX, true, BS>, BS,
                                                    smem) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

template <int METHOD, int DMAX>
int max_active(int block) {
  switch (block) {
    case 128: return max_active_bs<METHOD, DMAX, 128>();
    case 512: return max_active_bs<METHOD, DMAX, 512>();
    default: return max_active_bs<METHOD, DMAX, 256>();
  }
}

}  // namespace

cudaError_t launch_mc(McMethod m, const McLaunch& L, int grid, int max_d, int block, bool tensor,
                      cudaStream_t s) {
  if (grid <= 0) return cudaSuccess;
  switch (m) {
    case MC_EUR: return launch_bs<MC_EUR, 4>(L, grid, block, s);
    case MC_ASIA: return launch_bs<MC_ASIA, 4>(L, grid, block, s);
    case MC_BASKET:
      if (max_d <= 4) return launch_bs<MC_BASKET, 4>(L, grid, block, s);
      if (max_d <= 8) return launch_bs<MC_BASKET, 8>(L, grid, block, s);
      if (max_d <= 16) return launch_bs<MC_BASKET, 16>(L, grid, block, s);
      if (max_d <= 32 && !tensor) return launch_bs<MC_BASKET, 32>(L, grid, block, s);
      if (max_d <= 32) return L.cv ? launch_tc<32, true>(L, grid, s) : launch_tc<32, false>(L, grid, s);
      if (max_d <= 64) return L.cv ? launch_tc<64, true>(L, grid, s) : launch_tc<64, false>(L, grid, s);
      return cudaErrorInvalidValue;
  }
  return cudaErrorInvalidValue;
}

int mc_max_active_blocks(McMethod m, int max_d, int block, bool tensor) {
  switch (m) {
    case MC_EUR: return max_active<MC_EUR, 4>(block);
    case MC_ASIA: return max_active<MC_ASIA, 4>(block);
    case MC_BASKET:
      if (max_d <= 4) return max_active<MC_BASKET, 4>(block);
      if (max_d <= 8) return max_active<MC_BASKET, 8>(block);
      if (max_d <= 16) return max_active<MC_BASKET, 16>(block);
      if (max_d <= 32 && !tensor) return max_active<MC_BASKET, 32>(block);
      if (max_d <= 32) return tc_max_active<32>();
      return tc_max_active<64>();
  }
  return 1;
}

}  // namespace pcf

// ---- European Monte Carlo that allocates nothing ---------------------------
//
// Some callers cannot call cudaMalloc at pricing time. Examples: a plugin
// inside a framework whose caching allocator has already reserved the GPU's
// memory; a latency-critical loop where cudaMalloc/cudaFree would stall the
// device; code certified to allocate only at start-up. pcf_mc_eur_noalloc
// serves them. It is the European kernel above with its scratch (per-item
// partial sums and the completion ticket) in a fixed, file-scope device array
// that is part of the library's device image. Every GPU that loads the library
// holds the array until the process exits.

#include <mutex>

#include "pcf_api_internal.h"

namespace pcf {

namespace {

constexpr int kNoAllocMaxItems = 16384;  // work items one call may use
constexpr size_t kNoAllocTicketBytes = 256;
constexpr size_t kNoAllocBytes =
    kNoAllocTicketBytes + (size_t)kNoAllocMaxItems * kMoments * sizeof(float2);  // 640.25 KiB
// A work item covers at most 256 threads x 64 path quads, so 16384 items
// bound N at 2^30 paths.
constexpr long long kNoAllocMaxPaths = (long long)kNoAllocMaxItems * kBlock * 64 * 4;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

__global__ void __launch_bounds__(kBlock) mc_eur_noalloc_kernel(McContract C,
                                                                unsigned char* scratch,
                                                                double* out) {
  __shared__ DF sh[32 * kMoments];
  unsigned* ticket = (unsigned*)scratch;
  float2* partial = (float2*)(scratch + kNoAllocTicketBytes);
  const int j = blockIdx.x;
  Moments<true> mo;
  eur_item<true, kBlock>(C, j, mo);
  DF v[kMoments] = {df_of(mo.y), df_of(mo.yy), df_of(mo.g), df_of(mo.gg), df_of(mo.yg)};
  DF tot[kMoments];
  block_sum_df<kMoments>(v, sh, tot);
  grid_finalize_df<kMoments>(tot, partial, ticket, out, C.items, j);
}

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_addr[kNoAllocMaxDevices];

// Per-device set-up, done once with the device current: the device address
// of the scratch array (host code must not use the symbol itself).
int noalloc_setup(unsigned char** addr, int dev) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const int st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                               "cudaGetSymbolAddress(no-alloc scratch)");
    if (st) return st;
    g_noalloc_addr[dev] = (unsigned char*)p;
  }
  *addr = g_noalloc_addr[dev];
  return PCF_OK;
}

}  // namespace

}  // namespace pcf

extern "C" int pcf_mc_eur_noalloc(double S0, double E, double r, double sigma, double T,
                                  long long N, int payoff_fun, unsigned long long seed,
                                  double* d_sums, void* stream) {
  return pcf::abi_guard([&]() -> int {
    using namespace pcf;
    if (!d_sums) return set_error(PCF_EINVAL, "d_sums is NULL");
    int st = check_common(S0, E, r, sigma, T, N, payoff_fun);
    if (st) return st;
    if (N > kNoAllocMaxPaths)
      return set_error(PCF_EINVAL,
                       "N = %lld exceeds the no-allocation limit of %lld paths (the fixed "
                       "scratch holds %d work items)",
                       N, (long long)kNoAllocMaxPaths, kNoAllocMaxItems);
    int dev = 0;
    st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (st) return st;
    if (dev < 0 || dev >= kNoAllocMaxDevices)
      return set_error(PCF_EINVAL, "device %d beyond the no-allocation table", dev);
    unsigned char* scratch = nullptr;
    st = noalloc_setup(&scratch, dev);
    if (st) return st;
    // The built-in work shape (256-thread items of at most 64 quads per
    // thread), whatever a tuner chose: the scratch size above is derived from it.
    const McContract C = make_eur(S0, E, r, sigma, T, N, payoff_fun, seed, 0, TuneTable{});
    if (C.items > kNoAllocMaxItems)
      return set_error(PCF_EINVAL, "N = %lld needs %d work items; the fixed scratch holds %d", N,
                       C.items, kNoAllocMaxItems);
    cudaStream_t s = (cudaStream_t)stream;
    st = cuda_status(cudaMemsetAsync(scratch, 0, sizeof(unsigned), s), "memset no-alloc ticket");
    if (st) return st;
    mc_eur_noalloc_kernel<<<C.items, kBlock, 0, s>>>(C, scratch, d_sums);
    return cuda_status(cudaGetLastError(), "no-alloc kernel launch");
  });
}
