// Monte Carlo pricing kernels for the European (mc_eur), Asian (mc_asia) and
// basket (mc_eur_multi) paths of moledoc/parcompfin.
//
// One kernel template serves the one-contract drop-in call and batched
// launches. Work is cut into items (one 256-thread block of paths of one
// contract). A block either takes item = blockIdx.x, or, when launched
// persistently, pulls items from a device queue until it is empty. Per-path
// arithmetic is FP32: Philox4x32-10 -> Box-Muller -> GBM in the log2 domain
// (one FMA + one ex2 per step) -> payoff. Each thread accumulates Kahan-
// compensated FP32 moment sums. Blocks reduce them in FP64 and write one
// partial per item. The last item of a contract to finish sums that
// contract's partials in item order, so results do not depend on scheduling.
//
// Reference loops these kernels replace:
//   European  src/mc_eur.cpp:22-26,  src/mc_eur_omp.cpp:24-27
//   Asian     src/mc_asia.cpp:26-39, src/mc_asia_omp.cpp:33-44
//   basket    src/mc_eur_multi.cpp:19-34 with include/mvn.h:42-82
#include "pcf_device.cuh"
#include "pcf_internal.h"

namespace pcf {

namespace {

__device__ __forceinline__ float payoff(float S, float K, float pf) {
  return fmaxf(pf * (S - K), 0.f);
}

struct Moments {
  KSum y, yy, g, gg, yg;
  __device__ __forceinline__ void add(float Y, float G) {
    y.add(Y);
    yy.add(Y * Y);
    g.add(G);
    gg.add(G * G);
    yg.add(Y * G);
  }
};

// European: item j covers path quads [j*U, (j+1)*U), U = units_per_item.
// Quad q's four paths take the four normals of Philox block (x=q, y=0).
// y = payoff(S_T), g = S_T.
__device__ __forceinline__ void eur_item(const McContract& C, int j, Moments& mo) {
  const long long nq = (C.N + 3) >> 2;
  const long long q0 = (long long)j * C.units_per_item;
  const int qpt = C.units_per_item / kBlock;
  const RngKey key{C.seed_lo, C.seed_hi, C.stream, TAG_EUR};
  for (int k = 0; k < qpt; ++k) {
    const long long q = q0 + threadIdx.x + (long long)k * kBlock;
    if (q >= nq) break;
    const float4 z = normals4(draw_words(key, (uint64_t)q, 0u));
    const long long left = C.N - 4 * q;
    float s[4];
    s[0] = C.S0 * ex2_approx(fmaf(C.b2, z.x, C.a2));
    s[1] = C.S0 * ex2_approx(fmaf(C.b2, z.y, C.a2));
    s[2] = C.S0 * ex2_approx(fmaf(C.b2, z.z, C.a2));
    s[3] = C.S0 * ex2_approx(fmaf(C.b2, z.w, C.a2));
    float ys = 0.f, yys = 0.f, gs = 0.f, ggs = 0.f, ygs = 0.f;
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const bool ok = l < left;
      const float Y = ok ? payoff(s[l], C.K, C.pf) : 0.f;
      const float G = ok ? s[l] : 0.f;
      ys += Y;
      yys = fmaf(Y, Y, yys);
      gs += G;
      ggs = fmaf(G, G, ggs);
      ygs = fmaf(Y, G, ygs);
    }
    mo.y.add(ys);
    mo.yy.add(yys);
    mo.g.add(gs);
    mo.gg.add(ggs);
    mo.yg.add(ygs);
  }
}

// Asian: one path per thread; increment m uses lane m%4 of Philox block
// (x=path, y=m/4). log2 S is accumulated, S = S0 * 2^L.
// mode 0 (reference, src/mc_asia.cpp:31-35): I += S_m (c1 + c2 z_m) with S_m
//   the level before the step; A = I/M.
// mode 1: I += S_{m+1}; A = I/M (discrete mean of S_1..S_M).
// g = payoff of the geometric mean exp(sum_m w_m log S_m): mode 0 uses the
// trapezoid weights (w_M = 1/(2M), S_0's weight multiplies log S0/S0 = 0),
// mode 1 equal weights 1/M on S_1..S_M.
__device__ __forceinline__ void asia_item(const McContract& C, int j, Moments& mo) {
  const long long n = (long long)j * C.units_per_item + threadIdx.x;
  const RngKey key{C.seed_lo, C.seed_hi, C.stream, TAG_ASIA};
  const int M = C.M;
  const float w = 1.f / (float)M;
  float L = 0.f, I = 0.f, lg = 0.f;
  for (int m0 = 0; m0 < M; m0 += 4) {
    const float4 z = normals4(draw_words(key, (uint64_t)n, (uint32_t)(m0 >> 2)));
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const int m = m0 + l;
      if (m < M) {
        const float zl = lane4(z, l);
        if (C.mode == 0) {
          const float S = C.S0 * ex2_approx(L);
          I = fmaf(S, fmaf(C.c2, zl, C.c1), I);
          L += fmaf(C.b2, zl, C.a2);
          lg = fmaf(m == M - 1 ? C.w_last : w, L, lg);
        } else {
          L += fmaf(C.b2, zl, C.a2);
          I += C.S0 * ex2_approx(L);
          lg = fmaf(w, L, lg);
        }
      }
    }
  }
  const bool ok = n < C.N;
  const float Y = ok ? payoff(I * w, C.K, C.pf) : 0.f;
  const float G = ok ? payoff(C.S0 * ex2_approx(lg), C.K, C.pf) : 0.f;
  mo.add(Y, G);
}

// Basket of d <= DMAX assets: one path per thread. Asset a's normal is lane
// a%4 of Philox block (x=path, y=a/4). x = Lz with the lower Cholesky factor
// staged in shared memory; log2 S_a = l0_a + v_a x_a; y = payoff(mean_a S_a),
// g = payoff(2^(mean_a log2 S_a)). mode 0: the factor is lower triangular
// (Cholesky); mode 1: a full factor (eigen-decomposition fallback).
template <int DMAX>
__device__ __forceinline__ void basket_item(const McContract& C, int j, const float* fb,
                                            Moments& mo) {
  const long long n = (long long)j * C.units_per_item + threadIdx.x;
  const RngKey key{C.seed_lo, C.seed_hi, C.stream, TAG_BASKET};
  const int d = C.M;
  const float* l0 = fb;
  const float* vol = fb + d;
  const float* Lf = fb + 2 * d;
  float z[DMAX];
#pragma unroll
  for (int a0 = 0; a0 < DMAX; a0 += 4) {
    if (a0 < d) {
      const float4 zz = normals4(draw_words(key, (uint64_t)n, (uint32_t)(a0 >> 2)));
      z[a0] = zz.x;
      z[a0 + 1] = zz.y;
      z[a0 + 2] = zz.z;
      z[a0 + 3] = zz.w;
    } else {
      z[a0] = z[a0 + 1] = z[a0 + 2] = z[a0 + 3] = 0.f;
    }
  }
  float bsk = 0.f, geo = 0.f;
  if (C.mode == 0) {  // lower-triangular Cholesky factor
#pragma unroll
    for (int a = 0; a < DMAX; ++a) {
      if (a < d) {
        const float* row = Lf + a * d;
        float x = 0.f;
#pragma unroll
        for (int b = 0; b <= a; ++b) x = fmaf(row[b], z[b], x);
        const float l2 = fmaf(vol[a], x, l0[a]);
        bsk += ex2_approx(l2);
        geo += l2;
      }
    }
  } else {  // full factor from the eigen-decomposition fallback
    for (int a = 0; a < d; ++a) {
      const float* row = Lf + a * d;
      float x = 0.f;
#pragma unroll
      for (int b = 0; b < DMAX; ++b)
        if (b < d) x = fmaf(row[b], z[b], x);
      const float l2 = fmaf(vol[a], x, l0[a]);
      bsk += ex2_approx(l2);
      geo += l2;
    }
  }
  const float inv_d = 1.f / (float)d;
  const bool ok = n < C.N;
  const float Y = ok ? payoff(bsk * inv_d, C.K, C.pf) : 0.f;
  const float G = ok ? payoff(ex2_approx(geo * inv_d), C.K, C.pf) : 0.f;
  mo.add(Y, G);
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

template <int METHOD, int DMAX>
__global__ void __launch_bounds__(kBlock) mc_kernel(McLaunch L) {
  __shared__ double sh[32 * kMoments];
  __shared__ int s_item;
  extern __shared__ float s_fb[];
  for (int iter = 0;; ++iter) {
    int item;
    if (L.persistent) {
      if (threadIdx.x == 0) s_item = (int)atomicAdd(L.queue, 1u);
      __syncthreads();
      item = s_item;
      __syncthreads();
    } else {
      if (iter > 0) break;
      item = blockIdx.x;
    }
    if (item >= L.total_items) break;
    const int c = find_contract(L.item_start, L.ncontracts, item);
    const McContract C = L.contracts[c];
    const int j = item - __ldg(L.item_start + c);
    Moments mo;
    if (METHOD == MC_EUR) {
      eur_item(C, j, mo);
    } else if (METHOD == MC_ASIA) {
      asia_item(C, j, mo);
    } else {
      const int d = C.M;
      const float* src = L.basket_data + C.basket_off;
      for (int i = threadIdx.x; i < 2 * d + d * d; i += kBlock) s_fb[i] = src[i];
      __syncthreads();
      basket_item<DMAX>(C, j, s_fb, mo);
      __syncthreads();
    }
    double v[kMoments] = {mo.y.value(), mo.yy.value(), mo.g.value(), mo.gg.value(),
                          mo.yg.value()};
    double tot[kMoments];
    block_sum<kMoments>(v, sh, tot);
    const int base = __ldg(L.item_start + c);
    grid_finalize<kMoments>(tot, L.partial + (size_t)base * kMoments, L.tickets + c,
                            L.out + (size_t)c * kMoments, C.items, j);
    __syncthreads();
  }
}

template <int METHOD, int DMAX>
cudaError_t launch_one(const McLaunch& L, int grid, cudaStream_t s) {
  size_t smem = METHOD == MC_BASKET ? (size_t)(2 * DMAX + DMAX * DMAX) * sizeof(float) : 0;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(mc_kernel<METHOD, DMAX>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  mc_kernel<METHOD, DMAX><<<grid, kBlock, smem, s>>>(L);
  return cudaGetLastError();
}

template <int METHOD, int DMAX>
int max_active(void) {
  int n = 0;
  size_t smem = METHOD == MC_BASKET ? (size_t)(2 * DMAX + DMAX * DMAX) * sizeof(float) : 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mc_kernel<METHOD, DMAX>, kBlock, smem) !=
      cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

}  // namespace

cudaError_t launch_mc(McMethod m, const McLaunch& L, int grid, int max_d, cudaStream_t s) {
  if (grid <= 0) return cudaSuccess;
  switch (m) {
    case MC_EUR: return launch_one<MC_EUR, 4>(L, grid, s);
    case MC_ASIA: return launch_one<MC_ASIA, 4>(L, grid, s);
    case MC_BASKET:
      if (max_d <= 4) return launch_one<MC_BASKET, 4>(L, grid, s);
      if (max_d <= 8) return launch_one<MC_BASKET, 8>(L, grid, s);
      if (max_d <= 16) return launch_one<MC_BASKET, 16>(L, grid, s);
      if (max_d <= 32) return launch_one<MC_BASKET, 32>(L, grid, s);
      if (max_d <= 64) return launch_one<MC_BASKET, 64>(L, grid, s);
      return cudaErrorInvalidValue;
  }
  return cudaErrorInvalidValue;
}

int mc_max_active_blocks(McMethod m, int max_d) {
  switch (m) {
    case MC_EUR: return max_active<MC_EUR, 4>();
    case MC_ASIA: return max_active<MC_ASIA, 4>();
    case MC_BASKET:
      if (max_d <= 4) return max_active<MC_BASKET, 4>();
      if (max_d <= 8) return max_active<MC_BASKET, 8>();
      if (max_d <= 16) return max_active<MC_BASKET, 16>();
      if (max_d <= 32) return max_active<MC_BASKET, 32>();
      return max_active<MC_BASKET, 64>();
  }
  return 1;
}

}  // namespace pcf
