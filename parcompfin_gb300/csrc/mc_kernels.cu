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
// The kernels are issue-bound (Philox + Box-Muller + GBM is ~50 FP32/INT
// instructions against 3 SFU operations per path), so the control-variate
// sums are compiled in only when a launch asks for them (CV template flag).
//
// Reference loops these kernels replace:
//   European  src/mc_eur.cpp:22-26,  src/mc_eur_omp.cpp:24-27
//   Asian     src/mc_asia.cpp:26-39, src/mc_asia_omp.cpp:33-44
//   basket    src/mc_eur_multi.cpp:19-34 with include/mvn.h:42-82
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
template <bool CV>
__device__ __forceinline__ void eur_item(const McContract& C, int j, Moments<CV>& mo) {
  const long long nq = (C.N + 3) >> 2;
  const long long nfull = C.N >> 2;  // quads whose four paths are all < N
  const long long q0 = (long long)j * C.units_per_item + threadIdx.x;
  const int qpt = C.units_per_item / kBlock;
  const RngKey key{C.seed_lo, C.seed_hi, C.stream, TAG_EUR};
  const float a2 = C.a2 + C.l2S0;
  for (int k0 = 0; k0 < qpt; k0 += 4) {
    float cy = 0.f, cyy = 0.f, cg = 0.f, cgg = 0.f, cyg = 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
      const long long q = q0 + (long long)(k0 + kk) * kBlock;
      if (k0 + kk < qpt && q < nq) {
        const float4 z = normals4(draw_words(key, (uint64_t)q, 0u));
        float s[4] = {ex2_approx(fmaf(C.b2, z.x, a2)), ex2_approx(fmaf(C.b2, z.y, a2)),
                      ex2_approx(fmaf(C.b2, z.z, a2)), ex2_approx(fmaf(C.b2, z.w, a2))};
        float y[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) y[l] = payoff(C, s[l]);
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

// Asian: item j covers paths [j*U, (j+1)*U), U = units_per_item, U/256 per
// thread (path j*U + k*256 + thread); increment m uses lane m%4 of Philox block
// (x=path, y=m/4). log2(S/S0) is accumulated, S = S0 * 2^L.
// mode 0 (reference, src/mc_asia.cpp:31-35): I += S_m (c1 + c2 z_m) with S_m
//   the level before the step; A = I/M.
// mode 1: I += S_{m+1}; A = I/M (discrete mean of S_1..S_M).
// g = payoff of the geometric mean exp(sum_m w_m log S_m): mode 0 uses the
// trapezoid weights (w_M = 1/(2M), S_0's weight multiplies log S0/S0 = 0),
// mode 1 equal weights 1/M on S_1..S_M.
template <bool CV>
__device__ __forceinline__ void asia_item(const McContract& C, int j, Moments<CV>& mo) {
  const RngKey key{C.seed_lo, C.seed_hi, C.stream, TAG_ASIA};
  const int M = C.M;
  const float w = 1.f / (float)M;
  const int ppt = C.units_per_item / kBlock;
#pragma unroll 1
  for (int k = 0; k < ppt; ++k) {
    const long long n = (long long)j * C.units_per_item + (long long)k * kBlock + threadIdx.x;
    if (n >= C.N) break;
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
            if (CV) lg = fmaf(m == M - 1 ? C.w_last : w, L, lg);
          } else {
            L += fmaf(C.b2, zl, C.a2);
            I += C.S0 * ex2_approx(L);
            if (CV) lg = fmaf(w, L, lg);
          }
        }
      }
    }
    const float Y = payoff(C, I * w);
    const float G = CV ? payoff(C, C.S0 * ex2_approx(lg)) : 0.f;
    mo.add(Y, G);
  }
}

// Basket of d <= DMAX assets, one path. Asset a's normal is lane a%4 of
// Philox block (x=path, y=a/4). x = Lz with the correlation factor staged in
// shared memory; log2 S_a = l0_a + v_a x_a; y = payoff(mean_a S_a),
// g = payoff(2^(mean_a log2 S_a)). mode 0: the factor is lower triangular
// (Cholesky); mode 1: a full factor (eigen-decomposition fallback).
template <int DMAX, bool CV>
__device__ __forceinline__ void basket_path(const McContract& C, const float* fb, long long n,
                                            Moments<CV>& mo) {
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
  const float Y = payoff(C, bsk * inv_d);
  const float G = CV ? payoff(C, ex2_approx(geo * inv_d)) : 0.f;
  mo.add(Y, G);
}

// Basket item j covers paths [j*U, (j+1)*U), U = units_per_item: U/256 paths
// per thread (path j*U + k*256 + thread) for baskets of up to 8 assets, one
// path per thread for larger ones (their path loop would hold the whole
// unrolled factor product in registers).
template <int DMAX, bool CV>
__device__ __forceinline__ void basket_item(const McContract& C, int j, const float* fb,
                                            Moments<CV>& mo) {
  const long long n0 = (long long)j * C.units_per_item + threadIdx.x;
  if (DMAX <= 8) {
    const int ppt = C.units_per_item / kBlock;
    for (int k = 0; k < ppt; ++k) {
      const long long n = n0 + (long long)k * kBlock;
      if (n >= C.N) break;
      basket_path<DMAX, CV>(C, fb, n, mo);
    }
  } else if (n0 < C.N) {
    basket_path<DMAX, CV>(C, fb, n0, mo);
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

// Persistent launch: blocks take work items from a queue in increasing
// order. The next ticket is taken while the current item runs, and the item's
// contract is found in one round: the contract is the block's previous one or
// one of the next 255, so each thread tests one candidate (a binary search
// covers longer jumps).
template <int METHOD, int DMAX, bool CV>
__global__ void __launch_bounds__(kBlock) mc_kernel(McLaunch L) {
  __shared__ DF sh[32 * kMoments];
  __shared__ int s_item[2];
  __shared__ int s_c;
  extern __shared__ float s_fb[];
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
      eur_item<CV>(C, j, mo);
    } else if (METHOD == MC_ASIA) {
      asia_item<CV>(C, j, mo);
    } else {
      if (loaded != c) {  // the previous item's readers are past the final barrier
        const int d = C.M;
        const float* src = L.basket_data + C.basket_off;
        for (int i = threadIdx.x; i < 2 * d + d * d; i += kBlock) s_fb[i] = src[i];
        __syncthreads();
        loaded = c;
      }
      basket_item<DMAX, CV>(C, j, s_fb, mo);
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

constexpr size_t basket_smem(int dmax) { return (size_t)(2 * dmax + dmax * dmax) * sizeof(float); }

template <int METHOD, int DMAX, bool CV>
cudaError_t launch_one(const McLaunch& L, int grid, cudaStream_t s) {
  const size_t smem = METHOD == MC_BASKET ? basket_smem(DMAX) : 0;
  mc_kernel<METHOD, DMAX, CV><<<grid, kBlock, smem, s>>>(L);
  return cudaGetLastError();
}

template <int METHOD, int DMAX>
cudaError_t launch_cv(const McLaunch& L, int grid, cudaStream_t s) {
  return L.cv ? launch_one<METHOD, DMAX, true>(L, grid, s)
              : launch_one<METHOD, DMAX, false>(L, grid, s);
}

template <int METHOD, int DMAX>
int max_active(void) {
  int n = 0;
  const size_t smem = METHOD == MC_BASKET ? basket_smem(DMAX) : 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, mc_kernel<METHOD, DMAX, true>, kBlock,
                                                    smem) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

}  // namespace

cudaError_t launch_mc(McMethod m, const McLaunch& L, int grid, int max_d, cudaStream_t s) {
  if (grid <= 0) return cudaSuccess;
  switch (m) {
    case MC_EUR: return launch_cv<MC_EUR, 4>(L, grid, s);
    case MC_ASIA: return launch_cv<MC_ASIA, 4>(L, grid, s);
    case MC_BASKET:
      if (max_d <= 4) return launch_cv<MC_BASKET, 4>(L, grid, s);
      if (max_d <= 8) return launch_cv<MC_BASKET, 8>(L, grid, s);
      if (max_d <= 16) return launch_cv<MC_BASKET, 16>(L, grid, s);
      if (max_d <= 32) return launch_cv<MC_BASKET, 32>(L, grid, s);
      if (max_d <= 64) return launch_cv<MC_BASKET, 64>(L, grid, s);
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
  eur_item<true>(C, j, mo);
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
  const McContract C = make_eur(S0, E, r, sigma, T, N, payoff_fun, seed, 0);
  if (C.items > kNoAllocMaxItems)
    return set_error(PCF_EINVAL, "N = %lld needs %d work items; the fixed scratch holds %d", N,
                     C.items, kNoAllocMaxItems);
  cudaStream_t s = (cudaStream_t)stream;
  st = cuda_status(cudaMemsetAsync(scratch, 0, sizeof(unsigned), s), "memset no-alloc ticket");
  if (st) return st;
  mc_eur_noalloc_kernel<<<C.items, kBlock, 0, s>>>(C, scratch, d_sums);
  return cuda_status(cudaGetLastError(), "no-alloc kernel launch");
}
