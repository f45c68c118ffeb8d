// Device building blocks shared by every pricing kernel of the engine:
// the Philox4x32-10 generator, the FP32 Box-Muller mapping, compensated FP32
// accumulation, FP64 block reductions with a deterministic "last block"
// finaliser, and a bounded group barrier for persistent kernels.
//
// The random stream is part of the engine's contract: a draw is a pure
// function of (seed, stream, tag, x, y, lane), so any path can be regenerated
// on the host by an FP64 harness fed the identical uniforms.
//   key     = (seed & 0xffffffff, seed >> 32)
//   counter = (x & 0xffffffff, y, stream, (tag << 16) | ((x >> 32) & 0xffff))
// Philox4x32-10 follows Salmon et al., "Parallel Random Numbers: As Easy as
// 1, 2, 3" (SC'11). The reference draws with std::mt19937 +
// std::normal_distribution (src/mc_eur.cpp:17-20); that generator is
// sequential, so a reproducible counter-based stream replaces it.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pcf {

enum : uint32_t { TAG_EUR = 1, TAG_ASIA = 2, TAG_BASKET = 3, TAG_AMER = 4 };

struct RngKey {
  uint32_t k0, k1, stream, tag;
};

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    // The high and low words as two 32-bit multiplies (the same values as
    // one 64-bit product; measured 1 % faster on the Asian book).
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

__device__ __forceinline__ uint4 draw_words(const RngKey& k, uint64_t x, uint32_t y) {
  return philox4x32_10(
      make_uint4((uint32_t)x, y, k.stream, (k.tag << 16) | ((uint32_t)(x >> 32) & 0xffffu)),
      k.k0, k.k1);
}

// u = (2*(w >> 9) + 1) * 2^-24, exactly: 1.m - (1 - 2^-24) is an exact
// subtraction (Sterbenz), so no integer-to-float conversion is needed.
__device__ __forceinline__ float uniform_open(uint32_t w) {
  return __uint_as_float(0x3f800000u | (w >> 9)) - 0.99999994f;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sin_approx(float x) {
  float y;
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float cos_approx(float x) {
  float y;
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// The Box-Muller angle pi (2 u - 1) of u = uniform_open(w) in one FMA:
// f = 2 + (w >> 9) 2^-22 (exact, in [2, 4)) and pi (2 u - 1) = pi f - 3 pi +
// pi 2^-23 in exact arithmetic.
__device__ __forceinline__ float bm_angle(uint32_t w) {
  const float f = __uint_as_float(0x40000000u | (w >> 9));
  return fmaf(3.14159265359f, f, -9.42477758f);  // -3 pi + pi 2^-23, rounded
}

// Box-Muller on two uniform pairs: (z0,z1) from (w0,w1), (z2,z3) from (w2,w3).
// z = sqrt(-2 ln u0) * (cos, sin)(pi * (2 u1 - 1)).
__device__ __forceinline__ float4 normals4(uint4 w) {
  const float kNeg2Ln2 = -1.38629436112f;  // -2 ln 2: -2 ln u = -2 ln2 * log2 u
  const float u0 = uniform_open(w.x), u2 = uniform_open(w.z);
  const float r0 = sqrt_approx(kNeg2Ln2 * lg2_approx(u0));
  const float r1 = sqrt_approx(kNeg2Ln2 * lg2_approx(u2));
  const float t0 = bm_angle(w.y);
  const float t1 = bm_angle(w.w);
  return make_float4(r0 * cos_approx(t0), r0 * sin_approx(t0), r1 * cos_approx(t1),
                     r1 * sin_approx(t1));
}

// normals4 with the two pairs side by side in packed FP32x2 arithmetic: each
// lane rounds exactly as the scalar operation, so the normals are the same
// bits; the Monte Carlo kernels, issue-bound, spend fewer instructions on
// them (the Longstaff-Schwartz forward pass, bound by HBM writes, keeps the
// scalar form, which measured faster there).
__device__ __forceinline__ float4 normals4_x2(uint4 w) {
  const float kNeg2Ln2 = -1.38629436112f;
  const float2 f = __fadd2_rn(make_float2(__uint_as_float(0x3f800000u | (w.x >> 9)),
                                          __uint_as_float(0x3f800000u | (w.z >> 9))),
                              make_float2(-0.99999994f, -0.99999994f));  // uniform_open
  const float2 l = __fmul2_rn(make_float2(kNeg2Ln2, kNeg2Ln2),
                              make_float2(lg2_approx(f.x), lg2_approx(f.y)));
  const float2 r = make_float2(sqrt_approx(l.x), sqrt_approx(l.y));
  const float2 t = __ffma2_rn(make_float2(3.14159265359f, 3.14159265359f),
                              make_float2(__uint_as_float(0x40000000u | (w.y >> 9)),
                                          __uint_as_float(0x40000000u | (w.w >> 9))),
                              make_float2(-9.42477758f, -9.42477758f));  // bm_angle
  const float2 c = __fmul2_rn(r, make_float2(cos_approx(t.x), cos_approx(t.y)));
  const float2 s = __fmul2_rn(r, make_float2(sin_approx(t.x), sin_approx(t.y)));
  return make_float4(c.x, s.x, c.y, s.y);
}

__device__ __forceinline__ float lane4(const float4& v, int l) {
  return l == 0 ? v.x : (l == 1 ? v.y : (l == 2 ? v.z : v.w));
}

// Kahan-compensated FP32 sum: FP64 is scarce on GB300, so no per-path FP64
// arithmetic; value() widens once at the end.
struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Double-float value hi + lo (two FP32s, ~48 significant bits). GB300's FP64
// pipe runs at a small fraction of its FP32 rate, so reductions combine
// partial sums with the error-free TwoSum transformation in FP32 and widen
// to FP64 only once at the end.
struct DF {
  float hi, lo;
};

__device__ __forceinline__ DF df_add(DF a, DF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);  // TwoSum error of a.hi + b.hi
  e += a.lo + b.lo;
  const float hi = s + e;
  return DF{hi, e - (hi - s)};
}

__device__ __forceinline__ DF df_add_f(DF a, float b) {  // df_add(a, {b, 0})
  const float s = a.hi + b;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b - bb);
  e += a.lo;
  const float hi = s + e;
  return DF{hi, e - (hi - s)};
}

// Double-float product: the FP32 product of the high parts, its exact
// rounding error (an FMA) plus the cross terms, renormalised. The explicit
// _rn operations keep the compiler from contracting them into FMAs.
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float hi = __fadd_rn(p, e);
  return DF{hi, __fsub_rn(e, __fsub_rn(hi, p))};
}

__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }

__device__ __forceinline__ DF shfl_df(DF v, int src) {
  return DF{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

__device__ __forceinline__ DF shfl_xor_df(DF v, int o) {
  return DF{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

__device__ __forceinline__ DF df_of(const KSum& k) {  // k.s - k.c, exactly
  const float s = k.s, m = -k.c;
  const float hi = s + m;
  const float bb = hi - s;
  return DF{hi, (s - (hi - bb)) + (m - bb)};
}

__device__ __forceinline__ double df_value(DF a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ DF warp_sum_df(DF v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DF w;
    w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v = df_add(v, w);
  }
  return v;
}

// Sums K double-floats over the block; thread 0 gets the totals. `sh` must
// hold 32*K DFs. Deterministic for a fixed block size.
template <int K>
__device__ __forceinline__ void block_sum_df(DF (&v)[K], DF* sh, DF (&out)[K]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_sum_df(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) sh[wid * K + k] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      DF x = lane < nw ? sh[lane * K + k] : DF{0.f, 0.f};
      out[k] = warp_sum_df(x);
    }
  }
  __syncthreads();
}

// Deterministic last-block finaliser over double-float partials: each block
// stores its K totals as (hi, lo) pairs in partial[block_id*K..]; the block
// that takes the last ticket sums all partials in block order with one warp,
// writes out[k] in FP64 and re-arms the ticket.
template <int K>
__device__ __forceinline__ void grid_finalize_df(const DF (&tot)[K], float2* partial,
                                                 unsigned int* ticket, double* out,
                                                 int nblocks, int block_id) {
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k)
      partial[(size_t)block_id * K + k] = make_float2(tot[k].hi, tot[k].lo);
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    am_last = (t == (unsigned int)nblocks - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      DF x{0.f, 0.f};
      for (int b = lane; b < nblocks; b += 32) {
        const float2 p = __ldcg(partial + (size_t)b * K + k);
        x = df_add(x, DF{p.x, p.y});
      }
      x = warp_sum_df(x);
      if (lane == 0) out[k] = df_value(x);
    }
    if (lane == 0) *ticket = 0u;
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums K doubles over the block; thread 0 gets the totals in out[]. `sh` must
// hold 32*K doubles. Deterministic for a fixed block size.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* sh, double (&out)[K]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) sh[wid * K + k] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double x = lane < nw ? sh[lane * K + k] : 0.0;
      x = warp_sum(x);
      out[k] = x;
    }
  }
  __syncthreads();
}

// Deterministic grid reduction by the last block to finish: each block writes
// its K partials to partial[blockIdx*K..], the block that takes the last
// ticket sums all partials in block order with one warp and writes out[K],
// then re-arms the ticket for the next launch. Call with the block's totals
// in tot[] on thread 0. Returns true in the finalising block.
template <int K>
__device__ __forceinline__ void grid_finalize(const double (&tot)[K], double* partial,
                                              unsigned int* ticket, double* out,
                                              int nblocks, int block_id) {
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) partial[(size_t)block_id * K + k] = tot[k];
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    am_last = (t == (unsigned int)nblocks - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double x = 0.0;
      for (int b = lane; b < nblocks; b += 32) x += ((volatile double*)partial)[(size_t)b * K + k];
      x = warp_sum(x);
      if (lane == 0) out[k] = x;
    }
    if (lane == 0) *ticket = 0u;
  }
}

// ---- TMA bulk copies (cp.async.bulk) completed on an mbarrier ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
// Makes mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Orders this thread's earlier generic-proxy global writes before later
// async-proxy (TMA) reads of the same memory.
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// Global -> shared bulk copy; src, dst 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Waits for the mbarrier phase with the given parity; gives up after
// `limit` polls and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// mbar_wait without the hardware suspend of try_wait: polls test_wait, for
// waits that usually end within a few hundred cycles. Bounded.
__device__ __forceinline__ bool mbar_poll(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// ---- exchanges between the CTAs of a thread-block cluster ----
// Address of the same shared-memory object in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t cluster_map(const void* p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
// Asynchronous store of 16 bytes into another CTA's shared memory; its
// completion counts 16 bytes against that CTA's mbarrier (complete_tx), so
// the sender needs no fence and the receiver sees the data once the phase
// completes.
__device__ __forceinline__ void st_async_v4(uint32_t addr, float4 v, uint32_t bar) {
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, "
      "[%5];" ::"r"(addr),
      "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(bar)
      : "memory");
}

// Group barrier for a persistent kernel whose blocks are co-resident (the
// host launches it cooperatively). `counter` only grows, so no reset race:
// arrival number a (0-based) waits until the count reaches (a/G + 1)*G. The
// wait is bounded: after `limit` polls it raises *err and returns false.
__device__ __forceinline__ bool group_barrier(unsigned int* counter, unsigned int G,
                                              int* err, unsigned int limit) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    __threadfence();
    const unsigned int a = atomicAdd(counter, 1u);
    const unsigned int target = (a / G + 1u) * G;
    unsigned int polls = 0;
    while (true) {
      const unsigned int c = *((volatile unsigned int*)counter);
      if ((int)(c - target) >= 0) break;
      if (*((volatile int*)err) != 0 || ++polls > limit) {
        atomicExch(err, 1);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

}  // namespace pcf
