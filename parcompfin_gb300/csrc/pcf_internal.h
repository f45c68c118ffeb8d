// Internal host/device interface between the C-ABI layer (pcf_api.cpp) and
// the kernel translation units. Plain C++ structs only; nothing here crosses
// the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pcf {

// Moment sums every Monte Carlo kernel returns per contract:
// {sum y, sum y^2, sum g, sum g^2, sum y*g}, y the undiscounted payoff and g
// the kernel's control variate.
constexpr int kMoments = 5;
constexpr int kBlock = 256;  // threads per work item of the MC kernels (the default)

// One Monte Carlo contract as the kernels see it. Per-path arithmetic is
// FP32; the drift/vol terms are pre-multiplied by log2(e) on the host so each
// step is one FMA and one ex2.
struct McContract {
  float S0, K, pf;       // spot, strike, +1 call / -1 put
  float a2, b2;          // log2-domain drift and vol per step (European: per maturity)
  float c1, c2;          // Asian running-sum coefficients 1 + r dt/2, s sqrt(dt)/2
  float w_last;          // Asian: geometric weight of the last date
  int M;                 // steps (Asian), assets (basket)
  int mode;              // Asian: 0 reference running sum, 1 discrete mean
  int units_per_item;    // quads (European) or paths (Asian, basket) per work item
  int items;             // work items of this contract
  long long N;           // paths
  uint32_t seed_lo, seed_hi, stream, pad;
  int basket_off;        // basket: offset of this contract's factor block
  float nK;              // -pf * K: payoff = max(pf * S + nK, 0)
  float l2S0;            // log2(S0)
  float pad2;
  long long x0;          // first Philox x coordinate: path quad (European) or path, so a
                         // contract can continue the paths of an earlier run
};

// Basket factor block (device): per asset log2(S0_a) + (r - s_a^2/2) T log2e,
// s_a * ts * log2e, then the d x d lower Cholesky factor, row-major, FP32.
struct McLaunch {
  const McContract* contracts;
  const int* item_start;   // exclusive prefix of items per contract, size C+1
  const float* basket_data;
  int ncontracts;
  int total_items;
  unsigned int* queue;     // persistent mode: next item (reset to 0 by the host)
  double* partial;         // total_items * kMoments slots of 8 bytes (double-float pairs)
  unsigned int* tickets;   // per contract, re-armed by the finaliser
  double* out;             // ncontracts * kMoments
  int persistent;
  int cv;                  // accumulate the control-variate sums (else they are 0)
};

enum McMethod { MC_EUR = 0, MC_ASIA = 1, MC_BASKET = 2 };

// Launchers (mc_kernels.cu). `grid` = blocks to launch (items, or the
// persistent block count); `block` = threads per block (128, 256 or 512; the
// contracts' units_per_item are multiples of it). `tensor`: baskets of 17 to
// 32 assets run the tensor-core kernel (block fixed at 128 threads) instead
// of the CUDA-core one; above 32 assets the tensor-core kernel always runs.
cudaError_t launch_mc(McMethod m, const McLaunch& L, int grid, int max_d, int block, bool tensor,
                      cudaStream_t s);
int mc_max_active_blocks(McMethod m, int max_d, int block, bool tensor);

}  // namespace pcf
