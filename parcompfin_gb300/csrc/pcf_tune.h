// Work shapes of the kernels and the autotuner that picks them
// (pcf_autotune in include/pcf.h).
//
// A work shape is how much work one block or one thread takes: the block
// size of a Monte Carlo launch, the paths (or path quads) each thread prices
// in one work item, the tiles of 128 paths per item of the tensor-core
// basket kernel, and the cluster size and slice of the Longstaff-Schwartz
// cluster launch. Work items are sized from the contract and this table
// alone, so a contract's sums do not depend on what else is in its batch;
// the table changes only when pcf_autotune runs (or a tuning cache is
// loaded), and the built-in values are the ones measured by hand on GB300.
#pragma once
#include <string>

namespace pcf {

constexpr int kTuneEurClasses = 4;    // log2 N < 18, < 22, < 26, >= 26
constexpr int kTuneAsiaClasses = 4;   // M <= 16, <= 64, <= 256, > 256
constexpr int kTuneBasketClasses = 5; // d <= 4, <= 8, <= 16, <= 32, <= 64
constexpr int kTuneLsmClasses = 8;    // log2 N <= 14, 15, ..., 20, >= 21

struct TuneTable {
  int eur_block = 256;
  int eur_items[kTuneEurClasses] = {32, 32, 32, 32};  // target work items per contract
  int eur_max_quads = 64;                             // quads per thread, at most
  int asia_block = 256;
  int asia_steps[kTuneAsiaClasses] = {512, 512, 512, 512};  // monitoring steps per thread per item
  // Baskets on the CUDA cores: d <= 4, <= 8, <= 16, and 17..32 where those
  // are not routed to the tensor cores.
  int basket_block[4] = {256, 256, 256, 256};
  int basket_ppt[4] = {16, 8, 8, 4};  // paths per thread per item
  int tc_tiles[2] = {8, 8};           // 128-path tiles per item, tensor-core kernel (d <= 32, <= 64)
  // Baskets of at least this many assets take the tensor cores: measured at
  // 2^21 paths, the CUDA cores win at 17 and 20 assets, the tensor cores from
  // 24 on.
  int tc_min_d = 24;
  // Longstaff-Schwartz cluster launch: 0 takes the smallest cluster whose
  // CTAs cover the contract two to an SM; +1 doubles the cluster (half the
  // slice), -1 halves it (twice the slice, one CTA per SM if it must).
  int lsm_shift[kTuneLsmClasses] = {0, 0, 0, 0, 0, 0, 0, 0};
  bool tuned = false;
};

int eur_class(long long N);
int asia_class(int M);
int basket_class_of(int d);
int lsm_class(long long N);

// The table in force on a device (the built-in one until pcf_autotune ran
// on it, or a tuning cache named by PCF_TUNE_CACHE was loaded for it).
TuneTable tune_table(int device);
void tune_set(int device, const TuneTable& t);
void tune_reset(int device);
std::string tune_json(const TuneTable& t);

// Work sizes from the table.
int eur_quads_per_thread(long long N, const TuneTable& t);
int asia_paths_per_thread(int M, const TuneTable& t);
bool basket_tensor(int d, const TuneTable& t);         // the tensor-core kernel prices it
int basket_units_per_item(int d, const TuneTable& t);  // paths per work item
int mc_block(int method, int d, const TuneTable& t);   // threads per block of a launch

}  // namespace pcf
