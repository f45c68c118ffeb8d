// The plan object behind pcf_plan_* and the serving loop (host side).
#pragma once
#include <vector>

#include "pcf_api_internal.h"

namespace pcf {

struct Group {  // one persistent Monte Carlo launch
  McMethod method;
  int max_d = 0;
  int block = kBlock;         // threads per block (the tuning table's, for this group)
  bool tensor = false;        // baskets: the tensor-core kernel
  std::vector<int> req;       // request index of each contract (queue order)
  std::vector<McContract> cs;
  std::vector<float> fb;
  std::vector<int> start;     // item prefix, size C+1
  McLaunch L{};
  int grid = 0;
};

}  // namespace pcf

struct pcf_plan {
  pcf_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  int n = 0;
  std::vector<pcf::Group> groups;
  std::vector<long long> npaths;
  std::vector<double> mu_g, disc;
  std::vector<int> use_cv;
  std::vector<int> out_slot;  // request -> row of the device out table
  void* d_mem = nullptr;      // owned device memory (NULL when built in caller memory)
  void* h_own = nullptr;      // owned pinned memory
  double* h_out = nullptr;
  unsigned* d_tickets = nullptr;
  size_t tickets_bytes = 0;
  double* d_out = nullptr;
  // American requests: priced by an LSM batch; two flag words each (wait gave
  // up, singular dates) live in the ticket region, so the per-launch memset
  // clears them.
  pcf::LsmBatch* lsm = nullptr;
  std::vector<int> amer;               // request indices
  std::vector<pcf_mc_request> amer_q;  // their parameters (for the estimators)
  int* d_amer_flags = nullptr;
  int* h_amer_flags = nullptr;
  // CUDA graph replay: the second launch captures the launch sequence, later
  // launches replay it. graph_mode 0 never captures.
  // Fork/join: the LSM cluster launches run on `side`, concurrently with the
  // Monte Carlo groups on `stream`, so each fills the other's tail.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int graph_mode = 1;
  long long launches_done = 0;
  bool graph_failed = false;
  cudaGraphExec_t gexec = nullptr;
  long long graph_kernels = 0;
};

namespace pcf {

// Builds a plan on stream s. mem == NULL: owns its memory, uploads
// synchronously. Otherwise: takes memory from mem (no allocation) and only
// queues the upload. path0 (optional, one per request): the request's paths
// are paths [path0, path0 + N) of its stream, so a run can continue an
// earlier one and the two sets of sums add up (European, Asian and basket;
// path0 must be a multiple of 4 and is ignored for American requests).
int plan_build(pcf_ctx* c, int n, const pcf_mc_request* reqs, cudaStream_t s, ExtMem* mem,
               pcf_plan** out, const long long* path0 = nullptr);
int plan_launch(pcf_plan* p);
// Queues the device-to-host copy of the results (no wait).
int plan_fetch(pcf_plan* p);
// Estimators from the fetched sums (after the stream has reached plan_fetch).
int plan_fill_results(pcf_plan* p, pcf_mc_result* results);

}  // namespace pcf
