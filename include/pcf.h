/* pcf.h -- C ABI of the GB300 option-pricing engine (libpcf.so).
 *
 * Drop-in boundary for the pricing functions of moledoc/parcompfin. The
 * reference exposes one `double method(...)` C++ function per pricing method,
 * called from each program's main() between two clock reads; every entry
 * point below replaces one of them (file:line cited on each) and keeps its
 * parameters (S0, E, r, sigma, T, N, M, payoff_fun, assets, rho) in the same
 * order and meaning. payoff_fun is +1 for a call and -1 for a put, as in
 * include/common.h:56-60.
 *
 * Conventions:
 *   - every function returns a status (PCF_OK or a negative PCF_E* code);
 *     no C++ exception crosses the ABI. The reference throws
 *     std::invalid_argument for a bad payoff (src/mc_eur.cpp:42), an odd path
 *     count for the LSM paths (include/common.h:180) and a singular regression
 *     (include/common.h:115-117); those map to PCF_EINVAL / PCF_ESINGULAR.
 *   - results are written to caller-owned host memory; the library owns all
 *     device memory through a context.
 *   - ctx may be NULL: the calling thread's default context on device 0 is
 *     created on first use.
 *   - one context serves one host thread at a time (or serialise externally).
 *   - the Monte Carlo paths draw from a counter-based Philox4x32-10 stream
 *     keyed by `seed`, so a call is reproducible; the reference reseeds from
 *     time() (src/mc_eur.cpp:19) and is not.
 */
#ifndef PCF_H_
#define PCF_H_

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PCF_API __attribute__((visibility("default")))
#else
#define PCF_API
#endif

#define PCF_OK 0
#define PCF_EINVAL (-1)     /* bad parameter (payoff_fun not +/-1, N < 1, ...) */
#define PCF_ENOMEM (-2)     /* device or pinned allocation failed / over budget */
#define PCF_ESINGULAR (-3)  /* LSM normal equations with determinant <= 0 */
#define PCF_ETIMEOUT (-4)   /* a bounded device wait gave up */
#define PCF_ECUDA (-5)      /* CUDA runtime error */
#define PCF_ENODEV (-6)     /* no CUDA device */
#define PCF_PENDING 1       /* not an error: a served request is not finished yet */

typedef struct pcf_ctx pcf_ctx;

/* Result of a Monte Carlo price. `price`/`std_error` are the estimate that
 * was asked for: the plain discounted mean (use_cv = 0, what the reference
 * returns) or the control-variate estimate (use_cv = 1). `sums` are the raw
 * moment sums {sum y, sum y^2, sum g, sum g^2, sum y*g} over n_paths paths,
 * y the undiscounted payoff (the discounted cash flow for mc_amer) and g the
 * method's control variate. */
typedef struct pcf_mc_result {
  double price;
  double std_error;
  double price_plain;
  double std_error_plain;
  double price_cv;        /* NaN when use_cv = 0 */
  double std_error_cv;    /* NaN when use_cv = 0 */
  double cv_beta;
  double cv_mean;         /* exact E[g] */
  double discount;        /* factor applied to the mean of y */
  double sums[5];
  long long n_paths;
} pcf_mc_result;

/* Library version string. */
PCF_API const char* pcf_version(void);
/* Message for a status code. */
PCF_API const char* pcf_strerror(int status);
/* Details of the last error on this thread (empty if none). */
PCF_API const char* pcf_last_error(void);

/* Context: a CUDA stream plus device and pinned scratch that persists across
 * calls. Replaces nothing in the reference (it has no device state). */
PCF_API int pcf_ctx_create(int device, pcf_ctx** out);
PCF_API int pcf_ctx_destroy(pcf_ctx* ctx);
/* The context's cudaStream_t, for callers that time or order work on it. */
PCF_API void* pcf_ctx_stream(pcf_ctx* ctx);
/* Number of kernels this context has launched so far. */
PCF_API long long pcf_ctx_launch_count(pcf_ctx* ctx);
/* Frees the device and pinned memory the context keeps between calls (the
 * scratch arena, the resident LSM path matrix, the binomial tables, the
 * serving slots); the next call that needs them allocates them again. */
PCF_API int pcf_ctx_release(pcf_ctx* ctx);
/* Caps each device buffer the context allocates (the scratch arena, an LSM
 * path matrix, a plan, the serving slots' reservation) at `bytes`; a call
 * that would need more returns PCF_ENOMEM. 0 removes the cap. Buffers held
 * already are not shrunk: call pcf_ctx_release first. */
PCF_API int pcf_ctx_set_memory_limit(pcf_ctx* ctx, unsigned long long bytes);

/* European option, single-step GBM Monte Carlo.
 * Replaces double mc_eur(S0,E,r,sigma,T,N,payoff_fun), src/mc_eur.cpp:5-27
 * (OpenMP: src/mc_eur_omp.cpp:5-30). Control variate g = S_T. */
PCF_API int pcf_mc_eur(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T,
               long long N, int payoff_fun, unsigned long long seed, int use_cv,
               pcf_mc_result* out);

/* Fixed-strike arithmetic-average Asian option, M monitoring steps.
 * Replaces double mc_asia(S0,E,r,sigma,T,N,M,payoff_fun), src/mc_asia.cpp:5-40
 * (OpenMP: src/mc_asia_omp.cpp:5-48). mode 0 reproduces the reference's
 * running sum I += S (1 + r dt/2 + sigma dB/2) (src/mc_asia.cpp:33);
 * mode 1 averages S_1..S_M. Control variate: the geometric average payoff. */
PCF_API int pcf_mc_asia(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T,
                long long N, int M, int payoff_fun, int mode, unsigned long long seed,
                int use_cv, pcf_mc_result* out);

/* Equal-weight basket of `assets` assets with common S0 and sigma and
 * equicorrelation rho, single step.
 * Replaces double mc_eur(S0,E,r,sigma,T,N,payoff_fun,assets,rho),
 * src/mc_eur_multi.cpp:6-35 with mvnorm() of include/mvn.h:42-82. Like the
 * reference, the correlated draws are not scaled by sqrt(T) (include/mvn.h:55-60,
 * src/mc_eur_multi.cpp:30). Control variate: the geometric basket payoff. */
PCF_API int pcf_mc_eur_multi(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T,
                     long long N, int payoff_fun, int assets, double rho,
                     unsigned long long seed, int use_cv, pcf_mc_result* out);

/* General basket: per-asset S0[d] and sigma[d], correlation corr[d*d]
 * (row-major, symmetric positive semi-definite), 1 <= d <= 64. The factor is
 * Cholesky, or the eigen square root when Cholesky fails (include/mvn.h:63-76).
 * scale_by_sqrt_T = 1 scales the draws by sqrt(T) (a GBM basket); 0 keeps the
 * reference's unscaled draws. Extension of src/mc_eur_multi.cpp:6-35. */
PCF_API int pcf_mc_basket(pcf_ctx* ctx, int d, const double* S0, const double* sigma,
                  const double* corr, double r, double T, double E, long long N,
                  int payoff_fun, int scale_by_sqrt_T, unsigned long long seed, int use_cv,
                  pcf_mc_result* out);

/* American option by Longstaff-Schwartz least squares, M exercise dates,
 * antithetic path pairs (n, n + N/2); N must be even.
 * Replaces double mc_amer(S0,E,r,sigma,T,N,M,payoff_fun), src/mc_amer.cpp:5-114
 * (OpenMP: src/mc_amer_omp.cpp:5-117; paths: include/common.h:168-208).
 * ref_exercise = 0 exercises at payoff(S) (correct LSM); 1 reproduces the
 * reference's exercise value payoff(S - E, E) of src/mc_amer.cpp:100, which
 * makes its puts far too high. price = max(payoff(S0), mean discounted cash
 * flow) as src/mc_amer.cpp:113. Control variate (a martingale, mean =
 * Black-Scholes): with ref_exercise = 0, the European price at the path's
 * exercise date tau discounted to time 0 (the discounted payoff at T for a
 * path held to T); with ref_exercise = 1, whose exercise value does not
 * identify S_tau, the discounted European payoff at T. */
PCF_API int pcf_mc_amer(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T,
                        long long N, int M, int payoff_fun, int ref_exercise,
                        unsigned long long seed, int use_cv, pcf_mc_result* out);

/* pcf_mc_amer (use_cv = 1) plus an audit record of the sweep, for checking
 * the GPU's exercise policy against an FP64 re-run on the host. Any of the
 * buffers may be NULL:
 *   coef[M*4]  per date d (index d = 1..M-1; index 0 unused) {mode, c0, c1,
 *              c2}: mode 0 skipped (no in-the-money path, or a singular
 *              system), 1 at most two in-the-money paths, 2 the regression
 *              continuation value c0 + c1 u + c2 u^2 with
 *              u = payoff_fun (S - E) / E;
 *   sums[M*8]  the regression sums of date d as the solve saw them
 *              {n, sum u, u^2, u^3, u^4, y, y u, y u^2}, y the cash flow
 *              discounted to date d;
 *   tau[N]     each path's exercise date (M: held to T); paths p and
 *              p + N/2 are antithetic;
 *   u[M*N]     the FP32 path matrix: row m-1 holds max(u, 0) at date m
 *              (only paths in the money, u > 0, enter the sweep).
 * Has no counterpart in the reference. */
PCF_API int pcf_mc_amer_audit(pcf_ctx* ctx, double S0, double E, double r, double sigma,
                              double T, long long N, int M, int payoff_fun, int ref_exercise,
                              unsigned long long seed, pcf_mc_result* out, float* coef,
                              double* sums, unsigned short* tau, float* u);

/* Test hook for the failure paths (no counterpart in the reference): while
 * extra_arrivals > 0, the cooperative group barriers of pcf_mc_amer (plain
 * cooperative grid only: the cluster forms are not used while it is set) and
 * pcf_binom_vanilla wait for extra_arrivals blocks more than the grid holds,
 * so they cannot complete, and give up after poll_limit polls; the call then
 * returns PCF_ETIMEOUT. Waits on bulk copies keep their full limit, so no
 * block leaves with a copy in flight. extra_arrivals = 0 restores normal
 * operation; the counters are reset by every call. */
PCF_API int pcf_ctx_set_test_barrier(pcf_ctx* ctx, unsigned extra_arrivals, unsigned poll_limit);

/* European option by the closed binomial sum on the reference's
 * beta-parametrised lattice (u = beta + sqrt(beta^2 - 1), d = 1/u).
 * Replaces double binom(S0,E,r,sigma,T,N,payoff_fun), src/binom_embar.cpp:5-50
 * (OpenMP: src/binom_embar_omp.cpp:5-53), with comb() of include/common.h:63-72.
 * mode 0 reproduces the reference's FP64 result term by term, including the
 * rounding of its sequential log C(N,i) accumulator (parity 1e-10 relative);
 * mode 1 computes each binomial weight accurately (Loader's saddle-point
 * formula) and so differs from the reference by the reference's own
 * rounding drift. 1 <= N <= 1,000,000. */
typedef struct pcf_binom_contract {
  double S0, E, r, sigma, T;
  int N;
  int payoff_fun;
} pcf_binom_contract;

PCF_API int pcf_binom_embar(pcf_ctx* ctx, double S0, double E, double r, double sigma, double T,
                            int N, int payoff_fun, int mode, double* price);
/* n contracts of uneven N in one launch; prices[n]. */
PCF_API int pcf_binom_embar_batch(pcf_ctx* ctx, int n, const pcf_binom_contract* contracts,
                                  int mode, double* prices);

/* European or American option by backward induction on the same lattice.
 * Replaces double binom(S0,E,r,sigma,T,N,payoff_fun) of
 * src/binom_vanilla_eur.cpp:5-39 (american = 0) and
 * src/binom_vanilla_amer.cpp:5-40 (american = 1): bit for bit the reference's
 * FP64 result. One cooperative launch; 1 <= N <= 2,000,000. */
PCF_API int pcf_binom_vanilla(pcf_ctx* ctx, double S0, double E, double r, double sigma,
                              double T, int N, int payoff_fun, int american, double* price);

/* European option, single-step GBM Monte Carlo, with no memory allocation.
 * Has no counterpart in the reference: it serves callers that cannot call
 * cudaMalloc while pricing, such as a plugin hosted by a framework whose
 * caching allocator already holds the GPU's memory, a latency-critical loop
 * that cannot afford the device synchronisation cudaMalloc/cudaFree may
 * cause, or code that may allocate only at start-up. Same paths, same Philox
 * stream and same sums as pcf_mc_eur with use_cv = 1 (stream id 0).
 *   - The caller passes the inputs and a device buffer d_sums of 5 doubles,
 *     which receives {sum y, sum y^2, sum S_T, sum S_T^2, sum y S_T};
 *     price = exp(-rT) * d_sums[0] / N.
 *   - Work is queued on `stream` (a cudaStream_t, NULL for the legacy
 *     default stream); the call does not wait for it.
 *   - Scratch lives in one fixed device array inside the library (640 KiB per
 *     GPU that loads it, held until the process exits). N is limited to 2^30
 *     paths; larger N returns PCF_EINVAL.
 *   - The first call on each device looks up that array's device address
 *     (cudaGetSymbolAddress, with that device current) and keeps it for the
 *     life of the process; make that first call before any stream capture.
 *     After cudaDeviceReset the kept address is stale: restart the process.
 *   - All calls share the array, so calls whose kernels overlap on the GPU
 *     (concurrent streams, other host threads) race and must be serialised
 *     by the caller.
 *   - It calls no cudaMalloc, cudaFree or other allocating routine. */
PCF_API int pcf_mc_eur_noalloc(double S0, double E, double r, double sigma, double T,
                               long long N, int payoff_fun, unsigned long long seed,
                               double* d_sums, void* stream);

/* ---- Batched pricing -----------------------------------------------------
 * The reference prices one contract per process run (one main() per price).
 * A batch prices many contracts of mixed methods, uneven path and step
 * counts in one persistent launch per method, whose blocks pull work items
 * from a device queue. Each request draws from its own Philox stream
 * (seed, stream), so its result does not depend on what else is in the batch
 * beyond FP64 summation order. */
#define PCF_METHOD_EUR 0
#define PCF_METHOD_ASIA 1
#define PCF_METHOD_BASKET 2
#define PCF_METHOD_AMER 3

typedef struct pcf_mc_request {
  int method;             /* PCF_METHOD_* */
  int payoff_fun;         /* +1 call, -1 put */
  double S0, E, r, sigma, T;
  long long N;            /* paths */
  int M;                  /* Asian steps, American exercise dates */
  int mode;               /* Asian averaging mode; American: 1 = reference exercise rule */
  int use_cv;             /* report the control-variate estimate as `price` */
  int assets;             /* basket size d (1..64) */
  double rho;             /* basket equicorrelation, used when corr == NULL */
  const double* basket_S0;    /* [d] or NULL (all S0) */
  const double* basket_sigma; /* [d] or NULL (all sigma) */
  const double* corr;         /* [d*d] row-major or NULL (equicorrelation rho) */
  int scale_by_sqrt_T;    /* basket: 1 = GBM draws scaled by sqrt(T) */
  unsigned long long seed;
  unsigned int stream;    /* Philox stream id (e.g. the request id) */
} pcf_mc_request;

/* A plan holds a batch's contract tables and results on the device, so it
 * can be launched repeatedly (or captured in a CUDA graph) with no host
 * traffic. */
typedef struct pcf_plan pcf_plan;
PCF_API int pcf_plan_create(pcf_ctx* ctx, int n, const pcf_mc_request* reqs, pcf_plan** out);
/* Enqueue the plan's kernels on the context stream; returns without waiting.
 * From the second launch on, the launch sequence is captured once in a CUDA
 * graph and replayed (falling back to direct launches if capture fails). */
PCF_API int pcf_plan_launch(pcf_plan* plan);
/* mode 1 (default): replay through a CUDA graph from the second launch;
 * mode 0: always launch directly (drops a captured graph). */
PCF_API int pcf_plan_set_graph(pcf_plan* plan, int mode);
/* 1 if the plan's launches now replay a CUDA graph. */
PCF_API int pcf_plan_uses_graph(const pcf_plan* plan);
/* Wait for the plan's last launch and fill results[n]. */
PCF_API int pcf_plan_results(pcf_plan* plan, pcf_mc_result* results);
/* Kernels one pcf_plan_launch enqueues. */
PCF_API int pcf_plan_kernel_count(const pcf_plan* plan);
PCF_API int pcf_plan_destroy(pcf_plan* plan);

/* Price n requests in one call: create, launch, read back, destroy. */
PCF_API int pcf_price_batch(pcf_ctx* ctx, int n, const pcf_mc_request* reqs,
                            pcf_mc_result* results);

/* ---- Work shapes and the autotuner ---------------------------------------
 * Every launch takes its work shape from a per-device table: the block size
 * of the Monte Carlo launches (128, 256 or 512 threads), the paths each
 * thread prices in one work item (by class of N for European contracts, of
 * M for Asian ones, of d for baskets), the 128-path tiles per work item of
 * the tensor-core basket kernel, and the Longstaff-Schwartz cluster size and
 * slice (by class of N). The built-in table was measured by hand on GB300.
 * A work item's size depends only on its contract and the table, so results
 * are the same alone and in any batch while the table is unchanged; a new
 * table regroups the per-thread sums (differences of ~1e-8 relative).
 * The reference's only knob is a fixed OpenMP chunk of 1000 paths
 * (schedule(dynamic,1000), src/mc_eur_omp.cpp:24). */
#define PCF_TUNE_MC 1    /* European, Asian and basket shapes */
#define PCF_TUNE_LSM 2   /* Longstaff-Schwartz cluster shapes */
#define PCF_TUNE_SAVE 4  /* write the table to the file named by PCF_TUNE_CACHE */

/* Times candidate shapes per method and shape class on the context's device
 * (plans of synthetic contracts of each class, CUDA events, best of three)
 * and keeps a candidate where it beats the shape in force by more than 2 %.
 * flags = 0 tunes everything. Writes a JSON report (the table, the built-in
 * table and every trial) to report[report_len] if report is not NULL. Takes
 * seconds. A file named by the environment variable PCF_TUNE_CACHE is read
 * on a device's first use, if it was written for the same device model. */
PCF_API int pcf_autotune(pcf_ctx* ctx, int flags, char* report, int report_len);
/* pcf_autotune with every knob timed on the caller's own batch (a plan of
 * reqs[n], e.g. a representative slice of a served stream), so the table
 * fits that workload rather than each shape class alone. */
PCF_API int pcf_autotune_batch(pcf_ctx* ctx, int flags, int n, const pcf_mc_request* reqs,
                               char* report, int report_len);
/* The table in force on the context's device, as JSON
 * {"device": ..., "table": {...}}. */
PCF_API int pcf_tune_report(pcf_ctx* ctx, char* report, int report_len);
/* Restores the built-in table on the context's device. */
PCF_API int pcf_tune_reset(pcf_ctx* ctx);

/* ---- Serving ---------------------------------------------------------------
 * A continuous-batching loop. Requests arrive over time; every request whose
 * arrival time has passed is admitted into the next free batch slot. Slots
 * have device memory reserved up front, sized from the free HBM, so nothing is
 * allocated while serving. Several slots are in flight on their own streams,
 * so a batch admitted while others run overlaps with them on the device.
 * With target_rel_se > 0, each request is priced to that relative standard
 * error: a pilot run estimates the variance of its estimator (the
 * control-variate one when use_cv is set), and the main run uses the path
 * count that reaches the target, clamped to [pilot_paths, max_paths]
 * (American: [2^16, max_amer_paths], even). The reference has no serving
 * layer: its runscript_*.sh launch one process per price. */
typedef struct pcf_server_config {
  double target_rel_se;     /* <= 0: price each request at its own N, no pilot */
  long long pilot_paths;    /* 0: 2^14 */
  long long max_paths;      /* 0: 2^26 */
  long long max_amer_paths; /* 0: 2^21 */
  int max_batch;            /* requests per batch; 0: 2048 */
  int slots;                /* batches in flight; 0: 12 */
  double hbm_fraction;      /* share of free device memory reserved; 0: 0.5 */
} pcf_server_config;

typedef struct pcf_served_result {
  pcf_mc_result result;
  double arrival_s;   /* trace time the request arrived */
  double admit_s;     /* when it entered a batch */
  double done_s;      /* when its price was on the host */
  long long paths;    /* paths simulated for it (pilot + main) */
  int status;         /* PCF_OK or the error of its batch */
} pcf_served_result;

typedef struct pcf_server_stats {
  int completed;
  int batches;
  double wall_s;          /* first arrival to last completion */
  double p50_ms, p99_ms, mean_ms, max_ms;   /* arrival -> done */
  double contracts_per_s;
  double paths_per_s;
  long long paths;
  size_t reserved_bytes;  /* device memory the loop reserved */
} pcf_server_stats;

/* Replays a request trace (arrival_s non-decreasing, seconds from the start)
 * against the wall clock and serves it; fills out[n] and stats. */
PCF_API int pcf_serve_trace(pcf_ctx* ctx, const pcf_server_config* cfg, int n,
                            const pcf_mc_request* reqs, const double* arrival_s,
                            pcf_served_result* out, pcf_server_stats* stats);

/* The live server: the same continuous-batching loop on a worker thread of
 * its own, fed by callers while it runs (pcf_serve_trace replays a trace
 * known in advance). pcf_server_start reserves the context's serving slots
 * (kept in the context, as for pcf_serve_trace) and starts the worker; from
 * then until pcf_server_stop the context belongs to the server (no other call
 * may use it). Any thread may submit, poll and wait. A request's arrival time
 * is its submission, on the server's clock (seconds since start). Results
 * do not depend on what else is being served: the same request alone gives
 * the same result (the batching and the work shapes depend on the request
 * alone). No counterpart in the reference. */
typedef struct pcf_server pcf_server;
PCF_API int pcf_server_start(pcf_ctx* ctx, const pcf_server_config* cfg, pcf_server** out);
/* Queues one request; *ticket identifies it (0, 1, 2, ... in submission
 * order). The request is copied; arrays it points to (basket_S0,
 * basket_sigma, corr) must stay valid until its result is available. */
PCF_API int pcf_server_submit(pcf_server* srv, const pcf_mc_request* req, long long* ticket);
/* PCF_OK and *out filled if the request is finished (out->status holds its
 * own error, if any), PCF_PENDING if not yet. */
PCF_API int pcf_server_poll(pcf_server* srv, long long ticket, pcf_served_result* out);
/* As pcf_server_poll, waiting up to timeout_s seconds (< 0: no limit). */
PCF_API int pcf_server_wait(pcf_server* srv, long long ticket, double timeout_s,
                            pcf_served_result* out);
/* Finishes every submitted request, stops the worker, fills stats over all
 * requests served and frees the server (the slots stay with the context)
 * once every submit, poll or wait call already in progress on other threads
 * has returned (a submit that arrives meanwhile is refused). No call may
 * start on the handle after pcf_server_stop has returned. Returns the first
 * batch error, if any. */
PCF_API int pcf_server_stop(pcf_server* srv, pcf_server_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* PCF_H_ */
