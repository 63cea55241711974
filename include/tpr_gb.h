/*
 * tpr_gb.h -- C ABI of the GB300 tridiagonal solver library (libtprgb.so).
 *
 * Plain C: pointers, sizes and int status codes; no C++ or torch types.
 * Every function returns TPRGB_OK (0) or an error code and records a
 * message readable with tprgb_last_error() (per calling thread).  Nothing
 * here exits or aborts the process.
 *
 * Systems are  a[i] x[i-1] + b[i] x[i] + c[i] x[i+1] = d[i],  i = 0..n-1,
 * with a[0] and c[n-1] ignored (the reference requires them to be 0).
 * Entry points taking "d_" pointers expect device memory; "stream" is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   classes TPR / PTPR / CR / PCR    src/tpr.hpp:44-112, src/ptpr.hpp:44-110,
 *                                    src/cr.hpp:24-81, src/pcr.hpp:8-68
 *   free functions TPR_CU::tpr_cu, cr_cu, PTPR_CU::ptpr_cu, pcr_cu
 *                                    src/tpr.cuh:50-57, src/ptpr.cuh:50-57
 * The header-only C++ layer include/tpr_gb.hpp rebuilds the class and
 * namespace surface on top of these functions.
 */
#ifndef TPR_GB_H
#define TPR_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define TPRGB_API __attribute__((visibility("default")))
#else
#define TPRGB_API
#endif

/* ---- status codes (the reference asserts / aborts / exits instead:
 *      src/cr.hpp:72-75, src/tpr.cu:542-550, src/tpr.cu:575-579) -------- */
#define TPRGB_OK 0
#define TPRGB_EINVAL 1        /* bad argument (size, null pointer, kind)  */
#define TPRGB_ENOMEM 2        /* device or pinned allocation failed       */
#define TPRGB_EUNSUPPORTED 3  /* valid but outside this build's limits    */
#define TPRGB_ENONFINITE 4    /* a solution or residual is NaN / Inf      */
#define TPRGB_ETIMEOUT 5      /* a bounded device wait gave up            */
#define TPRGB_ECUDA 6         /* a CUDA runtime call failed               */
#define TPRGB_EBUSY 7         /* admission refused (budget or queue full) */
#define TPRGB_ENOTFOUND 8     /* unknown ticket / handle                  */

/* ---- solver families (src/lib.hpp:30-35 Solver concept) ---------------- */
#define TPRGB_PTPR 0 /* PCR-like TPR, PCR on the reduced system */
#define TPRGB_TPR 1  /* tree TPR, CR on the reduced system      */
#define TPRGB_CR 2   /* cyclic reduction (unit diagonal)        */
#define TPRGB_PCR 3  /* parallel cyclic reduction               */

/* ---- element types (src/lib.hpp:8-16 `real`) --------------------------- */
#define TPRGB_F32 0
#define TPRGB_F64 1

TPRGB_API const char *tprgb_last_error(void);
TPRGB_API const char *tprgb_version(void);

/* Reference flop count returned by solve() (src/ptpr.cpp:104-106,
 * src/tpr.cpp:96-98, src/cr.cpp:27, src/pcr.cpp:88). */
TPRGB_API int tprgb_flops(int kind, int n, int s, int *flops);

/* =========================================================================
 * Reference-semantics path: the reference's own algorithm (same
 * eliminations and operand order) on the GPU, bit-identical to its CPU
 * solvers on the same inputs.  Inputs are diag-normalised (unit diagonal).
 * ====================================================================== */

/* Scratch bytes tprgb_ref_solve_device needs for `nsys` systems (0 when the
 * system fits one CTA's shared memory: CR / PCR up to n = 8192 in FP32 and
 * 4096 in FP64; above, CR needs 3n and PCR 6n elements per system). */
TPRGB_API int tprgb_ref_workspace_bytes(int kind, int nsys, int n, int s,
                                        int prec, size_t *bytes);

/* Solve `nsys` systems of size n (system k at element offset k*n) with the
 * reference algorithm `kind` and slice size s (ignored for CR / PCR).
 * d_a, d_c, d_rhs: diag-normalised inputs, left untouched; d_x: output.
 * d_work: device scratch of tprgb_ref_workspace_bytes, or NULL if 0.
 * Asynchronous on `stream`.  Replaces the device part of
 * TPR_CU::tpr_cu / PTPR_CU::ptpr_cu / cr_cu / pcr_cu
 * (src/tpr.cu:574-723, src/ptpr.cu:542-707). */
TPRGB_API int tprgb_ref_solve_device(int kind, int nsys, int n, int s,
                                     int prec, const void *d_a,
                                     const void *d_c, const void *d_rhs,
                                     void *d_x, void *d_work,
                                     size_t work_bytes, void *stream);

/* Same as tprgb_ref_solve_device, but allocation-free, for callers that
 * cannot call cudaMalloc: plugins whose device memory belongs to a host
 * framework's allocator, and latency-critical loops where an allocation
 * would synchronise the device.  No counterpart in the reference.  The
 * workspace is the library's own 16 MiB device array (held by every GPU
 * that loads the library until exit).  The first call on a device (and
 * after a cudaDeviceReset) looks up the array's address, so make it before
 * any stream capture; workspace needs above 16 MiB (nsys * (3n + 3n/s)
 * elements for TPR / PTPR, nsys * 3n for CR and 6n for PCR above one CTA)
 * return TPRGB_EUNSUPPORTED; all calls share the array, so calls
 * that overlap on the GPU race. */
TPRGB_API int tprgb_ref_solve_device_static(int kind, int nsys, int n, int s,
                                            int prec, const void *d_a,
                                            const void *d_c, const void *d_rhs,
                                            void *d_x, void *stream);

/* a /= diag, c /= diag, rhs /= diag elementwise on the device: the 4-arg
 * set_tridiagonal_system (src/ptpr.hpp:80-90, src/tpr.hpp:80-89). */
TPRGB_API int tprgb_normalize_device(int prec, int64_t neq, void *d_a,
                                     const void *d_diag, void *d_c,
                                     void *d_rhs, void *stream);

/* ---- solver handle: the state of one TPR / PTPR / CR / PCR object ------ */
typedef struct tprgb_solver tprgb_solver;

/* Constructor (n, s) of the reference classes; s ignored for CR / PCR.
 * Allocates the device buffers once (src/ptpr.cpp:54-96). */
TPRGB_API int tprgb_create(int kind, int n, int s, int prec,
                           tprgb_solver **out);
TPRGB_API int tprgb_destroy(tprgb_solver *h);

/* set_tridiagonal_system: host arrays of n elements of the handle's type,
 * copied (through the handle's pinned staging) to the device; the caller
 * may reuse its arrays as soon as this returns.  diag == NULL is the 3-argument form (unit
 * diagonal assumed); otherwise the system is normalised by diag on the
 * device, as the 4-argument form does.  The caller's arrays are not
 * modified (the reference divides them in place). */
TPRGB_API int tprgb_set_system(tprgb_solver *h, const void *a,
                               const void *diag, const void *c,
                               const void *rhs);

/* solve(): enqueues the solve on the handle's stream; *flops (may be NULL)
 * receives the reference flop count.  get_ans waits for it. */
TPRGB_API int tprgb_solve(tprgb_solver *h, int *flops);

/* get_ans(x): copies the n-element solution to host memory. */
TPRGB_API int tprgb_get_ans(tprgb_solver *h, void *x);

/* Counterparts of the reference free functions (host arrays, unit
 * diagonal, synchronous; src/tpr.cuh:50-57, src/ptpr.cuh:50-57).  Unlike
 * the reference they keep a per-(kind, n, s) device context between calls
 * instead of cudaMalloc/cudaFree on every call, and the double versions are
 * implemented (the reference's are empty stubs, src/tpr.cu:726-734). */
TPRGB_API int tprgb_tpr_cu_f32(const float *a, const float *c,
                               const float *rhs, float *x, int n, int s);
TPRGB_API int tprgb_ptpr_cu_f32(const float *a, const float *c,
                                const float *rhs, float *x, int n, int s);
TPRGB_API int tprgb_cr_cu_f32(const float *a, const float *c,
                              const float *rhs, float *x, int n);
TPRGB_API int tprgb_pcr_cu_f32(const float *a, const float *c,
                               const float *rhs, float *x, int n);
TPRGB_API int tprgb_tpr_cu_f64(const double *a, const double *c,
                               const double *rhs, double *x, int n, int s);
TPRGB_API int tprgb_ptpr_cu_f64(const double *a, const double *c,
                                const double *rhs, double *x, int n, int s);
TPRGB_API int tprgb_cr_cu_f64(const double *a, const double *c,
                              const double *rhs, double *x, int n);
TPRGB_API int tprgb_pcr_cu_f64(const double *a, const double *c,
                               const double *rhs, double *x, int n);

/* Releases the device contexts kept by the *_cu functions. */
TPRGB_API int tprgb_release_cached(void);


/* =========================================================================
 * Batched path: many independent systems per launch, hierarchical TPR
 * (per-thread partition sweeps, warp-shuffle PCR inside a slice, PCR of the
 * reduced inter-slice system inside the CTA), FP32 arithmetic with optional
 * iterative refinement.  Raw (not diag-normalised) FP32 inputs a, b, c, d.
 * No reference counterpart for a single call: it replaces the reference's
 * pattern of one solver object per thread looping over systems
 * (test/examples.cpp:104-154) and one cooperative launch per system
 * (src/ptpr.cu:542-600).
 * ====================================================================== */
#define TPRGB_RESID_DF 0  /* residual in compensated FP32 (~2^-48)  */
#define TPRGB_RESID_F64 1 /* residual in native FP64, x kept in FP64:
                             cluster (variant 5), register (1) and queue
                             kernels; the staged variants refuse it */

typedef struct tprgb_batch_opts {
    int refine_steps;    /* 0: plain FP32 solve; k: k refinement steps      */
    int residual;        /* TPRGB_RESID_DF or TPRGB_RESID_F64               */
    int x_f64;           /* 1: x is double[neq]; 0: x is float[neq]         */
    int eq_per_thread;   /* 0: tuned table; otherwise 4, 8 (16: variants 3,4) */
    int threads_per_cta; /* 0: tuned table; otherwise 64 .. 1024 (below)    */
    int variant;         /* 0: tuned table; 1: inputs loaded to registers;
                            2: inputs staged in shared memory by TMA bulk
                               copies (persistent CTAs, 128/256/512
                               threads); 3: staged by swizzled 2D tensor-map
                               copies, two stages (8 or 16 equations per
                               thread, 64/128/256 threads, n >= 32);
                            4: as 3 with one stage;
                            5: one system per thread-block cluster of
                               P = n / (16 * threads) CTAs, P in {2, 4, 8,
                               16}, rows exchanged in distributed shared
                               memory (16 equations per thread,
                               64/128/256/512 threads)                     */
} tprgb_batch_opts;

/* Defaults: 1 refinement step, compensated residual, FP64 x, tuned tile. */
TPRGB_API int tprgb_batch_opts_default(tprgb_batch_opts *opts);

/* Solve nsys systems of size n laid out back to back (system k at element
 * k*n of every array).  n a power of two with 2*L <= n <= L * threads per
 * CTA (8192 with the default tiles), or up to 16 * 16 * threads (65536)
 * with the cluster variant, the default above 8192.
 * Asynchronous on `stream`; allocates nothing; can be captured in a CUDA
 * graph. */
TPRGB_API int tprgb_batch_solve(int nsys, int n, const float *d_a,
                                const float *d_b, const float *d_c,
                                const float *d_d, void *d_x,
                                const tprgb_batch_opts *opts, void *stream);

/* ---- host-buffer batched solve (pinned host arrays, e.g. for callers that
 * keep systems on the host; the counterpart of the reference wrappers'
 * H2D -> launch -> D2H sequence, src/ptpr.cu:542-600, without per-call
 * allocation).  The batch is cut into chunks, uploaded, solved and
 * downloaded on three streams (one per role) through a ring of three
 * device buffers: chunk k+1's upload overlaps chunk k's solve and the
 * downloads of earlier chunks.  Bound by the host link (GB300 machine
 * measured: 209 GB/s up, 193 GB/s down, 278 GB/s both ways at once). -- */
typedef struct tprgb_host_ctx tprgb_host_ctx;

/* Device buffers for chunks of up to chunk_eq equations (three in flight:
 * 24 B per equation each, 4 * chunk_eq floats in and chunk_eq doubles out). */
TPRGB_API int tprgb_host_ctx_create(int64_t chunk_eq, tprgb_host_ctx **out);
TPRGB_API int tprgb_host_ctx_destroy(tprgb_host_ctx *ctx);

/* Uniform batch from host arrays (system k at element k*n) into host x
 * (double or float per opts->x_f64).  Synchronous.  Host arrays should be
 * pinned (cudaHostAlloc / cudaHostRegister) for full copy bandwidth; with
 * a, b, c, d at one spacing in one allocation each chunk is uploaded by
 * one 2D copy (fewer copies, faster), otherwise by four. */
TPRGB_API int tprgb_batch_solve_host(tprgb_host_ctx *ctx, int nsys, int n,
                                     const float *a, const float *b,
                                     const float *c, const float *d, void *x,
                                     const tprgb_batch_opts *opts);

/* The same without waiting: the batch is queued behind the context's
 * earlier work, so a stream of batches overlaps one batch's downloads with
 * the next one's uploads instead of filling and draining the pipeline per
 * call.  The host arrays must stay untouched, and x unread, until
 * tprgb_host_ctx_wait returns.  No reference counterpart. */
TPRGB_API int tprgb_batch_solve_host_async(tprgb_host_ctx *ctx, int nsys, int n,
                                           const float *a, const float *b,
                                           const float *c, const float *d,
                                           void *x, const tprgb_batch_opts *opts);

/* Waits until every batch queued on the context is solved and in its x. */
TPRGB_API int tprgb_host_ctx_wait(tprgb_host_ctx *ctx);

/* ---- tile table (filled by the autotuner, tpr_gb300/autotune.py) ------
 * Tile of the uniform kernel for systems of size n: equations per thread,
 * threads per CTA and variant (as in tprgb_batch_opts).  Also gives the equations per thread the
 * uneven-batch plans use for that size. */
TPRGB_API int tprgb_tune_set(int n, int eq_per_thread, int threads_per_cta,
                             int variant);
TPRGB_API int tprgb_tune_get(int n, int *eq_per_thread, int *threads_per_cta,
                             int *variant);
TPRGB_API int tprgb_tune_clear(void);

/* ---- uneven batches: plan + persistent queue kernel ---------------------
 * A plan fixes the sizes and offsets of a batch of systems (any mix of
 * power-of-two n, 16 <= n <= 32 * CTA tile) and routes them by size:
 * systems of 256..4096 equations whose offsets are multiples of 32 go to
 * the swizzled staged kernel (one launch per size, per-system offsets),
 * 8192..65536 to the thread-block cluster kernel; the rest to one
 * cooperative launch of a persistent kernel whose CTAs pull work items
 * (largest systems first) from a device queue, systems larger than one
 * CTA's tile split over CTAs that exchange their reduced rows through the
 * plan's scratch with bounded waits.  opts->variant = 1 or the FP64
 * residual keeps every system on the queue kernel.  Replaces the
 * reference's one-launch-per-system loop (src/pm.cpp:224-238). */
typedef struct tprgb_plan tprgb_plan;

/* offsets[k]: first element of system k in every array (multiple of 4);
 * ns[k]: its size.  opts->threads_per_cta selects 256 or 512 (0 = 256). */
TPRGB_API int tprgb_plan_create(int nsys, const int64_t *offsets,
                                const int *ns, const tprgb_batch_opts *opts,
                                tprgb_plan **out);
TPRGB_API int tprgb_plan_destroy(tprgb_plan *plan);

/* enable != 0: the first execute with a given set of pointers captures the
 * reset + launch into a CUDA graph; later executes with the same pointers
 * replay it. */
TPRGB_API int tprgb_plan_use_graph(tprgb_plan *plan, int enable);

/* Asynchronous on `stream`; allocates nothing. */
TPRGB_API int tprgb_plan_execute(tprgb_plan *plan, const float *d_a,
                                 const float *d_b, const float *d_c,
                                 const float *d_d, void *d_x, void *stream);

TPRGB_API int tprgb_plan_info(const tprgb_plan *plan, int *nitems, int *grid,
                              int *nlarge, int *graph_active);

/* Systems on each route and the launches one execute makes. */
TPRGB_API int tprgb_plan_routes(const tprgb_plan *plan, int *staged_systems,
                                int *cluster_systems, int *queue_systems,
                                int *launches);

/* After an execute on `stream` (waits for it): sys_status[k] (may be NULL)
 * is 0 or 1 (non-finite solution) per system in the caller's order;
 * *device_code the kernel's own status.  Returns TPRGB_ETIMEOUT if a
 * multi-CTA wait gave up, TPRGB_ENONFINITE if any system is non-finite. */
TPRGB_API int tprgb_plan_status(tprgb_plan *plan, unsigned *sys_status,
                                unsigned *device_code, void *stream);

/* ---- seeded synthetic systems generated in device memory ---------------
 * System k (size d_ns[k], at d_offsets[k], seed d_seeds[k]) is written
 * into d_a..d_d.  kind: 0 dominant (b = |a|+|c|+U(1,2)), 1 uneven
 * (+U(0.1,1)), 2 weak (+10^U(-4,-1)).  Counter-based hashing, so the same
 * (n, seed, kind) always gives the same bits.  No reference counterpart
 * (the reference generates on the host, src/system.cpp:132-158). */
TPRGB_API int tprgb_generate_device(int nsys, const int64_t *d_offsets,
                                    const int *d_ns, const uint64_t *d_seeds,
                                    int kind, float *d_a, float *d_b,
                                    float *d_c, float *d_d, void *stream);

/* =========================================================================
 * Serving loop: continuous batching of solve requests (no reference
 * counterpart; the reference solves one system per call).  A request is a
 * set of systems, given either as host arrays or as seeds of the device
 * generator (state produced and kept on the device).  Requests are
 * admitted in FIFO order against a device-memory budget, their systems stay
 * resident until released, and every admitted request is merged into the
 * next step of the persistent queue kernel; the next step is queued behind
 * the running one.  Submission is thread-safe.
 * ====================================================================== */
typedef struct tprgb_server tprgb_server;

typedef struct tprgb_server_opts {
    size_t budget_bytes; /* device arena: 24 B per equation (default 8 GiB) */
    int max_pending;     /* queued, not yet admitted requests (default 2^20) */
    int refine_steps;    /* default 1                                      */
    int residual;        /* TPRGB_RESID_DF (default) or TPRGB_RESID_F64     */
    int threads_per_cta; /* 256 (default) or 512                           */
    long long max_step_eq; /* equations per step (0 = no cap); a larger
                              request is solved over several steps, so an
                              arrival never waits behind an unbounded step */
    int max_inflight;    /* steps queued on the device at once: 2 (default)
                            overlaps building the next step with the running
                            one; 1 makes an arrival wait for at most the
                            running step                                    */
    int kernel_routes;   /* 1 (default): a step's size groups of 256..4096
                            equations go to the staged kernel and of
                            8192..65536 to the cluster kernel, one launch
                            per size, the rest to the queue kernel; 0: the
                            whole step on the queue kernel                 */
} tprgb_server_opts;

typedef struct tprgb_request_info {
    int status;            /* TPRGB_OK, TPRGB_ENONFINITE, TPRGB_ETIMEOUT... */
    int nonfinite_systems; /* systems whose solution is not finite          */
    long long step;        /* the step that solved the request              */
    double latency_us;     /* submission -> solution resident on the device */
    long long x_offset;    /* first equation of the request in the arena    */
    long long neq;         /* equations in the request                      */
    double queue_us;       /* submission -> the step that finished it was
                              enqueued (admission, waiting for a step slot) */
    double step_us;        /* device time of that step                      */
} tprgb_request_info;

typedef struct tprgb_server_stats {
    long long steps, requests_done, systems_done, equations_done;
    long long pending, inflight_steps, arena_used_eq, arena_cap_eq;
} tprgb_server_stats;

TPRGB_API int tprgb_server_opts_default(tprgb_server_opts *opts);
TPRGB_API int tprgb_server_create(const tprgb_server_opts *opts,
                                  tprgb_server **out);
TPRGB_API int tprgb_server_destroy(tprgb_server *srv);

/* Seeded request: system k has size ns[k] (power of two >= 16) and is
 * generated on the device from seeds[k] (tprgb_generate_device kinds). */
TPRGB_API int tprgb_server_submit_seeded(tprgb_server *srv, int nsys,
                                         const int *ns, const uint64_t *seeds,
                                         int kind, uint64_t *ticket);

/* Host request: systems back to back in a..d (kept valid by the caller
 * until the request is done); x (may be NULL) receives the FP64 solution. */
TPRGB_API int tprgb_server_submit_host(tprgb_server *srv, int nsys,
                                       const int *ns, const float *a,
                                       const float *b, const float *c,
                                       const float *d, double *x,
                                       uint64_t *ticket);

/* Wait (timeout_ms < 0: forever) for a request; returns its status. */
TPRGB_API int tprgb_server_wait(tprgb_server *srv, uint64_t ticket,
                                int timeout_ms, tprgb_request_info *info);

/* Copy a finished request's solution (FP64) or its resident system out. */
TPRGB_API int tprgb_server_fetch(tprgb_server *srv, uint64_t ticket,
                                 double *x_host);
TPRGB_API int tprgb_server_fetch_system(tprgb_server *srv, uint64_t ticket,
                                        float *a, float *b, float *c,
                                        float *d);

/* Free a finished request's device memory. */
TPRGB_API int tprgb_server_release(tprgb_server *srv, uint64_t ticket);
TPRGB_API int tprgb_server_get_stats(tprgb_server *srv,
                                     tprgb_server_stats *st);

/* Load driver: submits nreq seeded requests with Poisson arrivals at
 * rate_per_s (<= 0: all at once), each with U{min_sys..max_sys} systems of
 * size 2^k, k ~ U{kmin..kmax}; waits for and releases them in order.
 * latencies_us[i] (may be NULL) receives each request's latency,
 * detail_us[3i..3i+2] (may be NULL) its queue_us, step_us and equations,
 * *elapsed_s first submission -> last completion, *systems_out the systems
 * solved. */
TPRGB_API int tprgb_server_run_load(tprgb_server *srv, int nreq,
                                    double rate_per_s, uint64_t seed,
                                    int min_sys, int max_sys, int kmin,
                                    int kmax, int kind, double *latencies_us,
                                    double *detail_us, double *elapsed_s,
                                    long long *systems_out);

/* ---- comparison solver -------------------------------------------------
 * cuSPARSE gtsv2_nopivot on one system from host arrays, as the reference's
 * benchmark runs it next to its own solvers (src/reference_cusparse.cu:
 * 166-205, selected by "cusparse" in src/pm.cpp:86): copies in, the solve,
 * copy out.  prec TPRGB_F32 / TPRGB_F64 (arrays of that type); diag NULL
 * means a unit diagonal (the 3-argument form).  *device_ms (may be NULL):
 * the solve alone, timed with CUDA events (the reference's device timer).
 * libcusparse is opened at run time; TPRGB_EUNSUPPORTED where it is absent. */
TPRGB_API int tprgb_cusparse_gtsv(int prec, int n, const void *a,
                                  const void *diag, const void *c,
                                  const void *rhs, void *x, float *device_ms);

/* Times `iters` host round trips of one system through a solver handle --
 * set_tridiagonal_system (3-argument with diag NULL, else 4-argument),
 * solve, get_ans -- in C++, after one untimed warm-up; *us_per_solve = the
 * mean microseconds per round trip.  The reference's timed loop
 * (src/pm.cpp:160-194) times its CPU solvers the same way (solve +
 * get_ans per iteration); this includes the setter's copy as well.  No
 * reference counterpart (a measurement helper). */
TPRGB_API int tprgb_time_roundtrip(tprgb_solver *h, const void *a, const void *diag,
                                   const void *c, const void *rhs, void *x, int iters,
                                   double *us_per_solve);

/* ---- diagnostics ------------------------------------------------------- */
/* Status word of the TMA-staged batched kernel: *code = TPRGB_ETIMEOUT if a
 * bounded wait gave up since the last reset (reset != 0 clears it). */
TPRGB_API int tprgb_batch_status(unsigned *code, int reset);

/* Runs one kind of the solver kernels' bounded device waits on a condition
 * that never comes true and reports what it recorded: status[0] = code
 * (TPRGB_ETIMEOUT when the wait gave up), status[1] = site, status[2] =
 * detail.  which: 0 the wait for a TMA load (polls: 1 .. 2^22; the
 * kernels use 2^18, 1.0 s on GB300), 1 the cluster row-exchange wait
 * (polls as for 0), 2 the global-memory barrier between the CTAs of one
 * system (its fixed limit, about 1.1 s; polls is ignored).  Nothing
 * faults; the context stays usable.  Synchronous. */
TPRGB_API int tprgb_selftest_wait_timeout(int which, unsigned polls,
                                          unsigned *status);

/* out[i] = hi[i] + lo[i] as the nearest double, computed on the device by
 * the same integer bit assembly the batched solver uses for its FP64
 * output (no reference counterpart; exposed for testing). */
TPRGB_API int tprgb_diag_pair_to_double(int64_t n, const float *d_hi,
                                        const float *d_lo, double *d_out,
                                        void *stream);

#ifdef __cplusplus
}
#endif

#endif /* TPR_GB_H */
