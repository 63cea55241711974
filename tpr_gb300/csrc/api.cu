// C ABI of libtprgb: status reporting, the reference-semantics path, the
// solver handle behind the TPR / PTPR / CR / PCR class surface, and the
// counterparts of the reference's *_cu free functions.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <chrono>
#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"

namespace tprgb {

static thread_local char g_err[512] = "";

int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    snprintf(g_err, sizeof(g_err), "%s: %s (%d)", what, cudaGetErrorString(e),
             (int)e);
    return e == cudaErrorMemoryAllocation ? TPRGB_ENOMEM : TPRGB_ECUDA;
}

// ref_kernels.cu
int ref_validate(int kind, int n, int s, int prec);
size_t ref_workspace_elems(int kind, int n, int s);
bool ref_needs_workspace(int kind, int n, int s, int prec);
int launch_ref(int kind, int nsys, int n, int s, int prec, const void *a,
               const void *c, const void *r, void *x, long long stride,
               void *work, cudaStream_t st);
int launch_normalize(int prec, long long neq, void *a, const void *diag,
                     void *c, void *r, cudaStream_t st);
bool ref_direct_ok(int kind, int n, int s, int prec);
int launch_ref_direct(int kind, int n, int s, int prec, const void *a, const void *diag,
                      const void *c, const void *r, void *x, unsigned *done,
                      cudaStream_t st);

static int flops_of(int kind, int n, int s) {
    int ln = ilog2(n);
    switch (kind) {
        case TPRGB_PTPR: {
            int m = n / s, ls = ilog2(s), lm = ilog2(m);
            return m * (14 * s * ls) + 14 * m + 9 * (m - 1) + 14 * m * lm +
                   m * 4 * (s - 1);
        }
        case TPRGB_TPR: {
            int m = n / s;
            return 28 * n - 14 * m + 9 * (m - 1) + 17 * m + m * 4 * (s - 1);
        }
        case TPRGB_CR:
            return n > 1 ? 17 * n : 0;
        default:
            return 14 * n * ln;
    }
}

}  // namespace tprgb

using namespace tprgb;

struct tprgb_solver {
    int kind, n, s, prec;
    size_t esz;
    void *d_a = nullptr, *d_c = nullptr, *d_r = nullptr, *d_diag = nullptr;
    // pinned, device-mapped staging (a, c, rhs, diag | x) so one solve costs
    // one host synchronisation (in get_ans)
    unsigned char *h_stage = nullptr, *h_x = nullptr;
    unsigned char *hd_stage = nullptr;  // the staging's device address
    cudaEvent_t staged = nullptr;  // the last solve has left h_stage
    void *d_x = nullptr, *d_work = nullptr;
    cudaStream_t stream = nullptr;
    bool has_system = false;
    // One-launch path (TPR / PTPR on a thread-block cluster, 2..16 slices
    // of the fused shape): the kernel reads the system, divides by the
    // diagonal and writes x in the pinned staging itself -- no copies, one
    // launch per solve (the GPU reaches host memory over the chip-to-chip
    // link; for one small system that beats two copies and a separate
    // normalising launch).  Other shapes upload, normalise and download.
    bool direct = false;
    bool use_diag = false;
    // One-launch path on a GPU with native atomics on host memory: the
    // kernel's CTAs count a mapped word up as their part of x lands, and the
    // handle waits for it by reading host memory (done / expect / seen:
    // counts enqueued and confirmed) instead of a driver synchronisation.
    unsigned *h_done = nullptr, *hd_done = nullptr;
    unsigned expect = 0, seen = 0;
    // The one-launch solve as a CUDA graph (its arguments never change: the
    // staging, the completion word; [1] with the diagonal), captured at the
    // second solve and replayed after; graph_failed: launch directly.
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    bool graph_failed = false;
};

// Waits until every enqueued one-launch solve has written x (and so has
// read the staging): polls the completion word for up to ~200 us, then
// falls back to a stream synchronisation, which also reports a failed
// launch.
static int wait_direct(tprgb_solver *h) {
    if (h->seen == h->expect) return TPRGB_OK;
    if (h->h_done) {
        const auto t0 = std::chrono::steady_clock::now();
        for (unsigned i = 1;; i++) {
            if (__atomic_load_n(h->h_done, __ATOMIC_ACQUIRE) == h->expect) {
                h->seen = h->expect;
                return TPRGB_OK;
            }
            if ((i & 255u) == 0 && std::chrono::steady_clock::now() - t0 >
                                       std::chrono::microseconds(200))
                break;
        }
    }
    TPRGB_CUDA(cudaStreamSynchronize(h->stream));
    if (h->h_done && __atomic_load_n(h->h_done, __ATOMIC_ACQUIRE) != h->expect)
        return fail(TPRGB_ECUDA, "one-launch solve ended without counting its parts");
    h->seen = h->expect;
    return TPRGB_OK;
}

extern "C" {

TPRGB_API const char *tprgb_last_error(void) { return g_err; }

TPRGB_API const char *tprgb_version(void) {
    return "tpr_gb300 1.0 (sm_103a)";
}

TPRGB_API int tprgb_flops(int kind, int n, int s, int *flops) {
    if (!flops) return fail(TPRGB_EINVAL, "flops is NULL");
    if (kind == TPRGB_CR || kind == TPRGB_PCR) s = n;
    if (!is_pow2(n) || !is_pow2(s) || s > n)
        return fail(TPRGB_EINVAL, "n=%d, s=%d must be powers of two, s<=n", n, s);
    *flops = flops_of(kind, n, s);
    return TPRGB_OK;
}

TPRGB_API int tprgb_ref_workspace_bytes(int kind, int nsys, int n, int s,
                                        int prec, size_t *bytes) {
    if (!bytes) return fail(TPRGB_EINVAL, "bytes is NULL");
    if (nsys < 0) return fail(TPRGB_EINVAL, "nsys=%d < 0", nsys);
    int rc = ref_validate(kind, n, s, prec);
    if (rc) return rc;
    size_t esz = prec == TPRGB_F32 ? 4 : 8;
    *bytes = ref_needs_workspace(kind, n, s, prec)
                 ? ref_workspace_elems(kind, n, s) * esz * (size_t)nsys
                 : 0;
    return TPRGB_OK;
}

TPRGB_API int tprgb_ref_solve_device(int kind, int nsys, int n, int s,
                                     int prec, const void *d_a,
                                     const void *d_c, const void *d_rhs,
                                     void *d_x, void *d_work,
                                     size_t work_bytes, void *stream) {
    int rc = ref_validate(kind, n, s, prec);
    if (rc) return rc;
    if (nsys < 0 || nsys > 65535)
        return fail(TPRGB_EINVAL, "nsys=%d outside [0, 65535]", nsys);
    if (nsys == 0) return TPRGB_OK;
    if (!d_a || !d_c || !d_rhs || !d_x)
        return fail(TPRGB_EINVAL, "null device pointer");
    size_t need = 0;
    tprgb_ref_workspace_bytes(kind, nsys, n, s, prec, &need);
    if (need > 0 && (d_work == nullptr || work_bytes < need))
        return fail(TPRGB_EINVAL,
                    "workspace of %zu bytes needed (got %zu at %p)", need,
                    work_bytes, d_work);
    return launch_ref(kind, nsys, n, s, prec, d_a, d_c, d_rhs, d_x,
                      (long long)n, d_work, (cudaStream_t)stream);
}

TPRGB_API int tprgb_normalize_device(int prec, int64_t neq, void *d_a,
                                     const void *d_diag, void *d_c,
                                     void *d_rhs, void *stream) {
    if (prec != TPRGB_F32 && prec != TPRGB_F64)
        return fail(TPRGB_EINVAL, "unknown precision %d", prec);
    if (neq < 0) return fail(TPRGB_EINVAL, "neq < 0");
    if (neq == 0) return TPRGB_OK;
    if (!d_a || !d_diag || !d_c || !d_rhs)
        return fail(TPRGB_EINVAL, "null device pointer");
    return launch_normalize(prec, neq, d_a, d_diag, d_c, d_rhs,
                            (cudaStream_t)stream);
}

static void free_handle(tprgb_solver *h) {
    if (!h) return;
    for (cudaGraphExec_t g : h->gexec)
        if (g) cudaGraphExecDestroy(g);
    if (h->staged) cudaEventDestroy(h->staged);
    cudaFreeHost(h->h_stage);
    if (h->h_done) cudaFreeHost(h->h_done);
    cudaFree(h->d_a);
    cudaFree(h->d_work);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

TPRGB_API int tprgb_create(int kind, int n, int s, int prec,
                           tprgb_solver **out) {
    if (!out) return fail(TPRGB_EINVAL, "out is NULL");
    *out = nullptr;
    if (kind == TPRGB_CR || kind == TPRGB_PCR) s = n;
    int rc = ref_validate(kind, n, s, prec);
    if (rc) return rc;
    tprgb_solver *h = new tprgb_solver();
    h->kind = kind;
    h->n = n;
    h->s = s;
    h->prec = prec;
    h->esz = prec == TPRGB_F32 ? 4 : 8;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free_handle(h);
        return cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    // one allocation: a, c, rhs, diag, x
    e = cudaMalloc(&h->d_a, 5 * (size_t)n * h->esz);
    if (e != cudaSuccess) {
        free_handle(h);
        return cuda_fail(e, "cudaMalloc(solver buffers)");
    }
    e = cudaHostAlloc((void **)&h->h_stage, 5 * (size_t)n * h->esz, cudaHostAllocMapped);
    if (e == cudaSuccess)
        e = cudaHostGetDevicePointer((void **)&h->hd_stage, h->h_stage, 0);
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&h->staged, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        free_handle(h);
        return cuda_fail(e, "pinned staging");
    }
    h->h_x = h->h_stage + 4 * (size_t)n * h->esz;
    h->direct = ref_direct_ok(kind, n, s, prec);
    if (h->direct) {
        int dev = 0, native = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess)
            e = cudaDeviceGetAttribute(&native, cudaDevAttrHostNativeAtomicSupported, dev);
        if (e == cudaSuccess && native) {
            e = cudaHostAlloc((void **)&h->h_done, 64, cudaHostAllocMapped);
            if (e == cudaSuccess) {
                *h->h_done = 0;
                e = cudaHostGetDevicePointer((void **)&h->hd_done, h->h_done, 0);
            }
        }
        if (e != cudaSuccess) {
            free_handle(h);
            return cuda_fail(e, "completion word");
        }
    }
    char *p = (char *)h->d_a;
    h->d_c = p + 1 * (size_t)n * h->esz;
    h->d_r = p + 2 * (size_t)n * h->esz;
    h->d_diag = p + 3 * (size_t)n * h->esz;
    h->d_x = p + 4 * (size_t)n * h->esz;
    if (ref_needs_workspace(kind, n, s, prec)) {
        e = cudaMalloc(&h->d_work, ref_workspace_elems(kind, n, s) * h->esz);
        if (e != cudaSuccess) {
            free_handle(h);
            return cuda_fail(e, "cudaMalloc(workspace)");
        }
    }
    *out = h;
    return TPRGB_OK;
}

TPRGB_API int tprgb_destroy(tprgb_solver *h) {
    if (!h) return fail(TPRGB_EINVAL, "handle is NULL");
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_handle(h);
    return TPRGB_OK;
}

TPRGB_API int tprgb_set_system(tprgb_solver *h, const void *a,
                               const void *diag, const void *c,
                               const void *rhs) {
    if (!h) return fail(TPRGB_EINVAL, "handle is NULL");
    if (!a || !c || !rhs) return fail(TPRGB_EINVAL, "null host array");
    const size_t bytes = (size_t)h->n * h->esz;
    // the previous upload (or one-launch solve) must have left the staging
    if (h->direct) {
        int rc = wait_direct(h);
        if (rc) return rc;
    } else {
        TPRGB_CUDA(cudaEventSynchronize(h->staged));
    }
    // CR ignores diag as the reference's setter does (src/cr.cpp:17-21)
    const bool use_diag = diag && h->kind != TPRGB_CR;
    memcpy(h->h_stage, a, bytes);
    memcpy(h->h_stage + bytes, c, bytes);
    memcpy(h->h_stage + 2 * bytes, rhs, bytes);
    if (use_diag) memcpy(h->h_stage + 3 * bytes, diag, bytes);
    h->use_diag = use_diag;
    if (h->direct) {  // the solve reads the staging itself
        h->has_system = true;
        return TPRGB_OK;
    }
    // device layout a, c, rhs, diag is contiguous: one copy
    TPRGB_CUDA(cudaMemcpyAsync(h->d_a, h->h_stage, (use_diag ? 4 : 3) * bytes,
                               cudaMemcpyHostToDevice, h->stream));
    TPRGB_CUDA(cudaEventRecord(h->staged, h->stream));
    if (use_diag) {
        int rc = launch_normalize(h->prec, h->n, h->d_a, h->d_diag, h->d_c,
                                  h->d_r, h->stream);
        if (rc) return rc;
    }
    h->has_system = true;
    return TPRGB_OK;
}

TPRGB_API int tprgb_solve(tprgb_solver *h, int *flops) {
    if (!h) return fail(TPRGB_EINVAL, "handle is NULL");
    if (!h->has_system)
        return fail(TPRGB_EINVAL, "set_tridiagonal_system was not called");
    // enqueued only: get_ans waits for it (and reports a failed launch)
    int rc;
    if (h->direct) {
        const size_t bytes = (size_t)h->n * h->esz;
        auto launch = [&]() {
            return launch_ref_direct(h->kind, h->n, h->s, h->prec, h->hd_stage,
                                     h->use_diag ? h->hd_stage + 3 * bytes : nullptr,
                                     h->hd_stage + bytes, h->hd_stage + 2 * bytes,
                                     h->hd_stage + 4 * bytes, h->hd_done, h->stream);
        };
        cudaGraphExec_t &gx = h->gexec[h->use_diag ? 1 : 0];
        // the first solve launches directly (and sets the kernel's
        // attributes); later ones capture it once and replay the graph
        if (!gx && !h->graph_failed && h->expect != 0) {
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                rc = launch();
                cudaError_t ee = cudaStreamEndCapture(h->stream, &g);
                if (rc == TPRGB_OK && ee == cudaSuccess)
                    e = cudaGraphInstantiate(&gx, g, 0);
                else
                    e = ee != cudaSuccess ? ee : cudaErrorUnknown;
                if (g) cudaGraphDestroy(g);
            }
            if (e != cudaSuccess) {
                cudaGetLastError();
                gx = nullptr;
                h->graph_failed = true;
            }
        }
        if (gx) {
            TPRGB_CUDA(cudaGraphLaunch(gx, h->stream));
        } else {
            rc = launch();
            if (rc) return rc;
        }
        // the next set_system / get_ans waits for this solve's parts
        h->expect += (unsigned)(h->n / h->s);
    } else {
        rc = launch_ref(h->kind, 1, h->n, h->s, h->prec, h->d_a, h->d_c,
                        h->d_r, h->d_x, h->n, h->d_work, h->stream);
        if (rc) return rc;
    }
    if (flops) *flops = flops_of(h->kind, h->n, h->s);
    return TPRGB_OK;
}

TPRGB_API int tprgb_get_ans(tprgb_solver *h, void *x) {
    if (!h) return fail(TPRGB_EINVAL, "handle is NULL");
    if (!x) return fail(TPRGB_EINVAL, "x is NULL");
    const size_t bytes = (size_t)h->n * h->esz;
    if (h->direct) {
        int rc = wait_direct(h);
        if (rc) return rc;
    } else {
        TPRGB_CUDA(cudaMemcpyAsync(h->h_x, h->d_x, bytes, cudaMemcpyDeviceToHost,
                                   h->stream));
        TPRGB_CUDA(cudaStreamSynchronize(h->stream));
    }
    memcpy(x, h->h_x, bytes);
    return TPRGB_OK;
}

TPRGB_API int tprgb_time_roundtrip(tprgb_solver *h, const void *a, const void *diag,
                                   const void *c, const void *rhs, void *x, int iters,
                                   double *us_per_solve) {
    if (!h) return fail(TPRGB_EINVAL, "handle is NULL");
    if (!us_per_solve || iters <= 0)
        return fail(TPRGB_EINVAL, "iters must be positive and us_per_solve set");
    auto once = [&]() {
        int rc = tprgb_set_system(h, a, diag, c, rhs);
        if (!rc) rc = tprgb_solve(h, nullptr);
        if (!rc) rc = tprgb_get_ans(h, x);
        return rc;
    };
    int rc = once();  // warm-up
    if (rc) return rc;
    const auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < iters && !rc; i++) rc = once();
    const auto t1 = std::chrono::steady_clock::now();
    if (rc) return rc;
    *us_per_solve = std::chrono::duration<double, std::micro>(t1 - t0).count() / iters;
    return TPRGB_OK;
}

// ---- *_cu counterparts ----------------------------------------------------
static std::mutex g_cache_mu;
static std::map<std::tuple<int, int, int, int>, tprgb_solver *> g_cache;

static int cu_solve(int kind, int prec, const void *a, const void *c,
                    const void *rhs, void *x, int n, int s) {
    if (!a || !c || !rhs || !x) return fail(TPRGB_EINVAL, "null host array");
    if (kind == TPRGB_CR || kind == TPRGB_PCR) s = n;
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto key = std::make_tuple(kind, prec, n, s);
    tprgb_solver *h;
    auto it = g_cache.find(key);
    if (it == g_cache.end()) {
        int rc = tprgb_create(kind, n, s, prec, &h);
        if (rc) return rc;
        g_cache[key] = h;
    } else {
        h = it->second;
    }
    int rc = tprgb_set_system(h, a, nullptr, c, rhs);
    if (!rc) rc = tprgb_solve(h, nullptr);
    if (!rc) rc = tprgb_get_ans(h, x);
    return rc;
}

TPRGB_API int tprgb_tpr_cu_f32(const float *a, const float *c,
                               const float *rhs, float *x, int n, int s) {
    return cu_solve(TPRGB_TPR, TPRGB_F32, a, c, rhs, x, n, s);
}
TPRGB_API int tprgb_ptpr_cu_f32(const float *a, const float *c,
                                const float *rhs, float *x, int n, int s) {
    return cu_solve(TPRGB_PTPR, TPRGB_F32, a, c, rhs, x, n, s);
}
TPRGB_API int tprgb_cr_cu_f32(const float *a, const float *c,
                              const float *rhs, float *x, int n) {
    return cu_solve(TPRGB_CR, TPRGB_F32, a, c, rhs, x, n, n);
}
TPRGB_API int tprgb_pcr_cu_f32(const float *a, const float *c,
                               const float *rhs, float *x, int n) {
    return cu_solve(TPRGB_PCR, TPRGB_F32, a, c, rhs, x, n, n);
}
TPRGB_API int tprgb_tpr_cu_f64(const double *a, const double *c,
                               const double *rhs, double *x, int n, int s) {
    return cu_solve(TPRGB_TPR, TPRGB_F64, a, c, rhs, x, n, s);
}
TPRGB_API int tprgb_ptpr_cu_f64(const double *a, const double *c,
                                const double *rhs, double *x, int n, int s) {
    return cu_solve(TPRGB_PTPR, TPRGB_F64, a, c, rhs, x, n, s);
}
TPRGB_API int tprgb_cr_cu_f64(const double *a, const double *c,
                              const double *rhs, double *x, int n) {
    return cu_solve(TPRGB_CR, TPRGB_F64, a, c, rhs, x, n, n);
}
TPRGB_API int tprgb_pcr_cu_f64(const double *a, const double *c,
                               const double *rhs, double *x, int n) {
    return cu_solve(TPRGB_PCR, TPRGB_F64, a, c, rhs, x, n, n);
}

TPRGB_API int tprgb_release_cached(void) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    for (auto &kv : g_cache) tprgb_destroy(kv.second);
    g_cache.clear();
    return TPRGB_OK;
}

}  // extern "C"
