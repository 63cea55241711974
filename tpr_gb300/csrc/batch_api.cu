// C ABI of the batched solver: options, tile selection, uniform batches.
#include <algorithm>
#include <mutex>
#include <vector>

#include "batch.cuh"

namespace tprgb {

// Default tile per system size (equations per thread, threads per CTA,
// variant): the tiles the autotuner measured fastest on GB300, so the
// staged and cluster kernels serve calls even without a loaded table;
// replaced at run time by the autotuner's table when one is loaded.
TileConfig default_tile(int n) {
    if (n < 32) return TileConfig{8, 128, 1};     // bulk-copy staged ring
    if (n <= 256) return TileConfig{8, 64, 2};    // swizzled, two stages
    if (n <= 1024) return TileConfig{16, 64, 3};  // swizzled, one stage
    if (n <= 2048) return TileConfig{16, 128, 3};
    if (n <= 4096) return TileConfig{16, 256, 3};
    if (n <= 16384) return TileConfig{16, n <= 8192 ? 256 : 128, 4};
    return TileConfig{16, 256, 4};  // one cluster of n / 4096 CTAs per system
}

// Tuned tiles per log2(n) (set by the autotuner through tprgb_tune_set).
// Read on every launch, possibly from the serving thread while another
// thread sets the table: a lock (uncontended in steady state) keeps each
// read whole.
static std::mutex g_tuned_mu;
static TileConfig g_tuned[32];
static bool g_has_tuned[32];

TileConfig tuned_tile(int n) {
    int k = ilog2(n);
    {
        std::lock_guard<std::mutex> lk(g_tuned_mu);
        if (k >= 0 && k < 32 && g_has_tuned[k]) return g_tuned[k];
    }
    return default_tile(n);
}

}  // namespace tprgb

using namespace tprgb;

extern "C" {

TPRGB_API int tprgb_batch_opts_default(tprgb_batch_opts *o) {
    if (!o) return fail(TPRGB_EINVAL, "opts is NULL");
    o->refine_steps = 1;
    o->residual = TPRGB_RESID_DF;
    o->x_f64 = 1;
    o->eq_per_thread = 0;
    o->threads_per_cta = 0;
    o->variant = 0;
    return TPRGB_OK;
}

TPRGB_API int tprgb_tune_set(int n, int eq_per_thread, int threads_per_cta,
                             int variant) {
    if (variant < 0 || variant > 5) return fail(TPRGB_EINVAL, "variant %d", variant);
    TileConfig c{eq_per_thread, threads_per_cta, variant >= 2 ? variant - 1 : 0};
    if (c.staged == 1 && c.nt != 128 && c.nt != 256 && c.nt != 512)
        return fail(TPRGB_EINVAL, "staged tiles use 128, 256 or 512 threads");
    if ((c.staged == 2 || c.staged == 3) &&
        ((c.nt != 64 && c.nt != 128 && c.nt != 256) || n < 32))
        return fail(TPRGB_EINVAL, "swizzled tiles use 64, 128 or 256 threads and n >= 32");
    int rc = batch_config_check(n, c);  // cluster tiles: cluster_parts' rules
    if (rc) return rc;
    int k = ilog2(n);
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    g_tuned[k] = c;
    g_has_tuned[k] = true;
    return TPRGB_OK;
}

TPRGB_API int tprgb_tune_get(int n, int *eq_per_thread, int *threads_per_cta,
                             int *variant) {
    if (!is_pow2(n)) return fail(TPRGB_EINVAL, "n=%d not a power of two", n);
    TileConfig c = tuned_tile(n);
    if (eq_per_thread) *eq_per_thread = c.L;
    if (threads_per_cta) *threads_per_cta = c.nt;
    if (variant) *variant = c.staged + 1;
    return TPRGB_OK;
}

TPRGB_API int tprgb_tune_clear(void) {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    for (int k = 0; k < 32; k++) g_has_tuned[k] = false;
    return TPRGB_OK;
}

TPRGB_API int tprgb_batch_solve(int nsys, int n, const float *d_a,
                                const float *d_b, const float *d_c,
                                const float *d_d, void *d_x,
                                const tprgb_batch_opts *opts, void *stream) {
    tprgb_batch_opts o;
    if (opts)
        o = *opts;
    else
        tprgb_batch_opts_default(&o);
    if (nsys < 0) return fail(TPRGB_EINVAL, "nsys=%d < 0", nsys);
    if (o.refine_steps < 0 || o.refine_steps > 8)
        return fail(TPRGB_EINVAL, "refine_steps=%d outside [0, 8]", o.refine_steps);
    if (o.residual != TPRGB_RESID_DF && o.residual != TPRGB_RESID_F64)
        return fail(TPRGB_EINVAL, "unknown residual mode %d", o.residual);
    if (nsys > 0 && (!d_a || !d_b || !d_c || !d_d || !d_x))
        return fail(TPRGB_EINVAL, "null device pointer");
    for (const void *p : {(const void *)d_a, (const void *)d_b,
                          (const void *)d_c, (const void *)d_d,
                          (const void *)d_x})
        if (((uintptr_t)p & 15) != 0)
            return fail(TPRGB_EINVAL, "device arrays must be 16-byte aligned");
    if (o.variant < 0 || o.variant > 5)
        return fail(TPRGB_EINVAL, "unknown kernel variant %d", o.variant);
    TileConfig cfg = tuned_tile(n);
    if (o.eq_per_thread) cfg.L = o.eq_per_thread;
    if (o.threads_per_cta) cfg.nt = o.threads_per_cta;
    if (o.variant) cfg.staged = o.variant - 1;
    BatchArgs A{d_a, d_b, d_c, d_d, d_x, nsys, n, o.refine_steps, o.residual,
                o.x_f64};
    const bool f64_resid = o.residual == TPRGB_RESID_F64 && o.refine_steps > 0;
    const bool staged_ok = (cfg.nt == 128 || cfg.nt == 256 || cfg.nt == 512) && !f64_resid;
    const bool sw_ok = (cfg.nt == 64 || cfg.nt == 128 || cfg.nt == 256) && n >= 32 &&
                       (cfg.L == 8 || cfg.L == 16) && !f64_resid;
    int P = 0;
    const bool cl_ok = cfg.staged == 4 && cfg.L == 16 &&
                       (cfg.nt == 64 || cfg.nt == 128 || cfg.nt == 256 || cfg.nt == 512) &&
                       n % (16 * cfg.nt) == 0 && (P = n / (16 * cfg.nt)) >= 2 && P <= 16;
    if (cl_ok) return launch_batch_cl(A, cfg, (cudaStream_t)stream);
    if (cfg.staged == 2 || cfg.staged == 3) {
        if (sw_ok) return launch_batch_sw(A, cfg, (cudaStream_t)stream);
    } else if (cfg.staged == 1 && staged_ok) {
        return launch_batch_tma(A, cfg, (cudaStream_t)stream);
    }
    if (o.variant >= 2)
        return fail(TPRGB_EUNSUPPORTED,
                    "variant %d does not serve this tile (L %d, threads %d, n %d) or residual",
                    o.variant, cfg.L, cfg.nt, n);
    // The table's kernel cannot serve this call (a caller-chosen shape, or
    // the FP64 residual, which the staged kernels lack; the cluster and
    // register kernels have it): the register kernel, with the caller's
    // shape where given, else one that covers n.
    if (!o.eq_per_thread) cfg.L = n >= 16 ? 8 : 4;
    if (!o.threads_per_cta) cfg.nt = std::min(1024, std::max(128, n / cfg.L));
    cfg.staged = 0;
    return launch_batch_uniform(A, cfg, (cudaStream_t)stream);
}

}  // extern "C"

// ---- host-buffer pipeline -------------------------------------------------
// Three streams by role: uploads, solves and downloads, with kHostBufs input
// and output buffers in a ring.  A chunk's upload waits only until the
// solve of the chunk kHostBufs earlier has read its input buffer, and its
// solve until that chunk's download has emptied the output buffer, so the
// link carries uploads back to back while downloads of earlier chunks run
// the other way.  (One stream per buffer, upload -> solve -> download in
// order, made each upload also wait for a download: 2 % slower end to end.)
constexpr int kHostBufs = 3;

struct tprgb_host_ctx {
    int64_t chunk_eq = 0;
    size_t max_pitch = 0;  // the device's largest pitch for 2D copies
    cudaStream_t up = nullptr, solve = nullptr, down = nullptr;
    cudaEvent_t uploaded[kHostBufs] = {}, solved[kHostBufs] = {}, downloaded[kHostBufs] = {};
    float *d_in[kHostBufs] = {};  // a, b, c, d of one chunk
    void *d_x[kHostBufs] = {};    // x of one chunk (8 B / eq)
    // chunks queued since creation: the ring position carries over from
    // call to call, so asynchronous calls pipeline into each other
    int64_t chunks = 0;
};

static void host_ctx_free(tprgb_host_ctx *h) {
    for (cudaStream_t s : {h->up, h->solve, h->down})
        if (s) cudaStreamDestroy(s);
    for (int i = 0; i < kHostBufs; i++) {
        for (cudaEvent_t e : {h->uploaded[i], h->solved[i], h->downloaded[i]})
            if (e) cudaEventDestroy(e);
        cudaFree(h->d_in[i]);
        cudaFree(h->d_x[i]);
    }
    delete h;
}

static void host_ctx_sync(tprgb_host_ctx *h) {
    for (cudaStream_t s : {h->up, h->solve, h->down}) cudaStreamSynchronize(s);
}

extern "C" {

TPRGB_API int tprgb_host_ctx_create(int64_t chunk_eq, tprgb_host_ctx **out) {
    if (!out) return fail(TPRGB_EINVAL, "out is NULL");
    *out = nullptr;
    if (chunk_eq <= 0 || (chunk_eq & 3))
        return fail(TPRGB_EINVAL, "chunk_eq=%lld must be a positive multiple of 4",
                    (long long)chunk_eq);
    tprgb_host_ctx *h = new tprgb_host_ctx();
    h->chunk_eq = chunk_eq;
    int dev = 0, pitch = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&pitch, cudaDevAttrMaxPitch, dev);
    h->max_pitch = pitch > 0 ? (size_t)pitch : 0;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->solve, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->down, cudaStreamNonBlocking);
    for (int i = 0; i < kHostBufs && e == cudaSuccess; i++) {
        e = cudaEventCreateWithFlags(&h->uploaded[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->solved[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->downloaded[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMalloc(&h->d_in[i], 4 * sizeof(float) * (size_t)chunk_eq);
        if (e == cudaSuccess) e = cudaMalloc(&h->d_x[i], sizeof(double) * (size_t)chunk_eq);
    }
    if (e != cudaSuccess) {
        host_ctx_free(h);
        return cuda_fail(e, "tprgb_host_ctx_create");
    }
    *out = h;
    return TPRGB_OK;
}

TPRGB_API int tprgb_host_ctx_destroy(tprgb_host_ctx *h) {
    if (!h) return fail(TPRGB_EINVAL, "ctx is NULL");
    host_ctx_sync(h);
    host_ctx_free(h);
    return TPRGB_OK;
}

// Queues one batch on the context's three streams (upload, solve,
// download) through its ring of device buffers, without waiting.
static int host_enqueue(tprgb_host_ctx *h, int nsys, int n, const float *a,
                        const float *b, const float *c, const float *d, void *x,
                        const tprgb_batch_opts *opts) {
    if (!h) return fail(TPRGB_EINVAL, "ctx is NULL");
    if (nsys < 0 || n <= 0) return fail(TPRGB_EINVAL, "bad nsys/n");
    if (nsys == 0) return TPRGB_OK;
    if (!a || !b || !c || !d || !x) return fail(TPRGB_EINVAL, "null host array");
    tprgb_batch_opts o;
    if (opts)
        o = *opts;
    else
        tprgb_batch_opts_default(&o);
    const int64_t per = h->chunk_eq / n;  // systems per chunk
    if (per < 1)
        return fail(TPRGB_EINVAL, "chunk of %lld equations < one system (n=%d)",
                    (long long)h->chunk_eq, n);
    const size_t xs = o.x_f64 ? sizeof(double) : sizeof(float);
    // Chunk sizes ramp up (1/8, 1/4, 1/2 of a full chunk) at the start and
    // down again at the end: the first solve and the first download start
    // sooner and the last chunk's solve and download are short, so less of
    // the link time is spent filling and draining the pipeline.
    std::vector<int64_t> sizes;
    {
        const int64_t ramp[3] = {std::max<int64_t>(1, per >> 3),
                                 std::max<int64_t>(1, per >> 2),
                                 std::max<int64_t>(1, per >> 1)};
        const int64_t edges = 2 * (ramp[0] + ramp[1] + ramp[2]);
        if (nsys > edges + per) {
            for (int64_t v : ramp) sizes.push_back(v);
            int64_t mid = nsys - edges;
            while (mid > 0) {
                sizes.push_back(std::min(per, mid));
                mid -= per;
            }
            for (int i = 2; i >= 0; i--) sizes.push_back(ramp[i]);
        } else {
            for (int64_t s0 = 0; s0 < nsys; s0 += per)
                sizes.push_back(std::min<int64_t>(per, nsys - s0));
        }
    }
    // on an error part-way, the work already queued is drained before
    // returning, so no copy still targets the caller's arrays
    auto drained = [&](int rc) {
        host_ctx_sync(h);
        return rc;
    };
    // a, b, c, d at one spacing (structure of arrays in one allocation):
    // each chunk's upload is one 2D copy of four rows instead of four
    // copies.  Every copy carries a fixed cost: on a 16384 x 1024 batch the
    // step went from 1.63 to 1.51 ms.  The spacing must be positive, hold
    // the largest chunk and fit the device's copy pitch.  The copy reads
    // exactly the four arrays' rows, so where the driver takes it the
    // result is right; it refuses a source range that spans separate pinned
    // allocations (arrays that merely sit at equal spacing), and then this
    // call falls back to four copies per chunk.
    const ptrdiff_t spacing = (const char *)b - (const char *)a;
    const int64_t max_chunk = sizes.empty() ? 0 : *std::max_element(sizes.begin(), sizes.end());
    bool one_copy = spacing > 0 && (const char *)c - (const char *)b == spacing &&
                          (const char *)d - (const char *)c == spacing &&
                          (size_t)spacing >= sizeof(float) * (size_t)(max_chunk * n) &&
                          (size_t)spacing <= h->max_pitch;
    int64_t s0 = 0;
    for (size_t ci = 0; ci < sizes.size(); ci++) {
        const int64_t g = h->chunks++;  // the chunk's place in the ring
        const int k = (int)(g % kHostBufs);
        const bool reuse = g >= kHostBufs;  // buffer k held chunk g - kHostBufs
        const int64_t ns = sizes[ci];
        const int64_t off = s0 * n, neq = ns * n;
        float *da = h->d_in[k], *db = da + h->chunk_eq, *dc = db + h->chunk_eq,
              *dd = dc + h->chunk_eq;
        const size_t bytes = sizeof(float) * (size_t)neq;
        cudaError_t e = cudaSuccess;
        if (reuse) e = cudaStreamWaitEvent(h->up, h->solved[k], 0);
        if (one_copy && e == cudaSuccess) {
            e = cudaMemcpy2DAsync(da, sizeof(float) * (size_t)h->chunk_eq, a + off,
                                  (size_t)spacing, bytes, 4, cudaMemcpyHostToDevice, h->up);
            if (e != cudaSuccess) {
                // refused before anything was queued (invalid value on this
                // driver): four copies from here on; an error that is not
                // the layout's fails those copies too and is reported
                cudaGetLastError();
                one_copy = false;
                e = cudaSuccess;
            }
        }
        if (!one_copy) {
            const float *src[4] = {a + off, b + off, c + off, d + off};
            float *dst[4] = {da, db, dc, dd};
            for (int i = 0; i < 4 && e == cudaSuccess; i++)
                e = cudaMemcpyAsync(dst[i], src[i], bytes, cudaMemcpyHostToDevice, h->up);
        }
        if (e == cudaSuccess) e = cudaEventRecord(h->uploaded[k], h->up);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h->solve, h->uploaded[k], 0);
        if (e == cudaSuccess && reuse) e = cudaStreamWaitEvent(h->solve, h->downloaded[k], 0);
        if (e != cudaSuccess) return drained(cuda_fail(e, "tprgb_batch_solve_host"));
        int rc = tprgb_batch_solve((int)ns, n, da, db, dc, dd, h->d_x[k], &o, h->solve);
        if (rc) return drained(rc);
        e = cudaEventRecord(h->solved[k], h->solve);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h->down, h->solved[k], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync((char *)x + off * xs, h->d_x[k], xs * (size_t)neq,
                                cudaMemcpyDeviceToHost, h->down);
        if (e == cudaSuccess) e = cudaEventRecord(h->downloaded[k], h->down);
        if (e != cudaSuccess) return drained(cuda_fail(e, "tprgb_batch_solve_host"));
        s0 += ns;
    }
    return TPRGB_OK;
}

static int host_wait(tprgb_host_ctx *h) {
    cudaError_t first = cudaSuccess;
    for (cudaStream_t s : {h->up, h->solve, h->down}) {
        const cudaError_t e = cudaStreamSynchronize(s);
        if (first == cudaSuccess) first = e;
    }
    if (first != cudaSuccess) return cuda_fail(first, "tprgb_host_ctx_wait");
    return TPRGB_OK;
}

TPRGB_API int tprgb_batch_solve_host(tprgb_host_ctx *h, int nsys, int n,
                                     const float *a, const float *b,
                                     const float *c, const float *d, void *x,
                                     const tprgb_batch_opts *opts) {
    int rc = host_enqueue(h, nsys, n, a, b, c, d, x, opts);
    if (rc) return rc;
    return host_wait(h);
}

TPRGB_API int tprgb_batch_solve_host_async(tprgb_host_ctx *h, int nsys, int n,
                                           const float *a, const float *b,
                                           const float *c, const float *d,
                                           void *x, const tprgb_batch_opts *opts) {
    return host_enqueue(h, nsys, n, a, b, c, d, x, opts);
}

TPRGB_API int tprgb_host_ctx_wait(tprgb_host_ctx *h) {
    if (!h) return fail(TPRGB_EINVAL, "ctx is NULL");
    return host_wait(h);
}

}  // extern "C"
