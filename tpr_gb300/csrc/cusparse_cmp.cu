// cuSPARSE gtsv2_nopivot as a comparison solver (the reference's benchmark
// times it next to TPR / PTPR, src/reference_cusparse.cu:166-205 and
// src/pm.cpp:86).  libcusparse is opened at run time (dlopen), so the
// library has no link dependency on it; the call fails with
// TPRGB_EUNSUPPORTED where it is absent.  Not on the solver's own path.
#include <cusparse.h>  // types and prototypes only
#include <dlfcn.h>

#include <mutex>
#include <vector>

#include "common.cuh"

namespace tprgb {
namespace {

using CreateFn = cusparseStatus_t (*)(cusparseHandle_t *);
using SetStreamFn = cusparseStatus_t (*)(cusparseHandle_t, cudaStream_t);
template <typename T>
using BufFn = cusparseStatus_t (*)(cusparseHandle_t, int, int, const T *, const T *,
                                   const T *, const T *, int, size_t *);
template <typename T>
using SolveFn = cusparseStatus_t (*)(cusparseHandle_t, int, int, const T *, const T *,
                                     const T *, T *, int, void *);

struct Ctx {
    std::mutex mu;
    void *lib = nullptr;
    bool tried = false;
    CreateFn create = nullptr;
    SetStreamFn set_stream = nullptr;
    BufFn<float> sbuf = nullptr;
    SolveFn<float> ssolve = nullptr;
    BufFn<double> dbuf = nullptr;
    SolveFn<double> dsolve = nullptr;
    cusparseHandle_t h = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    void *dev = nullptr;  // dl, d, du, B of the largest system so far
    size_t dev_bytes = 0;
    void *work = nullptr;
    size_t work_bytes = 0;
};

Ctx g_ctx;

int open_lib(Ctx &c) {
    if (c.lib) return TPRGB_OK;
    if (c.tried) return fail(TPRGB_EUNSUPPORTED, "libcusparse could not be opened");
    c.tried = true;
    for (const char *name : {"libcusparse.so.12", "libcusparse.so"}) {
        c.lib = dlopen(name, RTLD_NOW | RTLD_LOCAL);
        if (c.lib) break;
    }
    if (!c.lib) return fail(TPRGB_EUNSUPPORTED, "libcusparse could not be opened");
    c.create = (CreateFn)dlsym(c.lib, "cusparseCreate");
    c.set_stream = (SetStreamFn)dlsym(c.lib, "cusparseSetStream");
    c.sbuf = (BufFn<float>)dlsym(c.lib, "cusparseSgtsv2_nopivot_bufferSizeExt");
    c.ssolve = (SolveFn<float>)dlsym(c.lib, "cusparseSgtsv2_nopivot");
    c.dbuf = (BufFn<double>)dlsym(c.lib, "cusparseDgtsv2_nopivot_bufferSizeExt");
    c.dsolve = (SolveFn<double>)dlsym(c.lib, "cusparseDgtsv2_nopivot");
    if (!c.create || !c.set_stream || !c.sbuf || !c.ssolve || !c.dbuf || !c.dsolve)
        return fail(TPRGB_EUNSUPPORTED, "libcusparse lacks gtsv2_nopivot");
    if (c.create(&c.h) != CUSPARSE_STATUS_SUCCESS)
        return fail(TPRGB_ECUDA, "cusparseCreate failed");
    TPRGB_CUDA(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking));
    TPRGB_CUDA(cudaEventCreate(&c.e0));
    TPRGB_CUDA(cudaEventCreate(&c.e1));
    if (c.set_stream(c.h, c.st) != CUSPARSE_STATUS_SUCCESS)
        return fail(TPRGB_ECUDA, "cusparseSetStream failed");
    return TPRGB_OK;
}

template <typename T>
int solve(Ctx &c, int n, const T *a, const T *diag, const T *cc, const T *rhs, T *x,
          float *ms) {
    const size_t bytes = sizeof(T) * (size_t)n;
    if (c.dev_bytes < 4 * bytes) {
        cudaFree(c.dev);
        c.dev = nullptr;
        c.dev_bytes = 0;
        TPRGB_CUDA(cudaMalloc(&c.dev, 4 * bytes));
        c.dev_bytes = 4 * bytes;
    }
    T *dl = (T *)c.dev, *d = dl + n, *du = d + n, *B = du + n;
    TPRGB_CUDA(cudaMemcpyAsync(dl, a, bytes, cudaMemcpyHostToDevice, c.st));
    if (diag) {
        TPRGB_CUDA(cudaMemcpyAsync(d, diag, bytes, cudaMemcpyHostToDevice, c.st));
    } else {
        // the reference's 3-argument form solves with a unit diagonal
        static thread_local std::vector<T> ones;
        ones.assign((size_t)n, T(1));
        TPRGB_CUDA(cudaMemcpyAsync(d, ones.data(), bytes, cudaMemcpyHostToDevice, c.st));
        TPRGB_CUDA(cudaStreamSynchronize(c.st));
    }
    TPRGB_CUDA(cudaMemcpyAsync(du, cc, bytes, cudaMemcpyHostToDevice, c.st));
    TPRGB_CUDA(cudaMemcpyAsync(B, rhs, bytes, cudaMemcpyHostToDevice, c.st));
    size_t need = 0;
    cusparseStatus_t s = sizeof(T) == 4
        ? c.sbuf(c.h, n, 1, (const float *)dl, (const float *)d, (const float *)du,
                 (const float *)B, n, &need)
        : c.dbuf(c.h, n, 1, (const double *)dl, (const double *)d, (const double *)du,
                 (const double *)B, n, &need);
    if (s != CUSPARSE_STATUS_SUCCESS) return fail(TPRGB_ECUDA, "gtsv2 buffer size failed");
    if (c.work_bytes < need) {
        TPRGB_CUDA(cudaStreamSynchronize(c.st));
        cudaFree(c.work);
        c.work = nullptr;
        c.work_bytes = 0;
        TPRGB_CUDA(cudaMalloc(&c.work, need));
        c.work_bytes = need;
    }
    TPRGB_CUDA(cudaEventRecord(c.e0, c.st));
    s = sizeof(T) == 4
        ? c.ssolve(c.h, n, 1, (const float *)dl, (const float *)d, (const float *)du,
                   (float *)B, n, c.work)
        : c.dsolve(c.h, n, 1, (const double *)dl, (const double *)d, (const double *)du,
                   (double *)B, n, c.work);
    TPRGB_CUDA(cudaEventRecord(c.e1, c.st));
    if (s != CUSPARSE_STATUS_SUCCESS) return fail(TPRGB_ECUDA, "gtsv2_nopivot failed");
    TPRGB_CUDA(cudaMemcpyAsync(x, B, bytes, cudaMemcpyDeviceToHost, c.st));
    TPRGB_CUDA(cudaStreamSynchronize(c.st));
    if (ms) TPRGB_CUDA(cudaEventElapsedTime(ms, c.e0, c.e1));
    return TPRGB_OK;
}

}  // namespace
}  // namespace tprgb

extern "C" TPRGB_API int tprgb_cusparse_gtsv(int prec, int n, const void *a,
                                             const void *diag, const void *c,
                                             const void *rhs, void *x,
                                             float *device_ms) {
    using namespace tprgb;
    if (n < 2 || !a || !c || !rhs || !x) return fail(TPRGB_EINVAL, "bad arguments");
    if (prec != TPRGB_F32 && prec != TPRGB_F64) return fail(TPRGB_EINVAL, "prec %d", prec);
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    int rc = open_lib(g_ctx);
    if (rc) return rc;
    if (prec == TPRGB_F32)
        return solve<float>(g_ctx, n, (const float *)a, (const float *)diag,
                            (const float *)c, (const float *)rhs, (float *)x, device_ms);
    return solve<double>(g_ctx, n, (const double *)a, (const double *)diag,
                         (const double *)c, (const double *)rhs, (double *)x, device_ms);
}
