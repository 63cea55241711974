// Batched hierarchical TPR solver for many independent systems of one size
// n per launch, with optional iterative refinement (FP32 solve, residual in
// compensated FP32 or native FP64, solution accumulated as FP32 hi + lo).
//
// Geometry (per launch): L equations per thread, T = n / L threads per
// system (T <= NT), G = NT / T systems per CTA.  A system's threads are
// consecutive; lanes of a warp form segments of K = min(T, 32) lanes; a
// system spans W = T / K warp segments.  Grid = ceil(nsys / G) CTAs.
//
// HBM traffic per equation: a, b, c, d read once (16 B), x written once
// (4 B FP32 or 8 B FP64).  Refinement re-reads nothing: the raw system
// stays in registers.  The per-tile code is shared with the persistent
// queue kernel (tile.cuh).
#include <algorithm>

#include "batch.cuh"
#include "common.cuh"
#include "hier.cuh"
#include "tile.cuh"

namespace tprgb {
namespace bk {

// MODE: 0 = plain FP32 solve; 1 = refinement with compensated-FP32
// residual; 2 = refinement with native FP64 residual.  T = n / L threads
// per system (compile time), G = NT / T systems per CTA.
template <int L, int NT, int T, int MODE>
__global__ void __launch_bounds__(NT, (NT <= 256 ? 3 : (NT <= 512 ? 2 : 1)))
batch_uniform(const float *__restrict__ ga, const float *__restrict__ gb,
              const float *__restrict__ gc, const float *__restrict__ gd,
              void *__restrict__ gx, int nsys, int refine_steps, int x_f64) {
    __shared__ tile::Smem<NT> sm;
    constexpr int G = NT / T;
    constexpr int n = T * L;
    const int tid = threadIdx.x;
    const int g = tid / T, t = tid & (T - 1);
    const long long sys = (long long)blockIdx.x * G + g;
    const bool active = sys < nsys;
    const long long base = active ? sys * (long long)n + (long long)t * L : 0;
    tile::Part pc;
    pc.on = 0;
    pc.P = 1;
    pc.p = 0;
    pc.round = 0;
    tile::run_tile<L, NT, T, MODE>(ga, gb, gc, gd, gx, base, active, t, t == 0,
                                   t == T - 1, refine_steps, x_f64, sm, pc);
}

}  // namespace bk

// ---- host launch -----------------------------------------------------------

template <int L, int NT, int T, int MODE>
static int launch_uniform_t(const BatchArgs &A, cudaStream_t st) {
    constexpr int G = NT / T;
    const long long grid = (A.nsys + G - 1) / G;
    if (grid > 0x7fffffffLL)
        return fail(TPRGB_EUNSUPPORTED, "too many systems for one launch");
    bk::batch_uniform<L, NT, T, MODE><<<(unsigned)grid, NT, 0, st>>>(
        A.a, A.b, A.c, A.d, A.x, A.nsys, A.refine_steps, A.x_f64);
    TPRGB_CUDA(cudaGetLastError());
    return TPRGB_OK;
}

template <int L, int NT, int T>
static int launch_uniform_mode(const BatchArgs &A, cudaStream_t st) {
    if (A.refine_steps <= 0) return launch_uniform_t<L, NT, T, 0>(A, st);
    if (A.residual == TPRGB_RESID_F64) return launch_uniform_t<L, NT, T, 2>(A, st);
    return launch_uniform_t<L, NT, T, 1>(A, st);
}

// T = n / L in {2, 4, ..., NT}
template <int L, int NT>
static int launch_uniform_T(const BatchArgs &A, cudaStream_t st) {
    switch (A.n / L) {
        case 2: return launch_uniform_mode<L, NT, 2>(A, st);
        case 4: return launch_uniform_mode<L, NT, 4>(A, st);
        case 8: return launch_uniform_mode<L, NT, 8>(A, st);
        case 16: return launch_uniform_mode<L, NT, 16>(A, st);
        case 32: return launch_uniform_mode<L, NT, 32>(A, st);
        case 64: return launch_uniform_mode<L, NT, (NT >= 64 ? 64 : NT)>(A, st);
        case 128: return launch_uniform_mode<L, NT, (NT >= 128 ? 128 : NT)>(A, st);
        case 256: return launch_uniform_mode<L, NT, (NT >= 256 ? 256 : NT)>(A, st);
        case 512: return launch_uniform_mode<L, NT, (NT >= 512 ? 512 : NT)>(A, st);
        case 1024: return launch_uniform_mode<L, NT, (NT >= 1024 ? 1024 : NT)>(A, st);
        default: return fail(TPRGB_EINVAL, "unsupported threads per system");
    }
}

template <int L>
static int launch_uniform_nt(const BatchArgs &A, int nt, cudaStream_t st) {
    switch (nt) {
        case 128: return launch_uniform_T<L, 128>(A, st);
        case 256: return launch_uniform_T<L, 256>(A, st);
        case 512: return launch_uniform_T<L, 512>(A, st);
        case 1024: return launch_uniform_T<L, 1024>(A, st);
        default: return fail(TPRGB_EINVAL, "threads per CTA %d not in {128,256,512,1024}", nt);
    }
}

int batch_config_check(int n, const TileConfig &cfg) {
    if (cfg.staged == 4) {
        int P = 0;
        return cluster_parts(n, cfg, &P);
    }
    if (cfg.staged >= 2 ? (cfg.L != 8 && cfg.L != 16) : (cfg.L != 4 && cfg.L != 8))
        return fail(TPRGB_EINVAL, "equations per thread %d not in %s", cfg.L,
                    cfg.staged >= 2 ? "{8, 16}" : "{4, 8}");
    if (!is_pow2(n) || n < 2 * cfg.L)
        return fail(TPRGB_EINVAL, "n=%d must be a power of two >= %d", n, 2 * cfg.L);
    const int T = n / cfg.L;
    if (T > cfg.nt)
        return fail(TPRGB_EUNSUPPORTED,
                    "n=%d needs %d threads per system > %d per CTA", n, T, cfg.nt);
    return TPRGB_OK;
}

int launch_batch_uniform(const BatchArgs &A, const TileConfig &cfg,
                         cudaStream_t st) {
    int rc = batch_config_check(A.n, cfg);
    if (rc) return rc;
    if (A.nsys == 0) return TPRGB_OK;
    if (cfg.L == 4) return launch_uniform_nt<4>(A, cfg.nt, st);
    return launch_uniform_nt<8>(A, cfg.nt, st);
}

}  // namespace tprgb

namespace tprgb {
namespace bk {
__global__ void diag_pair_kernel(long long n, const float *hi, const float *lo,
                                 double *out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = hier::pair_to_double(hi[i], lo[i]);
}
}  // namespace bk
}  // namespace tprgb

extern "C" TPRGB_API int tprgb_diag_pair_to_double(int64_t n, const float *hi,
                                                   const float *lo, double *out,
                                                   void *stream) {
    using namespace tprgb;
    if (n < 0 || (n > 0 && (!hi || !lo || !out)))
        return fail(TPRGB_EINVAL, "bad arguments");
    if (n == 0) return TPRGB_OK;
    long long blocks = (n + 255) / 256;
    bk::diag_pair_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
        n, hi, lo, out);
    TPRGB_CUDA(cudaGetLastError());
    return TPRGB_OK;
}

// ---- bounded waits: self-test ------------------------------------------------
// Each kind of device wait in the solver kernels gives up after a bounded
// number of polls and reports TPRGB_ETIMEOUT instead of hanging.  This
// kernel runs one of them on a condition that never comes true (a flag
// nothing sets), so a test can check the give-up path and that the context
// stays usable afterwards.  which: 0 the mbarrier wait for a TMA load
// (tma::mbar_wait), 1 the cluster row-barrier wait (cl::mbar_wait, with
// cluster-scope acquire), 2 the barrier of a multi-CTA system in global
// memory (tile::part_barrier, for a system of two parts of which only this
// one runs).  Nothing faults or traps; the wait just runs out.
namespace tprgb {
namespace bk {
__global__ void selftest_wait_kernel(int which, unsigned polls, DeviceStatus *st,
                                     unsigned *counter) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ tile::Smem<32> sm;
    if (which == 0 || which == 1) {
        if (threadIdx.x == 0) {
            tma::mbar_init(&bar, 1);  // one arrival per phase; none comes
            tma::fence_barrier_init();
        }
        __syncthreads();
        const bool in = which == 0 ? tma::mbar_wait(&bar, 0, polls)
                                   : cl::mbar_wait(&bar, 0, polls);
        if (threadIdx.x == 0 && !in) {
            st->code = (unsigned)TPRGB_ETIMEOUT;
            st->where = (unsigned)which;
        }
        return;
    }
    tile::Part pc{};
    pc.on = 1;
    pc.P = 2;
    pc.p = 0;
    pc.counter = counter;
    pc.round = 0;
    pc.status = st;
    pc.item = 7;
    tile::part_barrier<32>(pc, sm, 2);
}
}  // namespace bk
}  // namespace tprgb

extern "C" TPRGB_API int tprgb_selftest_wait_timeout(int which, unsigned polls,
                                                     unsigned *status) {
    using namespace tprgb;
    if (which < 0 || which > 2 || !status) return fail(TPRGB_EINVAL, "bad arguments");
    if (which < 2 && (polls == 0 || polls > (1u << 22)))
        return fail(TPRGB_EINVAL, "polls=%u not in 1 .. 2^22", polls);
    unsigned *d = nullptr;  // DeviceStatus (4 words) then the counter
    TPRGB_CUDA(cudaMalloc(&d, 8 * sizeof(unsigned)));
    cudaError_t e = cudaMemset(d, 0, 8 * sizeof(unsigned));
    if (e == cudaSuccess) {
        bk::selftest_wait_kernel<<<1, 32>>>(which, polls,
                                            reinterpret_cast<DeviceStatus *>(d), d + 4);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(status, d, 3 * sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "tprgb_selftest_wait_timeout");
    return TPRGB_OK;
}
