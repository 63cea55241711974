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
// stays in registers.
#include <algorithm>

#include "batch.cuh"
#include "common.cuh"
#include "hier.cuh"

namespace tprgb {
namespace bk {

using hier::Chunk;
using hier::Row;

// Segment rows exchanged between the warps of a system (level 2).
struct SegRows {
    Row R0, R1;
};

template <int L>
__device__ __forceinline__ void load_chunk(const float *__restrict__ p,
                                           float (&v)[L]) {
    const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
    for (int i = 0; i < L / 4; i++) {
        float4 t = __ldg(q + i);
        v[4 * i + 0] = t.x;
        v[4 * i + 1] = t.y;
        v[4 * i + 2] = t.z;
        v[4 * i + 3] = t.w;
    }
}

// Full hierarchical solve of the system whose rows this thread holds.
// Returns x for the thread's L equations.  All threads of the CTA must call
// it (it contains CTA barriers when a system spans several warps).
template <int L, int NT>
__device__ __forceinline__ void solve_levels(const float (&a)[L],
                                             const float (&b)[L],
                                             const float (&c)[L],
                                             const float (&d)[L], int T,
                                             float (&x)[L], SegRows *sh_rows,
                                             float2 *sh_x) {
    const int tid = threadIdx.x;
    const int K = T < 32 ? T : 32;
    const int q = (tid & 31) % K;      // lane within the segment
    Chunk<L> ck;
    hier::level0<L>(a, b, c, d, ck);
    Row R0 = ck.F, R1 = ck.E;
    hier::seg_reduce(R0, R1, q, K);
    float xf, xl;
    if (T <= 32) {
        hier::seg_top(R0, R1, q, K, xf, xl);
    } else {
        // level 2: segment boundary rows of this system -> shared memory
        const int W = T >> 5;                 // warp segments per system
        const int warp = tid >> 5;
        const int sys_warp0 = warp & ~(W - 1);  // first warp of the system
        const int w = warp - sys_warp0;
        if (q == 0) sh_rows[warp].R0 = R0;
        if (q == 31) sh_rows[warp].R1 = R1;
        __syncthreads();
        if (w == 0) {
            // lanes 0..W-1 of the system's first warp solve the 2W rows
            const int lane = tid & 31;
            Row S0, S1;
            if (lane < W) {
                S0 = sh_rows[sys_warp0 + lane].R0;
                S1 = sh_rows[sys_warp0 + lane].R1;
            } else {
                S0 = Row{0.f, 0.f, 0.f};
                S1 = Row{0.f, 0.f, 0.f};
            }
            const int q2 = lane % W;
            hier::seg_reduce(S0, S1, q2, W);
            float yf, yl, y0, y1;
            hier::seg_top(S0, S1, q2, W, yf, yl);
            hier::seg_back(S0, S1, q2, W, yf, yl, y0, y1);
            if (lane < W) sh_x[sys_warp0 + lane] = make_float2(y0, y1);
        }
        __syncthreads();
        float2 v = sh_x[warp];
        xf = v.x;
        xl = v.y;
    }
    float x0, x1;
    hier::seg_back(R0, R1, q, K, xf, xl, x0, x1);
    hier::level0_back<L>(ck, x0, x1, x);
}

// Neighbour values x[-1] (from the previous thread of the system) and
// x[L] (from the next), zero at the system boundaries.
template <int L, int NT>
__device__ __forceinline__ void neighbours(float hfirst, float hlast,
                                           float lfirst, float llast, int T,
                                           float &hm, float &lm, float &hp,
                                           float &lp, float4 *sh_edge) {
    const int tid = threadIdx.x;
    const int t = tid % T;  // thread index within the system
    const int lane = tid & 31;
    const int K = T < 32 ? T : 32;
    hm = __shfl_up_sync(0xffffffffu, hlast, 1, K);
    lm = __shfl_up_sync(0xffffffffu, llast, 1, K);
    hp = __shfl_down_sync(0xffffffffu, hfirst, 1, K);
    lp = __shfl_down_sync(0xffffffffu, lfirst, 1, K);
    if (T > 32) {
        const int warp = tid >> 5;
        if (lane == 0) sh_edge[2 * warp] = make_float4(hfirst, lfirst, 0.f, 0.f);
        if (lane == 31) sh_edge[2 * warp + 1] = make_float4(hlast, llast, 0.f, 0.f);
        __syncthreads();
        if (lane == 0 && t > 0) {
            float4 v = sh_edge[2 * (warp - 1) + 1];
            hm = v.x;
            lm = v.y;
        }
        if (lane == 31 && t < T - 1) {
            float4 v = sh_edge[2 * (warp + 1)];
            hp = v.x;
            lp = v.y;
        }
        __syncthreads();
    }
    if (t == 0) {
        hm = 0.f;
        lm = 0.f;
    }
    if (t == T - 1) {
        hp = 0.f;
        lp = 0.f;
    }
}

// MODE: 0 = plain FP32 solve; 1 = refinement with compensated-FP32
// residual; 2 = refinement with native FP64 residual.
template <int L, int NT, int MODE>
__global__ void __launch_bounds__(NT)
batch_uniform(const float *__restrict__ ga, const float *__restrict__ gb,
              const float *__restrict__ gc, const float *__restrict__ gd,
              void *__restrict__ gx, int nsys, int n, int refine_steps,
              int x_f64) {
    __shared__ SegRows sh_rows[NT / 32];
    __shared__ float2 sh_x[NT / 32];
    __shared__ float4 sh_edge[2 * (NT / 32)];

    const int T = n / L;
    const int G = NT / T;
    const int tid = threadIdx.x;
    const int g = tid / T, t = tid - g * T;
    const long long sys = (long long)blockIdx.x * G + g;
    const bool active = sys < nsys;
    const long long base = sys * (long long)n + (long long)t * L;

    float a[L], b[L], c[L], d[L];
    if (active) {
        load_chunk<L>(ga + base, a);
        load_chunk<L>(gb + base, b);
        load_chunk<L>(gc + base, c);
        load_chunk<L>(gd + base, d);
    } else {
#pragma unroll
        for (int i = 0; i < L; i++) {
            a[i] = 0.f;
            b[i] = 1.f;
            c[i] = 0.f;
            d[i] = 0.f;
        }
    }
    // a[0] and c[n-1] of the system do not take part
    if (t == 0) a[0] = 0.f;
    if (t == T - 1) c[L - 1] = 0.f;

    float xh[L];
    solve_levels<L, NT>(a, b, c, d, T, xh, sh_rows, sh_x);

    float xlo[L];
    double xd[L];
#pragma unroll
    for (int i = 0; i < L; i++) {
        xlo[i] = 0.f;
        if (MODE == 2) xd[i] = (double)xh[i];
    }

    if (MODE != 0) {
        for (int step = 0; step < refine_steps; step++) {
            float r[L];
            if (MODE == 1) {
                float hm, lm, hp, lp;
                neighbours<L, NT>(xh[0], xh[L - 1], xlo[0], xlo[L - 1], T, hm,
                                  lm, hp, lp, sh_edge);
#pragma unroll
                for (int i = 0; i < L; i++) {
                    float xmh = i > 0 ? xh[i - 1] : hm;
                    float xml = i > 0 ? xlo[i - 1] : lm;
                    float xph = i < L - 1 ? xh[i + 1] : hp;
                    float xpl = i < L - 1 ? xlo[i + 1] : lp;
                    r[i] = hier::residual_df(a[i], b[i], c[i], d[i], xmh, xml,
                                             xh[i], xlo[i], xph, xpl);
                }
            } else {
                // native FP64: exchange x as (hi, lo) float pairs of the
                // double so the neighbour exchange stays 32-bit
                float hm, lm, hp, lp;
                float f_h = (float)xd[0], f_l = (float)(xd[0] - (double)f_h);
                float l_h = (float)xd[L - 1];
                float l_l = (float)(xd[L - 1] - (double)l_h);
                neighbours<L, NT>(f_h, l_h, f_l, l_l, T, hm, lm, hp, lp,
                                  sh_edge);
                double xm = (double)hm + (double)lm;
                double xp = (double)hp + (double)lp;
#pragma unroll
                for (int i = 0; i < L; i++) {
                    double xl_ = i > 0 ? xd[i - 1] : xm;
                    double xr_ = i < L - 1 ? xd[i + 1] : xp;
                    double rr = (double)d[i];
                    rr = fma(-(double)b[i], xd[i], rr);
                    rr = fma(-(double)a[i], xl_, rr);
                    rr = fma(-(double)c[i], xr_, rr);
                    r[i] = (float)rr;
                }
            }
            float dx[L];
            solve_levels<L, NT>(a, b, c, r, T, dx, sh_rows, sh_x);
#pragma unroll
            for (int i = 0; i < L; i++) {
                if (MODE == 1)
                    xlo[i] += dx[i];
                else
                    xd[i] += (double)dx[i];
            }
        }
    }

    if (!active) return;
    if (x_f64) {
        double2 *o = reinterpret_cast<double2 *>((double *)gx + base);
#pragma unroll
        for (int i = 0; i < L / 2; i++) {
            double v0, v1;
            if (MODE == 2) {
                v0 = xd[2 * i];
                v1 = xd[2 * i + 1];
            } else {
                v0 = hier::pair_to_double(xh[2 * i], xlo[2 * i]);
                v1 = hier::pair_to_double(xh[2 * i + 1], xlo[2 * i + 1]);
            }
            o[i] = make_double2(v0, v1);
        }
    } else {
        float4 *o = reinterpret_cast<float4 *>((float *)gx + base);
#pragma unroll
        for (int i = 0; i < L / 4; i++) {
            float v[4];
#pragma unroll
            for (int j = 0; j < 4; j++)
                v[j] = MODE == 2 ? (float)xd[4 * i + j]
                                 : xh[4 * i + j] + xlo[4 * i + j];
            o[i] = make_float4(v[0], v[1], v[2], v[3]);
        }
    }
}

}  // namespace bk

// ---- host launch -----------------------------------------------------------

template <int L, int NT, int MODE>
static int launch_uniform_t(const BatchArgs &A, cudaStream_t st) {
    const int T = A.n / L;
    const int G = NT / T;
    const long long grid = (A.nsys + G - 1) / G;
    if (grid > 0x7fffffffLL)
        return fail(TPRGB_EUNSUPPORTED, "too many systems for one launch");
    bk::batch_uniform<L, NT, MODE><<<(unsigned)grid, NT, 0, st>>>(
        A.a, A.b, A.c, A.d, A.x, A.nsys, A.n, A.refine_steps, A.x_f64);
    TPRGB_CUDA(cudaGetLastError());
    return TPRGB_OK;
}

template <int L, int NT>
static int launch_uniform_mode(const BatchArgs &A, cudaStream_t st) {
    if (A.refine_steps <= 0) return launch_uniform_t<L, NT, 0>(A, st);
    if (A.residual == TPRGB_RESID_F64) return launch_uniform_t<L, NT, 2>(A, st);
    return launch_uniform_t<L, NT, 1>(A, st);
}

template <int L>
static int launch_uniform_nt(const BatchArgs &A, int nt, cudaStream_t st) {
    switch (nt) {
        case 128: return launch_uniform_mode<L, 128>(A, st);
        case 256: return launch_uniform_mode<L, 256>(A, st);
        case 512: return launch_uniform_mode<L, 512>(A, st);
        case 1024: return launch_uniform_mode<L, 1024>(A, st);
        default: return fail(TPRGB_EINVAL, "threads per CTA %d not in {128,256,512,1024}", nt);
    }
}

int batch_config_check(int n, const TileConfig &cfg) {
    if (cfg.L != 4 && cfg.L != 8)
        return fail(TPRGB_EINVAL, "equations per thread %d not in {4, 8}", cfg.L);
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
