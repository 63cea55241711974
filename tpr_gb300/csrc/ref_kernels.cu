// Reference-semantics TPR / PTPR / CR / PCR kernels.
//
// These reproduce the reference solvers' arithmetic step for step -- the
// same eliminations, the same operand order, IEEE division, and this
// translation unit is compiled with -fmad=false -- so on the same inputs
// they return the same bits as the reference's CPU classes
// (src/ptpr.cpp:103-287, src/tpr.cpp:95-308, src/cr.cpp:23-116,
// src/pcr.cpp:15-89).  They are the plain single-system path (one system per
// CTA, any number of systems per launch) and the FP64 path.
//
// Two shapes:
//  * fused: one CTA holds a whole system in shared memory and runs stage 1,
//    the intermediate stage, stage 2 and stage 3 with CTA barriers only.
//    The reference instead needs one CTA per slice and a cooperative grid
//    sync between stages (src/ptpr.cu:48-150), which caps it at n <= s^2.
//  * sliced (systems too large for one CTA's shared memory): stage 1 per
//    slice CTA -> global workspace, stage 2 in one CTA per system, stage 3
//    per slice CTA.  Three launches on one stream, no grid sync.
#include <cooperative_groups.h>

#include <algorithm>
#include <mutex>
#include <type_traits>

#include "common.cuh"

namespace tprgb {
namespace refk {

constexpr int kThreads = 1024;
constexpr int kEpt = 8;  // max elements per thread in a CTA sweep

// ---- three-point updates (operand order of the CPU reference) ----------
// mid: src/ptpr.cpp:145-166, upper: :131-143, lower: :168-180
template <typename T>
__device__ __forceinline__ void upd_mid(const T *a, const T *c, const T *r,
                                        int kl, int k, int kr, T &oa, T &oc,
                                        T &orr) {
    T inv = T(1) / (T(1) - c[kl] * a[k] - a[kr] * c[k]);
    oa = -inv * a[kl] * a[k];
    oc = -inv * c[kr] * c[k];
    orr = inv * (r[k] - r[kl] * a[k] - r[kr] * c[k]);
}
template <typename T>
__device__ __forceinline__ void upd_upper(const T *a, const T *c, const T *r,
                                          int k, int kr, T &oa, T &oc,
                                          T &orr) {
    T inv = T(1) / (T(1) - a[kr] * c[k]);
    oa = inv * a[k];
    oc = -inv * c[kr] * c[k];
    orr = inv * (r[k] - r[kr] * c[k]);
}
template <typename T>
__device__ __forceinline__ void upd_lower(const T *a, const T *c, const T *r,
                                          int kl, int k, T &oa, T &oc,
                                          T &orr) {
    T inv = T(1) / (T(1) - c[kl] * a[k]);
    oa = -inv * a[kl] * a[k];
    oc = inv * c[k];
    orr = inv * (r[k] - r[kl] * a[k]);
}

// PTPR stage 1 on rows [0, n) of shared arrays holding whole slices of size
// s: log2(s) PCR steps with slice-local boundaries (src/ptpr.cpp:130-190).
template <typename T>
__device__ void ptpr_stage1(T *a, T *c, T *r, int n, int s) {
    const int ls = ilog2(s);
    for (int p = 1; p <= ls; p++) {
        const int u = 1 << (p - 1);
        T na[kEpt], nc[kEpt], nr[kEpt];
#pragma unroll
        for (int e = 0; e < kEpt; e++) {
            int i = threadIdx.x + e * blockDim.x;
            if (i < n) {
                int li = i & (s - 1);
                if (li < u)
                    upd_upper(a, c, r, i, i + u, na[e], nc[e], nr[e]);
                else if (li <= s - 1 - u)
                    upd_mid(a, c, r, i - u, i, i + u, na[e], nc[e], nr[e]);
                else
                    upd_lower(a, c, r, i - u, i, na[e], nc[e], nr[e]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < kEpt; e++) {
            int i = threadIdx.x + e * blockDim.x;
            if (i < n) {
                a[i] = na[e];
                c[i] = nc[e];
                r[i] = nr[e];
            }
        }
        __syncthreads();
    }
}

// PTPR stage 1 on one slice of s rows, EPT rows per thread (s <= EPT *
// blockDim.x), double-buffered: step p reads one copy of a, c, r and writes
// the other, so a step needs one CTA barrier.  The per-row arithmetic is
// ptpr_stage1's.  Returns 1 when the result is in the second copy (an odd
// number of steps), else 0.
template <typename T, int EPT>
__device__ int ptpr_stage1_slice(T *a0, T *c0, T *r0, T *a1, T *c1, T *r1, int s) {
    const int ls = ilog2(s);
    for (int p = 1; p <= ls; p++) {
        const int u = 1 << (p - 1);
        const bool odd = (p & 1) == 0;  // step p reads copy (p - 1) & 1
        const T *a = odd ? a1 : a0, *c = odd ? c1 : c0, *r = odd ? r1 : r0;
        T *oa = odd ? a0 : a1, *oc = odd ? c0 : c1, *orr = odd ? r0 : r1;
#pragma unroll
        for (int e = 0; e < EPT; e++) {
            const int i = threadIdx.x + e * blockDim.x;
            if (i < s) {
                T na, nc, nr;
                if (i < u)
                    upd_upper(a, c, r, i, i + u, na, nc, nr);
                else if (i <= s - 1 - u)
                    upd_mid(a, c, r, i - u, i, i + u, na, nc, nr);
                else
                    upd_lower(a, c, r, i - u, i, na, nc, nr);
                oa[i] = na;
                oc[i] = nc;
                orr[i] = nr;
            }
        }
        __syncthreads();
    }
    return ls & 1;
}

// TPR stage 1 on one slice of s rows, EPT rows per thread.  At level p >= 2
// the rows updated (li % 2^p in {0, 2^p - 1}) are never the neighbours
// (li +- 2^(p-1)) of an updated row, so a level writes in place after its
// reads with one CTA barrier; level 1 updates every row and keeps two.  The
// per-row arithmetic is tpr_stage1's.
template <typename T, int EPT>
__device__ void tpr_stage1_slice(T *a, T *c, T *r, int s) {
    const int ls = ilog2(s);
    // levels from pw on update at most 32 rows (2 s / 2^p): warp 0 runs them
    // alone with warp barriers; the caller's CTA barrier publishes them
    int pw = ls + 1;
    while (pw - 1 >= 2 && ((2 * s) >> (pw - 1)) <= 32) pw--;
    for (int p = 1; p < pw; p++) {
        const int u = 1 << (p - 1), p2k = 1 << p;
        T na[EPT], nc[EPT], nr[EPT];
        bool sel[EPT];
#pragma unroll
        for (int e = 0; e < EPT; e++) {
            const int i = threadIdx.x + e * blockDim.x;
            sel[e] = i < s && (((i & (p2k - 1)) == 0) || (((i + 1) & (p2k - 1)) == 0));
            if (sel[e]) {
                if (i == 0)
                    upd_upper(a, c, r, i, i + u, na[e], nc[e], nr[e]);
                else if (i == s - 1)
                    upd_lower(a, c, r, i - u, i, na[e], nc[e], nr[e]);
                else
                    upd_mid(a, c, r, i - u, i, i + u, na[e], nc[e], nr[e]);
            }
        }
        if (p == 1) __syncthreads();
#pragma unroll
        for (int e = 0; e < EPT; e++) {
            const int i = threadIdx.x + e * blockDim.x;
            if (sel[e]) {
                a[i] = na[e];
                c[i] = nc[e];
                r[i] = nr[e];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        for (int p = pw; p <= ls; p++) {  // lane: row pair k = lane / 2, end lane & 1
            const int u = 1 << (p - 1), p2k = 1 << p;
            const int k = lane >> 1;
            if (k < (s >> p)) {
                const int i = k * p2k + ((lane & 1) ? p2k - 1 : 0);
                T na, nc, nr;
                if (i == 0)
                    upd_upper(a, c, r, i, i + u, na, nc, nr);
                else if (i == s - 1)
                    upd_lower(a, c, r, i - u, i, na, nc, nr);
                else
                    upd_mid(a, c, r, i - u, i, i + u, na, nc, nr);
                a[i] = na;
                c[i] = nc;
                r[i] = nr;
            }
            __syncwarp();
        }
    }
}

// TPR stage 1 tree levels (src/tpr.cpp:123-230): at level p only rows with
// li % 2^p == 0 or (li+1) % 2^p == 0 are updated.
template <typename T, int EPT = kEpt>
__device__ void tpr_stage1(T *a, T *c, T *r, int n, int s) {
    const int ls = ilog2(s);
    for (int p = 1; p <= ls; p++) {
        const int u = 1 << (p - 1), p2k = 1 << p;
        T na[EPT], nc[EPT], nr[EPT];
        bool sel[EPT];
#pragma unroll
        for (int e = 0; e < EPT; e++) {
            int i = threadIdx.x + e * blockDim.x;
            sel[e] = false;
            if (i < n) {
                int li = i & (s - 1);
                sel[e] = ((li & (p2k - 1)) == 0) || (((li + 1) & (p2k - 1)) == 0);
                if (sel[e]) {
                    if (li == 0)
                        upd_upper(a, c, r, i, i + u, na[e], nc[e], nr[e]);
                    else if (li == s - 1)
                        upd_lower(a, c, r, i - u, i, na[e], nc[e], nr[e]);
                    else
                        upd_mid(a, c, r, i - u, i, i + u, na[e], nc[e], nr[e]);
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < EPT; e++) {
            int i = threadIdx.x + e * blockDim.x;
            if (sel[e]) {
                a[i] = na[e];
                c[i] = nc[e];
                r[i] = nr[e];
            }
        }
        __syncthreads();
    }
}

// E_st <- E_st + s1 E_ed (src/ptpr.cpp:192-201, src/tpr.cpp:327-340).
template <typename T>
__device__ __forceinline__ void est_update(T *a, T *c, T *r, int st, int ed) {
    T s1;
    if (fabs(c[ed]) < Eps<T>::value)
        s1 = T(-1.0);
    else
        s1 = -c[st] / c[ed];
    a[st] += s1 * a[ed];
    c[st] = s1;
    r[st] += s1 * r[ed];
}

// Reduced equation j from rows ed_j = j*s + s - 1 and ed_j + 1
// (src/ptpr.cpp:218-241).  row(k) returns (a, c, r) of row k.
template <typename T>
__device__ __forceinline__ void inter_eq(T ak, T ck, T rk, T akr, T ckr,
                                         T rkr, T &sa, T &sc, T &sr) {
    T inv = T(1) / (T(1) - akr * ck);
    sa = inv * ak;
    sc = -inv * ckr * ck;
    sr = inv * (rk - rkr * ck);
}

// Row k of one PCR step at distance s over m rows (src/pcr.cpp:30-75):
// reads rows k - s, k, k + s of the previous step.
template <typename T>
__device__ __forceinline__ void pcr_row(const T *a, const T *c, const T *r,
                                        int k, int m, int s, T &na, T &nc,
                                        T &nr) {
    if (k < s) {
        int kr = k + s;
        T ee = T(1) / (T(1) - c[k] * a[kr]);
        na = ee * a[k];
        nc = -ee * c[k] * c[kr];
        nr = ee * (r[k] - c[k] * r[kr]);
    } else if (k < m - s) {
        int kl = k - s, kr = k + s;
        T ap = a[k], cp = c[k];
        T ee = T(1) / (T(1) - ap * c[kl] - cp * a[kr]);
        na = -ee * ap * a[kl];
        nc = -ee * cp * c[kr];
        nr = ee * (r[k] - ap * r[kl] - cp * r[kr]);
    } else {
        int kl = k - s;
        T ap = a[k], cp = c[k];
        T ee = T(1) / (T(1) - ap * c[kl]);
        na = -ee * ap * a[kl];
        nc = ee * cp;
        nr = ee * (r[k] - ap * r[kl]);
    }
}

// Row i of CR forward level p (u = 2^p; src/cr.cpp:48-69): reads rows
// i - u, i, i + u.
template <typename T>
__device__ __forceinline__ void cr_row(const T *a, const T *c, const T *r,
                                       int i, int u, int m, T &na, T &nc,
                                       T &nr) {
    if (i < m - 2 * u)
        upd_mid(a, c, r, i - u, i, i + u, na, nc, nr);
    else
        upd_lower(a, c, r, i - u, i, na, nc, nr);
}

// The last two rows of CR, m >= 2 (src/cr.cpp:89-96).
template <typename T>
__device__ __forceinline__ void cr_top(const T *a, const T *c, const T *r,
                                       T *x, int m) {
    const int i = m / 2 - 1, u = m / 2;
    T inv_det = T(1) / (T(1) - c[i] * a[i + u]);
    x[i] = (r[i] - c[i] * r[i + u]) * inv_det;
    x[i + u] = (r[i + u] - r[i] * a[i + u]) * inv_det;
}

// Row i of CR back substitution at distance u, i < m - u
// (src/cr.cpp:98-112).
template <typename T>
__device__ __forceinline__ T cr_back_row(const T *a, const T *c, const T *r,
                                         const T *x, int i, int u) {
    if (i == u - 1) return r[i] - c[i] * x[i + u];
    return r[i] - a[i] * x[i - u] - c[i] * x[i + u];
}

// PCR on m rows in shared memory (src/pcr.cpp:15-89); rhs holds x on exit.
template <typename T, int EPT = kEpt>
__device__ void cta_pcr(T *a, T *c, T *r, int m) {
    const int pn = ilog2(m);
    for (int p = 0; p < pn; p++) {
        const int s = 1 << p;
        T na[EPT], nc[EPT], nr[EPT];
#pragma unroll
        for (int e = 0; e < EPT; e++) {
            int k = threadIdx.x + e * blockDim.x;
            if (k < m) pcr_row<T>(a, c, r, k, m, s, na[e], nc[e], nr[e]);
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < EPT; e++) {
            int k = threadIdx.x + e * blockDim.x;
            if (k < m) {
                a[k] = na[e];
                c[k] = nc[e];
                r[k] = nr[e];
            }
        }
        __syncthreads();
    }
}

// CR on m rows in shared memory (src/cr.cpp:23-116); solution into x.
template <typename T, int EPT = kEpt>
__device__ void cta_cr(T *a, T *c, T *r, T *x, int m) {
    if (m <= 1) {
        if (threadIdx.x == 0) x[0] = r[0];
        __syncthreads();
        return;
    }
    const int ln = ilog2(m);
    for (int p = 0; p < ln - 1; p++) {
        const int u = 1 << p, ux = 1 << (p + 1);
        const int rows = m / ux;  // rows ux-1 + ux*j, j < rows; last is m-1
        T na[EPT], nc[EPT], nr[EPT];
#pragma unroll
        for (int e = 0; e < EPT; e++) {
            int j = threadIdx.x + e * blockDim.x;
            if (j < rows)
                cr_row<T>(a, c, r, ux - 1 + ux * j, u, m, na[e], nc[e], nr[e]);
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < EPT; e++) {
            int j = threadIdx.x + e * blockDim.x;
            if (j < rows) {
                int i = ux - 1 + ux * j;
                a[i] = na[e];
                c[i] = nc[e];
                r[i] = nr[e];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) cr_top<T>(a, c, r, x, m);
    __syncthreads();
    for (int k = ln - 2; k >= 0; k--) {
        const int u = 1 << k;
        const int rows = m / (2 * u);  // rows u-1 + 2u*j
        for (int j = threadIdx.x; j < rows; j += blockDim.x) {
            const int i = u - 1 + 2 * u * j;  // i < m - u for every j
            x[i] = cr_back_row<T>(a, c, r, x, i, u);
        }
        __syncthreads();
    }
}

// PCR on m <= 32 rows by one warp (lane k: row k): cta_pcr's arithmetic and
// order with warp barriers; the caller's CTA barrier publishes the result.
template <typename T>
__device__ void warp_pcr(T *a, T *c, T *r, int m) {
    const int lane = threadIdx.x & 31;
    const int pn = ilog2(m);
    for (int p = 0; p < pn; p++) {
        T na, nc, nr;
        if (lane < m) pcr_row<T>(a, c, r, lane, m, 1 << p, na, nc, nr);
        __syncwarp();
        if (lane < m) {
            a[lane] = na;
            c[lane] = nc;
            r[lane] = nr;
        }
        __syncwarp();
    }
}

// CR on m <= 32 rows by one warp, solution into x: cta_cr's arithmetic and
// order with warp barriers.
template <typename T>
__device__ void warp_cr(T *a, T *c, T *r, T *x, int m) {
    const int lane = threadIdx.x & 31;
    if (m <= 1) {
        if (lane == 0) x[0] = r[0];
        __syncwarp();
        return;
    }
    const int ln = ilog2(m);
    for (int p = 0; p < ln - 1; p++) {
        const int u = 1 << p, ux = 2 * u;
        const int i = ux - 1 + ux * lane;
        const bool on = lane < m / ux;
        T na, nc, nr;
        if (on) cr_row<T>(a, c, r, i, u, m, na, nc, nr);
        __syncwarp();
        if (on) {
            a[i] = na;
            c[i] = nc;
            r[i] = nr;
        }
        __syncwarp();
    }
    if (lane == 0) cr_top<T>(a, c, r, x, m);
    __syncwarp();
    for (int k = ln - 2; k >= 0; k--) {
        const int u = 1 << k;
        if (lane < m / (2 * u)) {
            const int i = u - 1 + 2 * u * lane;
            x[i] = cr_back_row<T>(a, c, r, x, i, u);
        }
        __syncwarp();
    }
}

// Shared-memory footprint of the fused kernel, in elements of T.
__host__ __device__ inline long long fused_elems(int n, int s) {
    long long m = n / s;
    return 4LL * n + 2 + 7 * m;
}

// One CTA per system: the whole TPR / PTPR solve in shared memory.
// Inputs are diag-normalised (unit diagonal) and left untouched.
template <typename T, int KIND>
__global__ void __launch_bounds__(kThreads)
fused_tpr(const T *__restrict__ ga, const T *__restrict__ gc,
          const T *__restrict__ gr, T *__restrict__ gx, int n, int s,
          long long stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    const int m = n / s;
    T *a = sm, *c = sm + n, *r = sm + 2 * n;
    T *xs = sm + 3 * n;  // xs[0] is the x[-1] = 0 sentinel
    T *x = xs + 1;
    T *sa = xs + n + 1, *sc = sa + m, *sr = sc + m, *sx = sr + m;
    T *ba = sx + m, *bc = ba + m, *br = bc + m;
    const long long base = (long long)blockIdx.x * stride;
    ga += base;
    gc += base;
    gr += base;
    gx += base;

    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        a[i] = ga[i];
        c[i] = gc[i];
        r[i] = gr[i];
    }
    if (threadIdx.x == 0) xs[0] = T(0);
    __syncthreads();

    if (KIND == TPRGB_PTPR)
        ptpr_stage1(a, c, r, n, s);
    else
        tpr_stage1(a, c, r, n, s);

    for (int j = threadIdx.x; j < m; j += blockDim.x) {
        int st = j * s, ed = st + s - 1;
        if (KIND == TPRGB_PTPR) {  // backup E_st for stage 3
            ba[j] = a[st];
            bc[j] = c[st];
            br[j] = r[st];
        }
        est_update(a, c, r, st, ed);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
        int k = j * s + s - 1;
        if (j < m - 1)
            inter_eq(a[k], c[k], r[k], a[k + 1], c[k + 1], r[k + 1], sa[j],
                     sc[j], sr[j]);
        else {
            sa[j] = a[n - 1];
            sc[j] = c[n - 1];
            sr[j] = r[n - 1];
        }
    }
    __syncthreads();

    if (KIND == TPRGB_PTPR) {
        cta_pcr(sa, sc, sr, m);  // src/ptpr.cpp:246-258
        for (int j = threadIdx.x; j < m; j += blockDim.x)
            x[j * s + s - 1] = sr[j];
        for (int j = threadIdx.x; j < m; j += blockDim.x) {
            int st = j * s;  // restore E_st, src/ptpr.cpp:266-271
            a[st] = ba[j];
            c[st] = bc[j];
            r[st] = br[j];
        }
        __syncthreads();
        // stage 3, src/ptpr.cpp:263-287
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            int st = i & ~(s - 1), ed = st + s - 1;
            if (i == ed) continue;
            T key = T(1) / c[ed] * (r[ed] - a[ed] * x[st - 1] - x[ed]);
            if (c[ed] == T(0)) key = T(0);
            x[i] = r[i] - a[i] * x[st - 1] - c[i] * key;
        }
        __syncthreads();
    } else {
        cta_cr(sa, sc, sr, sx, m);  // src/tpr.cpp:263-275
        for (int j = threadIdx.x; j < m; j += blockDim.x)
            x[j * s + s - 1] = sx[j];
        // restore: even slice-local rows from the untouched inputs, odd
        // rows keep their post-stage-1 values (src/tpr.cpp:236-325,381-387)
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            if (((i & (s - 1)) & 1) == 0) {
                a[i] = ga[i];
                c[i] = gc[i];
                r[i] = gr[i];
            }
        }
        __syncthreads();
        const int ls = ilog2(s);
        for (int p = ls - 1; p >= 0; p--) {  // src/tpr.cpp:277-308
            const int u = 1 << p;
            const int per = s / (2 * u);  // rows per slice at this level
            for (int t = threadIdx.x; t < m * per; t += blockDim.x) {
                int j = t / per, q = t - j * per;
                int i = j * s + u - 1 + 2 * u * q;
                T xu = (i - u < 0) ? T(0) : x[i - u];
                x[i] = r[i] - a[i] * xu - c[i] * x[i + u];
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) gx[i] = x[i];
}

// Standalone CR / PCR on one system per CTA (src/cr.cpp, src/pcr.cpp).
template <typename T, int KIND>
__global__ void __launch_bounds__(kThreads)
fused_crpcr(const T *__restrict__ ga, const T *__restrict__ gc,
            const T *__restrict__ gr, T *__restrict__ gx, int n,
            long long stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    T *a = sm, *c = sm + n, *r = sm + 2 * n, *x = sm + 3 * n;
    const long long base = (long long)blockIdx.x * stride;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        a[i] = ga[base + i];
        c[i] = gc[base + i];
        r[i] = gr[base + i];
    }
    __syncthreads();
    if (KIND == TPRGB_PCR) {
        cta_pcr(a, c, r, n);
        for (int i = threadIdx.x; i < n; i += blockDim.x) gx[base + i] = r[i];
    } else {
        cta_cr(a, c, r, x, n);
        for (int i = threadIdx.x; i < n; i += blockDim.x) gx[base + i] = x[i];
    }
}

// ---- standalone CR / PCR on systems larger than one CTA's shared memory ----
// The rows live in a global workspace (L2-resident at these sizes) and each
// level is one launch over all rows of all systems (blockIdx.y = system), or
// -- for CR's levels of at most kThreads rows -- one CTA per system runs them
// back to back.  Same per-row arithmetic as the shared-memory kernels.

// One PCR step at distance s: reads the previous step's rows (the inputs at
// s = 1), writes this step's; the last step writes only x (into orr).
template <typename T>
__global__ void __launch_bounds__(256)
pcr_step(const T *__restrict__ ia, const T *__restrict__ ic,
         const T *__restrict__ ir, long long istride, T *__restrict__ oa,
         T *__restrict__ oc, T *__restrict__ orr, long long ostride, int m,
         int s, int last) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const long long ib = blockIdx.y * istride, ob = blockIdx.y * ostride;
    T na, nc, nr;
    pcr_row<T>(ia + ib, ic + ib, ir + ib, k, m, s, na, nc, nr);
    if (!last) {
        oa[ob + k] = na;
        oc[ob + k] = nc;
    }
    orr[ob + k] = nr;
}

// CR forward level 0 from the inputs into the workspace w (stride
// wstride): odd rows reduced, even rows copied, so that w holds every row
// the later levels and the back substitution read.
template <typename T>
__global__ void __launch_bounds__(256)
cr_first(const T *__restrict__ ga, const T *__restrict__ gc,
         const T *__restrict__ gr, long long stride, T *__restrict__ wa,
         T *__restrict__ wc, T *__restrict__ wr, long long wstride, int m) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m / 2) return;
    const long long gb = blockIdx.y * stride, wb = blockIdx.y * wstride;
    ga += gb;
    gc += gb;
    gr += gb;
    wa += wb;
    wc += wb;
    wr += wb;
    const int i = 2 * j + 1;
    T na, nc, nr;
    cr_row<T>(ga, gc, gr, i, 1, m, na, nc, nr);
    wa[i - 1] = ga[i - 1];
    wc[i - 1] = gc[i - 1];
    wr[i - 1] = gr[i - 1];
    wa[i] = na;
    wc[i] = nc;
    wr[i] = nr;
}

// CR forward level p >= 1 in place: row i = 2u - 1 + 2u j reads rows i +- u,
// which this level does not write, so no row is read after another thread
// wrote it.
template <typename T>
__global__ void __launch_bounds__(256)
cr_forward(T *wa, T *wc, T *wr, long long wstride, int m, int p) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int u = 1 << p;
    if (j >= (m >> (p + 1))) return;
    const long long wb = blockIdx.y * wstride;
    const int i = 2 * u - 1 + 2 * u * j;
    T na, nc, nr;
    cr_row<T>(wa + wb, wc + wb, wr + wb, i, u, m, na, nc, nr);
    wa[wb + i] = na;
    wc[wb + i] = nc;
    wr[wb + i] = nr;
}

// CR back substitution at distance u = 2^k into x (stride xstride).
template <typename T>
__global__ void __launch_bounds__(256)
cr_backward(const T *wa, const T *wc, const T *wr, long long wstride, T *gx,
            long long xstride, int m, int k) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int u = 1 << k;
    if (j >= (m >> (k + 1))) return;
    const long long wb = blockIdx.y * wstride;
    const int i = u - 1 + 2 * u * j;
    T *x = gx + blockIdx.y * xstride;
    x[i] = cr_back_row<T>(wa + wb, wc + wb, wr + wb, x, i, u);
}

// CR levels p0 .. log2(m) - 2 forward, the last two rows, and back
// substitution down to level p0, on one CTA per system: every level of
// these has at most blockDim.x rows.  Global writes of one level are
// visible to the block's other threads after the barrier.
template <typename T>
__global__ void __launch_bounds__(kThreads)
cr_tail(T *wa, T *wc, T *wr, long long wstride, T *gx, long long xstride,
        int m, int p0) {
    const long long wb = blockIdx.x * wstride;
    wa += wb;
    wc += wb;
    wr += wb;
    T *x = gx + blockIdx.x * xstride;
    const int ln = ilog2(m);
    for (int p = p0; p < ln - 1; p++) {
        const int u = 1 << p;
        const int j = threadIdx.x;
        if (j < (m >> (p + 1))) {
            const int i = 2 * u - 1 + 2 * u * j;
            T na, nc, nr;
            cr_row<T>(wa, wc, wr, i, u, m, na, nc, nr);
            wa[i] = na;
            wc[i] = nc;
            wr[i] = nr;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) cr_top<T>(wa, wc, wr, x, m);
    __syncthreads();
    for (int k = ln - 2; k >= p0; k--) {
        const int u = 1 << k;
        const int j = threadIdx.x;
        if (j < (m >> (k + 1))) {
            const int i = u - 1 + 2 * u * j;
            x[i] = cr_back_row<T>(wa, wc, wr, x, i, u);
        }
        __syncthreads();
    }
}

// One system on a thread-block cluster of m = n / s CTAs (2 <= m <= 16), CTA
// j holding slice j: stage 1 of the m slices runs on m SMs at once.  After
// the E_st update each CTA writes its slice's first row (E_st, updated) and
// last row (E_ed) into every CTA's shared memory (distributed shared
// memory, one cluster barrier); warp 0 of every CTA then forms the m
// reduced equations and solves stage 2 itself -- the same arithmetic on the
// same values, so the same bits in every CTA -- and the CTA runs stage 3 on
// its slice.  Per row the operations and their order are those of
// fused_tpr; steps touching at most 32 rows (the reduced system, TPR's top
// tree and back-substitution levels) run on one warp with warp barriers.  gd (may
// be null): the diagonal, dividing a, c, r on load exactly as the 4-argument
// setter does (normalize_kernel) -- so inputs and output may also sit in
// pinned host memory and one launch serves a whole host round trip.  done
// (may be null; a word the host reads): every CTA adds 1 once its part of
// x is visible system-wide, so the host can watch a system complete
// without a driver synchronisation.
template <typename T, int KIND, int EPT>
__global__ void __launch_bounds__(kThreads)
cluster_tpr(const T *__restrict__ ga, const T *__restrict__ gd,
            const T *__restrict__ gc, const T *__restrict__ gr,
            T *__restrict__ gx, int n, int s, long long stride,
            unsigned *done) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    const int m = n / s;
    const int j = (int)cluster.block_rank();
    T *a = sm, *c = sm + s, *r = sm + 2 * s, *x = sm + 3 * s;
    // PTPR's second copy; TPR keeps its loaded even rows there for stage 3
    T *a2 = sm + 4 * s, *c2 = sm + 5 * s, *r2 = sm + 6 * s;
    T *ends = sm + 7 * s;  // [m][6]: E_st (a, c, r) after the update, E_ed (a, c, r)
    T *sa = ends + 6 * m, *sc = sa + m, *sr = sc + m, *sx = sr + m;
    T *bk = sx + m;        // this slice's E_st before the update (PTPR)
    const long long base = (long long)(blockIdx.x / m) * stride + (long long)j * s;
    ga += base;
    gc += base;
    gr += base;
    gx += base;
    if (gd) gd += base;
    auto load = [&](int i) {  // row i of the inputs, diag-normalised
        if (gd) {
            const T dd = gd[i];
            a[i] = ga[i] / dd;
            c[i] = gc[i] / dd;
            r[i] = gr[i] / dd;
        } else {
            a[i] = ga[i];
            c[i] = gc[i];
            r[i] = gr[i];
        }
    };
    for (int i = threadIdx.x; i < s; i += blockDim.x) {
        load(i);
        if (KIND == TPRGB_TPR && (i & 1) == 0) {
            a2[i] = a[i];
            c2[i] = c[i];
            r2[i] = r[i];
        }
    }
    // every CTA of the cluster must have started (its shared memory
    // exists) before any CTA writes into it: arrive now, wait just before
    // the writes, so the barrier's latency overlaps stage 1
    asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
    __syncthreads();
    if (KIND == TPRGB_PTPR) {
        if (ptpr_stage1_slice<T, EPT>(a, c, r, a2, c2, r2, s)) {
            T *t;
            t = a; a = a2; a2 = t;
            t = c; c = c2; c2 = t;
            t = r; r = r2; r2 = t;
        }
    } else {
        tpr_stage1_slice<T, EPT>(a, c, r, s);
    }
    if (threadIdx.x == 0) {
        if (KIND == TPRGB_PTPR) {
            bk[0] = a[0];
            bk[1] = c[0];
            bk[2] = r[0];
        }
        est_update(a, c, r, 0, s - 1);
    }
    __syncthreads();
    asm volatile("barrier.cluster.wait.aligned;" ::: "memory");
    if (threadIdx.x < m) {  // thread q writes this slice's rows into CTA q
        T *dst = cluster.map_shared_rank(ends, (unsigned)threadIdx.x) + 6 * j;
        dst[0] = a[0];
        dst[1] = c[0];
        dst[2] = r[0];
        dst[3] = a[s - 1];
        dst[4] = c[s - 1];
        dst[5] = r[s - 1];
    }
    cluster.sync();  // every slice's rows are in every CTA; no remote access after
    if (threadIdx.x < 32) {  // warp 0: the m <= 16 reduced equations and stage 2
        for (int q = threadIdx.x; q < m; q += 32) {
            const T *e = ends + 6 * q;
            if (q < m - 1)  // E_ed of slice q with E_st of slice q + 1
                inter_eq(e[3], e[4], e[5], e[6], e[7], e[8], sa[q], sc[q], sr[q]);
            else {
                sa[q] = e[3];
                sc[q] = e[4];
                sr[q] = e[5];
            }
        }
        __syncwarp();
        if (KIND == TPRGB_PTPR)
            warp_pcr<T>(sa, sc, sr, m);  // src/ptpr.cpp:246-258
        else
            warp_cr<T>(sa, sc, sr, sx, m);  // src/tpr.cpp:263-275
    }
    __syncthreads();
    // x of the previous slice's last row (0 before the first) and of this
    // slice's last row, from stage 2
    T xprev, xed;
    if (KIND == TPRGB_PTPR) {
        xprev = j > 0 ? sr[j - 1] : T(0);
        xed = sr[j];
        if (threadIdx.x == 0) {  // restore E_st, src/ptpr.cpp:266-271
            a[0] = bk[0];
            c[0] = bk[1];
            r[0] = bk[2];
        }
        __syncthreads();
        // stage 3, src/ptpr.cpp:263-287
        for (int i = threadIdx.x; i < s - 1; i += blockDim.x) {
            T key = T(1) / c[s - 1] * (r[s - 1] - a[s - 1] * xprev - xed);
            if (c[s - 1] == T(0)) key = T(0);
            x[i] = r[i] - a[i] * xprev - c[i] * key;
        }
        if (threadIdx.x == 0) x[s - 1] = xed;
        __syncthreads();
    } else {
        xprev = j > 0 ? sx[j - 1] : T(0);
        xed = sx[j];
        // restore: even slice-local rows as loaded, odd rows keep their
        // post-stage-1 values (src/tpr.cpp:236-325,381-387)
        for (int i = threadIdx.x; i < s; i += blockDim.x)
            if ((i & 1) == 0) {
                a[i] = a2[i];
                c[i] = c2[i];
                r[i] = r2[i];
            }
        if (threadIdx.x == 0) x[s - 1] = xed;
        __syncthreads();
        const int ls = ilog2(s);
        // src/tpr.cpp:277-308; the levels of at most 32 rows on warp 0
        int p = ls - 1;
        while (p >= 0 && (s >> (p + 1)) <= 32) p--;
        if (threadIdx.x < 32) {
            for (int pp = ls - 1; pp > p; pp--) {
                const int u = 1 << pp;
                if (threadIdx.x < (s >> (pp + 1))) {
                    const int i = u - 1 + 2 * u * (int)threadIdx.x;
                    const T xu = i - u < 0 ? xprev : x[i - u];
                    x[i] = r[i] - a[i] * xu - c[i] * x[i + u];
                }
                __syncwarp();
            }
        }
        __syncthreads();
        for (; p >= 0; p--) {
            const int u = 1 << p;
            const int per = s / (2 * u);
            for (int q = threadIdx.x; q < per; q += blockDim.x) {
                const int i = u - 1 + 2 * u * q;
                const T xu = i - u < 0 ? xprev : x[i - u];
                x[i] = r[i] - a[i] * xu - c[i] * x[i + u];
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < s; i += blockDim.x) gx[i] = x[i];
    if (done) {  // count this CTA's slice as written, at system scope
        __threadfence_system();
        __syncthreads();
        if (threadIdx.x == 0) atomicAdd_system(done, 1u);
    }
}

// ---- sliced shape (large systems) ---------------------------------------
// workspace per system: wa, wc, wr [n] (rows after stage 1 and the E_st
// update), then ba, bc, br [m] (E_st backups, PTPR only).
template <typename T, int KIND>
__global__ void __launch_bounds__(kThreads)
sliced_stage1(const T *__restrict__ ga, const T *__restrict__ gc,
              const T *__restrict__ gr, T *__restrict__ work, int n, int s,
              long long stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *a = reinterpret_cast<T *>(smem_raw), *c = a + s, *r = c + s;
    const int m = n / s, j = blockIdx.x;
    const long long base = (long long)blockIdx.y * stride + (long long)j * s;
    T *wbase = work + (long long)blockIdx.y * (3LL * n + 3LL * m);
    for (int i = threadIdx.x; i < s; i += blockDim.x) {
        a[i] = ga[base + i];
        c[i] = gc[base + i];
        r[i] = gr[base + i];
    }
    __syncthreads();
    if (KIND == TPRGB_PTPR)
        ptpr_stage1(a, c, r, s, s);
    else
        tpr_stage1(a, c, r, s, s);
    if (threadIdx.x == 0) {
        if (KIND == TPRGB_PTPR) {
            wbase[3LL * n + j] = a[0];
            wbase[3LL * n + m + j] = c[0];
            wbase[3LL * n + 2 * m + j] = r[0];
        }
        est_update(a, c, r, 0, s - 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < s; i += blockDim.x) {
        wbase[(long long)j * s + i] = a[i];
        wbase[(long long)n + j * s + i] = c[i];
        wbase[2LL * n + j * s + i] = r[i];
    }
}

template <typename T, int KIND>
__global__ void __launch_bounds__(kThreads)
sliced_stage2(const T *__restrict__ work, T *__restrict__ gx, int n, int s,
              long long stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int m = n / s;
    T *sa = reinterpret_cast<T *>(smem_raw), *sc = sa + m, *sr = sc + m,
      *sx = sr + m;
    const T *wa = work + (long long)blockIdx.x * (3LL * n + 3LL * m);
    const T *wc = wa + n, *wr = wa + 2LL * n;
    gx += (long long)blockIdx.x * stride;
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
        long long k = (long long)j * s + s - 1;
        if (j < m - 1)
            inter_eq(wa[k], wc[k], wr[k], wa[k + 1], wc[k + 1], wr[k + 1],
                     sa[j], sc[j], sr[j]);
        else {
            sa[j] = wa[n - 1];
            sc[j] = wc[n - 1];
            sr[j] = wr[n - 1];
        }
    }
    __syncthreads();
    if (KIND == TPRGB_PTPR) {
        cta_pcr(sa, sc, sr, m);
        for (int j = threadIdx.x; j < m; j += blockDim.x)
            gx[(long long)j * s + s - 1] = sr[j];
    } else {
        cta_cr(sa, sc, sr, sx, m);
        for (int j = threadIdx.x; j < m; j += blockDim.x)
            gx[(long long)j * s + s - 1] = sx[j];
    }
}

template <typename T, int KIND>
__global__ void __launch_bounds__(kThreads)
sliced_stage3(const T *__restrict__ ga, const T *__restrict__ gc,
              const T *__restrict__ gr, const T *__restrict__ work,
              T *__restrict__ gx, int n, int s, long long stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int m = n / s, j = blockIdx.x;
    const long long sys = (long long)blockIdx.y * stride;
    const T *wa = work + (long long)blockIdx.y * (3LL * n + 3LL * m);
    const T *wc = wa + n, *wr = wa + 2LL * n;
    const long long st = (long long)j * s, ed = st + s - 1;
    T *x = gx + sys;
    const T xl = (j == 0) ? T(0) : x[st - 1];
    if (KIND == TPRGB_PTPR) {
        const T *ba = wa + 3LL * n;
        const T aed = wa[ed], ced = wc[ed], red = wr[ed], xed = x[ed];
        T key = T(1) / ced * (red - aed * xl - xed);
        if (ced == T(0)) key = T(0);
        for (int i = threadIdx.x; i < s - 1; i += blockDim.x) {
            long long g = st + i;
            T ai = (i == 0) ? ba[j] : wa[g];
            T ci = (i == 0) ? ba[m + j] : wc[g];
            T ri = (i == 0) ? ba[2 * m + j] : wr[g];
            x[g] = ri - ai * xl - ci * key;
        }
    } else {
        T *a = reinterpret_cast<T *>(smem_raw), *c = a + s, *r = c + s;
        T *xs = r + s;  // xs[0] = x[st-1], xs[1..s] = slice
        for (int i = threadIdx.x; i < s; i += blockDim.x) {
            long long g = st + i;
            bool even = (i & 1) == 0;
            a[i] = even ? ga[sys + g] : wa[g];
            c[i] = even ? gc[sys + g] : wc[g];
            r[i] = even ? gr[sys + g] : wr[g];
        }
        if (threadIdx.x == 0) {
            xs[0] = xl;
            xs[s] = x[ed];
        }
        __syncthreads();
        const int ls = ilog2(s);
        for (int p = ls - 1; p >= 0; p--) {
            const int u = 1 << p;
            for (int q = threadIdx.x; q < s / (2 * u); q += blockDim.x) {
                int i = u - 1 + 2 * u * q;
                // x index i (slice-local) lives at xs[i + 1]
                xs[i + 1] = r[i] - a[i] * xs[i + 1 - u] - c[i] * xs[i + 1 + u];
            }
            __syncthreads();
        }
        for (int i = threadIdx.x; i < s - 1; i += blockDim.x)
            x[st + i] = xs[i + 1];
    }
}

template <typename T>
__global__ void normalize_kernel(long long neq, T *a, const T *diag, T *c,
                                 T *r) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long step = (long long)gridDim.x * blockDim.x;
    for (; i < neq; i += step) {
        T d = diag[i];
        a[i] = a[i] / d;
        c[i] = c[i] / d;
        r[i] = r[i] / d;
    }
}

}  // namespace refk

// ---- host side -------------------------------------------------------------

static const size_t kFusedSmemLimit = 200 * 1024;

// Raise a kernel's dynamic shared-memory limit to `smem` unless an earlier
// call on this device already raised it at least that far (the attribute
// is per function and device; setting it is a host call that would
// otherwise cost every launch).  set_to: the limit set so far per device.
// Raising takes a lock, so that two threads asking for different limits
// cannot leave the smaller one set with the larger one recorded.
template <typename K>
static int smem_attr(K k, size_t smem, DeviceOnce &set_to) {
    int dev = 0;
    TPRGB_CUDA(cudaGetDevice(&dev));
    if ((size_t)set_to.get(dev) >= smem) return TPRGB_OK;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if ((size_t)set_to.get(dev) >= smem) return TPRGB_OK;
    TPRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    set_to.set(dev, (int)smem);
    return TPRGB_OK;
}

template <typename T>
static bool ref_uses_fused(int kind, int n, int s) {
    if (kind == TPRGB_CR || kind == TPRGB_PCR)
        return 4LL * n * (long long)sizeof(T) <= (long long)kFusedSmemLimit &&
               n <= refk::kThreads * refk::kEpt;
    return refk::fused_elems(n, s) * (long long)sizeof(T) <=
               (long long)kFusedSmemLimit &&
           n <= refk::kThreads * refk::kEpt;
}

int ref_validate(int kind, int n, int s, int prec) {
    if (kind < TPRGB_PTPR || kind > TPRGB_PCR)
        return fail(TPRGB_EINVAL, "unknown solver kind %d", kind);
    if (prec != TPRGB_F32 && prec != TPRGB_F64)
        return fail(TPRGB_EINVAL, "unknown precision %d", prec);
    if (!is_pow2(n))
        return fail(TPRGB_EINVAL, "n=%d must be a power of two", n);
    const size_t esz = prec == TPRGB_F32 ? 4 : 8;
    if (kind == TPRGB_CR || kind == TPRGB_PCR) return TPRGB_OK;
    if (!is_pow2(s) || s < 2 || s > n)
        return fail(TPRGB_EINVAL,
                    "s=%d must be a power of two with 2 <= s <= n=%d", s, n);
    const int m = n / s;
    bool fused = prec == TPRGB_F32 ? ref_uses_fused<float>(kind, n, s)
                                   : ref_uses_fused<double>(kind, n, s);
    if (!fused) {
        if (s > refk::kThreads * refk::kEpt || (size_t)(3 * s + 2) * esz > kFusedSmemLimit)
            return fail(TPRGB_EUNSUPPORTED, "slice s=%d too large for one CTA", s);
        if (m > refk::kThreads * refk::kEpt || (size_t)4 * m * esz > kFusedSmemLimit)
            return fail(TPRGB_EUNSUPPORTED,
                        "reduced system m=n/s=%d too large for one CTA", m);
    }
    return TPRGB_OK;
}

size_t ref_workspace_elems(int kind, int n, int s) {
    if (kind == TPRGB_PCR) return 6ULL * n;
    if (kind == TPRGB_CR) return 3ULL * n;
    return 3ULL * n + 3ULL * (n / s);
}

bool ref_needs_workspace(int kind, int n, int s, int prec) {
    if (kind == TPRGB_CR || kind == TPRGB_PCR) s = n;
    return prec == TPRGB_F32 ? !ref_uses_fused<float>(kind, n, s)
                             : !ref_uses_fused<double>(kind, n, s);
}

// One system per thread-block cluster of m = n / s CTAs (2 <= m <= 16),
// one slice per CTA, EPT = s / threads rows per thread.
template <typename T, int KIND, int EPT>
static int launch_cluster_tpr(int nsys, int n, int s, const T *a, const T *diag,
                              const T *c, const T *r, T *x, long long stride,
                              unsigned *done, cudaStream_t st) {
    const int m = n / s;
    const size_t smem = (7ULL * s + 10ULL * m + 3) * sizeof(T);
    const int threads = std::min(refk::kThreads, std::max(32, s));
    auto k = refk::cluster_tpr<T, KIND, EPT>;
    static DeviceOnce set_to, nonportable;
    int rc = smem_attr(k, smem, set_to);
    if (rc) return rc;
    int dev = 0;
    TPRGB_CUDA(cudaGetDevice(&dev));
    if (!nonportable.get(dev)) {
        TPRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        nonportable.set(dev, 1);
    }
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)m;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nsys * m), 1, 1);
    cfg.blockDim = dim3((unsigned)threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    TPRGB_CUDA(cudaLaunchKernelEx(&cfg, k, a, diag, c, r, x, n, s, stride, done));
    return TPRGB_OK;
}

template <typename T, int KIND>
static int launch_cluster_ept(int nsys, int n, int s, const T *a, const T *diag, const T *c,
                              const T *r, T *x, long long stride, unsigned *done,
                              cudaStream_t st) {
    switch (std::max(1, s / refk::kThreads)) {
        case 1: return launch_cluster_tpr<T, KIND, 1>(nsys, n, s, a, diag, c, r, x, stride, done, st);
        case 2: return launch_cluster_tpr<T, KIND, 2>(nsys, n, s, a, diag, c, r, x, stride, done, st);
        case 4: return launch_cluster_tpr<T, KIND, 4>(nsys, n, s, a, diag, c, r, x, stride, done, st);
        default: return launch_cluster_tpr<T, KIND, 8>(nsys, n, s, a, diag, c, r, x, stride, done, st);
    }
}

template <typename T, int KIND>
static int launch_tpr_kind(int nsys, int n, int s, const T *a, const T *c,
                           const T *r, T *x, long long stride, T *work,
                           cudaStream_t st) {
    const int m = n / s;
    if (ref_uses_fused<T>(KIND, n, s) && m >= 2 && m <= 16) {
        // one slice per CTA of a thread-block cluster
        return launch_cluster_ept<T, KIND>(nsys, n, s, a, nullptr, c, r, x, stride, nullptr, st);
    }
    if (ref_uses_fused<T>(KIND, n, s)) {
        size_t smem = (size_t)refk::fused_elems(n, s) * sizeof(T);
        int threads = std::min(refk::kThreads, std::max(64, n));
        auto k = refk::fused_tpr<T, KIND>;
        {
            static DeviceOnce set_to;
            int rc = smem_attr(k, smem, set_to);
            if (rc) return rc;
        }
        k<<<nsys, threads, smem, st>>>(a, c, r, x, n, s, stride);
        TPRGB_CUDA(cudaGetLastError());
        return TPRGB_OK;
    }
    if (work == nullptr)
        return fail(TPRGB_EINVAL, "sliced solve (n=%d, s=%d) needs a workspace",
                    n, s);
    {
        size_t smem = 3ULL * s * sizeof(T);
        int threads = std::min(refk::kThreads, std::max(64, s));
        auto k = refk::sliced_stage1<T, KIND>;
        {
            static DeviceOnce set_to;
            int rc = smem_attr(k, smem, set_to);
            if (rc) return rc;
        }
        k<<<dim3(m, nsys), threads, smem, st>>>(a, c, r, work, n, s, stride);
        TPRGB_CUDA(cudaGetLastError());
    }
    {
        size_t smem = 4ULL * m * sizeof(T);
        int threads = std::min(refk::kThreads, std::max(64, m));
        auto k = refk::sliced_stage2<T, KIND>;
        {
            static DeviceOnce set_to;
            int rc = smem_attr(k, smem, set_to);
            if (rc) return rc;
        }
        k<<<nsys, threads, smem, st>>>(work, x, n, s, stride);
        TPRGB_CUDA(cudaGetLastError());
    }
    {
        size_t smem = KIND == TPRGB_TPR ? (4ULL * s + 2) * sizeof(T) : 0;
        int threads = std::min(refk::kThreads, std::max(64, s));
        auto k = refk::sliced_stage3<T, KIND>;
        if (smem) {
            static DeviceOnce set_to;
            int rc = smem_attr(k, smem, set_to);
            if (rc) return rc;
        }
        k<<<dim3(m, nsys), threads, smem, st>>>(a, c, r, work, x, n, s, stride);
        TPRGB_CUDA(cudaGetLastError());
    }
    return TPRGB_OK;
}

// Standalone CR / PCR of more rows than one CTA's shared memory holds: one
// launch per level over the workspace (PCR: two sets of a, c, rhs per
// system, written alternately; CR: one set, reduced in place), CR's levels
// of at most kThreads rows on one CTA per system.
template <typename T>
static int launch_crpcr_stepped(int kind, int nsys, int n, const T *a,
                                const T *c, const T *r, T *x, long long stride,
                                T *work, cudaStream_t st) {
    if (work == nullptr)
        return fail(TPRGB_EINVAL, "standalone %s of n=%d needs a workspace",
                    kind == TPRGB_CR ? "CR" : "PCR", n);
    int ln = 0;
    while ((1 << ln) < n) ln++;
    const long long ws = (long long)ref_workspace_elems(kind, n, n);
    constexpr int kB = 256;
    if (kind == TPRGB_PCR) {
        for (int p = 0; p < ln; p++) {
            const T *set_in = work + ((p - 1) & 1) * 3LL * n;
            T *set_out = work + (p & 1) * 3LL * n;
            const bool first = p == 0, last = p == ln - 1;
            refk::pcr_step<T><<<dim3(n / kB, nsys), kB, 0, st>>>(
                first ? a : set_in, first ? c : set_in + n,
                first ? r : set_in + 2LL * n, first ? stride : ws,
                last ? x : set_out, last ? x : set_out + n,
                last ? x : set_out + 2LL * n, last ? stride : ws, n, 1 << p,
                last ? 1 : 0);
            TPRGB_CUDA(cudaGetLastError());
        }
        return TPRGB_OK;
    }
    T *wa = work, *wc = work + n, *wr = work + 2LL * n;
    int p0 = 1;  // first level of at most kThreads rows
    while ((n >> (p0 + 1)) > refk::kThreads) p0++;
    refk::cr_first<T><<<dim3(n / 2 / kB, nsys), kB, 0, st>>>(a, c, r, stride, wa,
                                                             wc, wr, ws, n);
    TPRGB_CUDA(cudaGetLastError());
    for (int p = 1; p < p0; p++) {
        refk::cr_forward<T><<<dim3((n >> (p + 1)) / kB, nsys), kB, 0, st>>>(
            wa, wc, wr, ws, n, p);
        TPRGB_CUDA(cudaGetLastError());
    }
    refk::cr_tail<T><<<nsys, refk::kThreads, 0, st>>>(wa, wc, wr, ws, x, stride,
                                                       n, p0);
    TPRGB_CUDA(cudaGetLastError());
    for (int k = p0 - 1; k >= 0; k--) {
        refk::cr_backward<T><<<dim3((n >> (k + 1)) / kB, nsys), kB, 0, st>>>(
            wa, wc, wr, ws, x, stride, n, k);
        TPRGB_CUDA(cudaGetLastError());
    }
    return TPRGB_OK;
}

template <typename T>
static int launch_ref_t(int kind, int nsys, int n, int s, const T *a,
                        const T *c, const T *r, T *x, long long stride,
                        T *work, cudaStream_t st) {
    switch (kind) {
        case TPRGB_PTPR:
            return launch_tpr_kind<T, TPRGB_PTPR>(nsys, n, s, a, c, r, x,
                                                  stride, work, st);
        case TPRGB_TPR:
            return launch_tpr_kind<T, TPRGB_TPR>(nsys, n, s, a, c, r, x,
                                                 stride, work, st);
        default: {
            if (!ref_uses_fused<T>(kind, n, n))
                return launch_crpcr_stepped<T>(kind, nsys, n, a, c, r, x,
                                               stride, work, st);
            size_t smem = 4ULL * n * sizeof(T);
            int threads = std::min(refk::kThreads, std::max(64, n));
            auto k = kind == TPRGB_CR ? refk::fused_crpcr<T, TPRGB_CR>
                                      : refk::fused_crpcr<T, TPRGB_PCR>;
            static DeviceOnce set_cr, set_pcr;
            int rc = smem_attr(k, smem, kind == TPRGB_CR ? set_cr : set_pcr);
            if (rc) return rc;
            k<<<nsys, threads, smem, st>>>(a, c, r, x, n, stride);
            TPRGB_CUDA(cudaGetLastError());
            return TPRGB_OK;
        }
    }
}

int launch_ref(int kind, int nsys, int n, int s, int prec, const void *a,
               const void *c, const void *r, void *x, long long stride,
               void *work, cudaStream_t st) {
    if (prec == TPRGB_F32)
        return launch_ref_t<float>(kind, nsys, n, s, (const float *)a,
                                   (const float *)c, (const float *)r,
                                   (float *)x, stride, (float *)work, st);
    return launch_ref_t<double>(kind, nsys, n, s, (const double *)a,
                                (const double *)c, (const double *)r,
                                (double *)x, stride, (double *)work, st);
}

// The one-launch path of a solver handle: one TPR / PTPR system on a
// thread-block cluster (2 <= n / s <= 16 slices of the fused shape), inputs
// (with the diagonal, or diag null) and output at device-accessible
// addresses -- pinned host memory in the handle's case.
bool ref_direct_ok(int kind, int n, int s, int prec) {
    if (kind != TPRGB_PTPR && kind != TPRGB_TPR) return false;
    if (n / s < 2 || n / s > 16) return false;
    return prec == TPRGB_F32 ? ref_uses_fused<float>(kind, n, s)
                             : ref_uses_fused<double>(kind, n, s);
}

int launch_ref_direct(int kind, int n, int s, int prec, const void *a, const void *diag,
                      const void *c, const void *r, void *x, unsigned *done,
                      cudaStream_t st) {
    if (!ref_direct_ok(kind, n, s, prec))
        return fail(TPRGB_EUNSUPPORTED, "no one-launch path for n=%d, s=%d", n, s);
    if (prec == TPRGB_F32) {
        auto f = [&](auto kd) {
            constexpr int K = decltype(kd)::value;
            return launch_cluster_ept<float, K>(1, n, s, (const float *)a, (const float *)diag,
                                                (const float *)c, (const float *)r,
                                                (float *)x, n, done, st);
        };
        return kind == TPRGB_PTPR ? f(std::integral_constant<int, TPRGB_PTPR>())
                                  : f(std::integral_constant<int, TPRGB_TPR>());
    }
    auto f = [&](auto kd) {
        constexpr int K = decltype(kd)::value;
        return launch_cluster_ept<double, K>(1, n, s, (const double *)a, (const double *)diag,
                                             (const double *)c, (const double *)r,
                                             (double *)x, n, done, st);
    };
    return kind == TPRGB_PTPR ? f(std::integral_constant<int, TPRGB_PTPR>())
                              : f(std::integral_constant<int, TPRGB_TPR>());
}

int launch_normalize(int prec, long long neq, void *a, const void *diag,
                     void *c, void *r, cudaStream_t st) {
    int blocks = (int)std::min<long long>((neq + 255) / 256, 152LL * 16);
    if (blocks < 1) blocks = 1;
    if (prec == TPRGB_F32)
        refk::normalize_kernel<float><<<blocks, 256, 0, st>>>(
            neq, (float *)a, (const float *)diag, (float *)c, (float *)r);
    else
        refk::normalize_kernel<double><<<blocks, 256, 0, st>>>(
            neq, (double *)a, (const double *)diag, (double *)c, (double *)r);
    TPRGB_CUDA(cudaGetLastError());
    return TPRGB_OK;
}

}  // namespace tprgb

// ---- reference-semantics solve with a built-in workspace ---------------------
// For callers that cannot allocate device memory themselves: plugins and
// host applications whose device memory belongs to another allocator (a
// framework's caching pool, a simulation code's own arena) that forbids or
// cannot see outside cudaMalloc calls, and latency-critical loops where an
// allocation would synchronise the device.  The sliced path's workspace
// (3n + 3n/s elements per system) lives in this file-scope array instead of
// caller memory.  Every GPU that loads the library holds it until the
// process exits.
#include <cuda.h>  // CUcontext (driver entry points fetched at run time)

#include <mutex>

namespace tprgb {

constexpr size_t kStaticWorkBytes = 16u << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_static_work[kStaticWorkBytes];

// The array's device address belongs to the context the library's module
// is loaded in.  It is looked up (cudaGetSymbolAddress, with the device
// current) once per device and context: a cudaDeviceReset, or a caller that
// makes another driver context current, gives a new context id and hence
// a new lookup, never a stale address.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

static int current_ctx_id(unsigned long long *id) {
    static std::atomic<CtxGetCurrentFn> get_cur{nullptr};
    static std::atomic<CtxGetIdFn> get_id{nullptr};
    CtxGetCurrentFn f1 = get_cur.load(std::memory_order_acquire);
    CtxGetIdFn f2 = get_id.load(std::memory_order_acquire);
    if (!f1 || !f2) {
        void *p1 = nullptr, *p2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p1, 12000,
                                                          cudaEnableDefault, &q1);
        cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &p2, 12000,
                                                          cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !p1 || !p2)
            return fail(TPRGB_EUNSUPPORTED, "cuCtxGetCurrent / cuCtxGetId not available");
        f1 = reinterpret_cast<CtxGetCurrentFn>(p1);
        f2 = reinterpret_cast<CtxGetIdFn>(p2);
        get_cur.store(f1, std::memory_order_release);
        get_id.store(f2, std::memory_order_release);
    }
    CUcontext ctx = nullptr;
    if (f1(&ctx) != CUDA_SUCCESS) return fail(TPRGB_ECUDA, "cuCtxGetCurrent failed");
    *id = 0;  // 0: no context current yet on this thread
    if (ctx && f2(ctx, id) != CUDA_SUCCESS) return fail(TPRGB_ECUDA, "cuCtxGetId failed");
    return TPRGB_OK;
}

struct StaticSlot {
    unsigned long long ctx_id;  // context the address belongs to (0: none)
    void *ptr;
};
static std::mutex g_static_mu;
static StaticSlot g_static_slot[64];

static int static_work_ptr(void **out) {
    int dev = 0;
    TPRGB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(TPRGB_EUNSUPPORTED, "device %d", dev);
    unsigned long long id = 0;
    int rc = current_ctx_id(&id);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_static_mu);
    StaticSlot &sl = g_static_slot[dev];
    if (id == 0 || sl.ctx_id != id || !sl.ptr) {
        // set-up for this device and context: the runtime makes the
        // device's context current first if none is
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_work);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_work)");
        rc = current_ctx_id(&id);
        if (rc) return rc;
        sl.ctx_id = id;
        sl.ptr = p;
    }
    *out = sl.ptr;
    return TPRGB_OK;
}

}  // namespace tprgb

// Same contract and results as tprgb_ref_solve_device, with the workspace
// taken from the library's own 16 MiB device array instead of the caller:
// nothing is allocated (no cudaMalloc, no cudaFree, no allocating library
// call).  The first call on a device (and after a cudaDeviceReset, or under
// another driver context) looks up the array's device address with
// cudaGetSymbolAddress; make that first call before any stream capture.
// Systems whose workspace exceeds 16 MiB in total (nsys * (3n + 3n/s)
// elements for TPR / PTPR, nsys * 3n for CR and 6n for PCR) are rejected with TPRGB_EUNSUPPORTED.  All calls share the
// array and it keeps the last call's contents (no part of it needs to
// start at zero: every workspace element is written before it is read), so
// calls that overlap on the GPU -- on different streams, or from different
// threads -- race; keep them ordered on one stream.
extern "C" TPRGB_API int tprgb_ref_solve_device_static(
    int kind, int nsys, int n, int s, int prec, const void *d_a,
    const void *d_c, const void *d_rhs, void *d_x, void *stream) {
    using namespace tprgb;
    int rc = ref_validate(kind, n, s, prec);
    if (rc) return rc;
    if (nsys < 0 || nsys > 65535)
        return fail(TPRGB_EINVAL, "nsys=%d outside [0, 65535]", nsys);
    if (nsys == 0) return TPRGB_OK;
    if (!d_a || !d_c || !d_rhs || !d_x)
        return fail(TPRGB_EINVAL, "null device pointer");
    void *work = nullptr;
    if (ref_needs_workspace(kind, n, s, prec)) {
        const size_t esz = prec == TPRGB_F32 ? 4 : 8;
        const size_t need = ref_workspace_elems(kind, n, s) * esz * (size_t)nsys;
        if (need > kStaticWorkBytes)
            return fail(TPRGB_EUNSUPPORTED,
                        "workspace of %zu bytes exceeds the built-in %zu bytes "
                        "(use tprgb_ref_solve_device with caller memory)",
                        need, kStaticWorkBytes);
        rc = static_work_ptr(&work);
        if (rc) return rc;
    }
    return launch_ref(kind, nsys, n, s, prec, d_a, d_c, d_rhs, d_x,
                      (long long)n, work, (cudaStream_t)stream);
}
