// Tile solver shared by the batched kernels and the persistent queue
// kernel: a CTA of NT threads solves either several whole systems (T = n / L
// threads each) or one part of a system that spans several CTAs.  The parts
// exchange their boundary rows through global scratch at counter barriers
// (queue kernel), or every warp sends its segment rows through distributed
// shared memory with st.async onto each part's row mbarriers (thread-block
// clusters).
#pragma once

#include "cluster.cuh"
#include "common.cuh"
#include "hier.cuh"
#include "tma.cuh"

namespace tprgb {
namespace tile {

using hier::Chunk;
using hier::Row;

// polls of a multi-CTA barrier in global memory before giving up: about
// 1.1 s on GB300 with the back-off of part_barrier (2^23 polls measured
// 4.3 s with tprgb_selftest_wait_timeout)
constexpr unsigned kSpinLimit = 1u << 21;

struct SegRows {
    Row R0, R1;
};

// Shared memory of one tile.
template <int NT>
struct Smem {
    SegRows rows[NT / 32];
    float2 x[NT / 32];
    float4 edge[2 * (NT / 32)];
    float2 part_nb;  // previous part's last / next part's first unknown
    int ok;
};

// Cluster parts' rows as every CTA of a cluster holds them:
// [parity][segment][row F / E], (a, c, d, 0) per row, where segment g =
// part * W + warp is the g-th 32-lane warp segment of the system (W warps
// per part) -- or, for systems of more than 64 segments (two-stage
// exchange), [parity][part][row F / E] of the parts' level-2 rows.
template <int NT, int P>
constexpr int cluster_row_slots() {
    return (NT / 32) * P <= 64 ? 2 * (NT / 32) * P * 2 : 2 * P * 2;
}

// Multi-CTA system context.  on = 1: the parts are CTAs of a persistent
// grid meeting at counter barriers in global scratch (per system: counter,
// then rows [2 parity][32 parts][8 floats] and edges [2 parity][32 parts][4
// floats]); on = 2: the parts are the CTAs of one thread-block cluster,
// exchanging segment rows through distributed shared memory (crows: this
// CTA's row buffer of cluster_row_slots entries; rbar: its two row
// barriers, one per parity; cstatus: timeout record (code, site, detail)).
struct Part {
    int on, P, p;
    float4 *crows;
    uint64_t *rbar;
    unsigned *cstatus;
    unsigned *counter;
    float *rows, *edges;
    unsigned round;
    DeviceStatus *status;
    int item;
    // neighbouring parts' edge unknowns as (hi, lo) pairs, taken from the
    // level-3 solution every part computes: nb_hm/nb_lm = previous part's
    // last, nb_hp/nb_lp = next part's first.  Solve 0 sets hi, corrections
    // accumulate into lo.
    int nsolve;
    float nb_hm, nb_lm, nb_hp, nb_lp;
};

constexpr int kScratchFloats = 4 + 2 * 32 * 8 + 2 * 32 * 4;  // per system
// polls of a cluster row barrier before giving up: 1.0 s on GB300
constexpr unsigned kRowWaitLimit = 1u << 18;

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Barrier between the CTAs holding the parts of one system.  Bounded: on
// timeout it records TPRGB_ETIMEOUT and returns false (results of that
// system are then invalid, the kernel still finishes).
// Threads that wrote scratch for this round fence their writes themselves
// (writer_fence) before the barrier; the others need no fence.
__device__ __forceinline__ void writer_fence() { __threadfence(); }

template <int NT>
__device__ bool part_barrier(Part &pc, Smem<NT> &sm, int where) {
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(pc.counter, 1u);
        const unsigned target = (pc.round + 1u) * (unsigned)pc.P;
        unsigned it = 0, ns = 32;
        int ok = 1;
        while (ld_acquire(pc.counter) < target) {
            if (++it > kSpinLimit) {
                ok = 0;
                atomicCAS(&pc.status->code, 0u, (unsigned)TPRGB_ETIMEOUT);
                pc.status->where = (unsigned)where;
                pc.status->detail = (unsigned)pc.item;
                break;
            }
            __nanosleep(ns);
            if (ns < 256) ns <<= 1;
        }
        __threadfence();
        sm.ok = ok;
    }
    __syncthreads();
    pc.round++;
    return sm.ok != 0;
}

// Levels 2 and 3 of a system spread over the P CTAs of a thread-block
// cluster, as one reduction.  After level 1 every warp of every part holds
// its segment's two boundary rows (F on lane 0, E on lane 31); in the
// order F_0, E_0, F_1, E_1, ... of all W * P segments of the system these
// rows form a tridiagonal system with unit diagonal (2 W P rows).  Each
// warp sends its two rows straight into every part's row buffer with
// st.async, completing 32 bytes on that part's row mbarrier of the round's
// parity, so no CTA barrier and no separate level-2 pass come before the
// exchange.  Warp 0 of each part waits (bounded) for all W P segments,
// then solves the whole reduced system redundantly: J = W P / 32 segments
// per lane (2J rows, the thread-level partition elimination of level 0 on
// unit-diagonal rows), a warp-wide reduction over K lanes, the top block,
// and back.  It writes the first / last unknowns of its own W segments and
// the neighbouring parts' edge unknowns to shared memory; the caller's CTA
// barrier hands them to the other warps.
//
// Slot reuse: the rows of a parity are overwritten two rounds later.  A
// warp sends round r + 2 only after its part's round r + 1 exchange, which
// needs every part's round r + 1 rows, which each part's warps send only
// after their CTA barrier of round r -- after warp 0 there has read the
// round r rows.  The same ordering puts every round r + 2 byte after the
// round r phase of the barrier completed.
template <int NT, int P, int NTS>
__device__ __forceinline__ void cluster_levels23(const Row &R0, const Row &R1,
                                                 Smem<NTS> &sm, Part &pc) {
    constexpr int W = NT / 32;       // warp segments per part
    constexpr int S = W * P;         // segments of the system
    constexpr int K = S < 32 ? S : 32;  // lanes of the reduction
    constexpr int J = S / K;         // segments per lane
    static_assert(S % K == 0 && J >= 1, "segments per lane");
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const unsigned par = pc.round & 1u;
    // every warp: its two rows to slot (p W + warp) of every part's buffer
    {
        const float a0 = __shfl_sync(0xffffffffu, R0.a, 0);
        const float c0 = __shfl_sync(0xffffffffu, R0.c, 0);
        const float d0 = __shfl_sync(0xffffffffu, R0.d, 0);
        const float a1 = __shfl_sync(0xffffffffu, R1.a, 31);
        const float c1 = __shfl_sync(0xffffffffu, R1.c, 31);
        const float d1 = __shfl_sync(0xffffffffu, R1.d, 31);
        if (warp == 0 && lane == 0) tma::mbar_expect_tx(pc.rbar + par, 32u * S);
        if (lane < P) {
            const int slot = (int)par * S + pc.p * W + warp;
            const uint32_t dst = cl::map(pc.crows + slot * 2, (unsigned)lane);
            const uint32_t bar = cl::map(pc.rbar + par, (unsigned)lane);
            cl::st_async4(dst, make_float4(a0, c0, d0, 0.f), bar);
            cl::st_async4(dst + 16u, make_float4(a1, c1, d1, 0.f), bar);
        }
    }
    if (warp == 0) {
        const bool in = cl::mbar_wait(pc.rbar + par, (pc.round >> 1) & 1u, kRowWaitLimit);
        if (!in && lane == 0) {
            atomicCAS(&pc.cstatus[0], 0u, (unsigned)TPRGB_ETIMEOUT);
            pc.cstatus[1] = 4;
            pc.cstatus[2] = pc.round;
        }
        // lane q: segments q J .. q J + J - 1 as 2J unit-diagonal rows
        const int q = lane & (K - 1);
        float ra[2 * J], rb[2 * J], rc[2 * J], rd[2 * J];
        const float4 *src = pc.crows + ((int)par * S + q * J) * 2;
#pragma unroll
        for (int i = 0; i < 2 * J; i++) {
            const float4 v = src[i];
            ra[i] = v.x;
            rb[i] = 1.0f;
            rc[i] = v.y;
            rd[i] = v.z;
        }
        Row U0, U1;
        Chunk<2 * J> ck;
        if constexpr (J > 1) {
            hier::level0<2 * J>(ra, rb, rc, rd, ck);
            U0 = ck.F;
            U1 = ck.E;
        } else {
            U0 = Row{ra[0], rc[0], rd[0]};
            U1 = Row{ra[2 * J - 1], rc[2 * J - 1], rd[2 * J - 1]};
        }
        hier::seg_reduce_k<K>(U0, U1, q);
        float zf, zl, z0, z1;
        hier::seg_top_k<K>(U0, U1, zf, zl);
        hier::seg_back(U0, U1, q, K, zf, zl, z0, z1);
        float xs[2 * J];
        if constexpr (J > 1) {
            hier::level0_back<2 * J>(ck, z0, z1, xs);
        } else {
            xs[0] = z0;
            xs[2 * J - 1] = z1;
        }
        // this part's segments and the neighbouring parts' edge unknowns
        const int g0 = pc.p * W;
        if (lane < K) {
#pragma unroll
            for (int j = 0; j < J; j++) {
                const int g = q * J + j;
                if (g >= g0 && g < g0 + W) sm.x[g - g0] = make_float2(xs[2 * j], xs[2 * j + 1]);
                if (g == g0 - 1) sm.part_nb.x = xs[2 * j + 1];
                if (g == g0 + W) sm.part_nb.y = xs[2 * j];
            }
        }
        if (lane == 0 && pc.p == 0) sm.part_nb.x = 0.f;
        if (lane == 0 && pc.p == P - 1) sm.part_nb.y = 0.f;
    }
    pc.round++;
}

// Levels 2 and 3 of a cluster part in two stages, for systems of more than
// 64 warp segments (where the one-pass reduction's per-lane rows and 128
// senders per round cost more than a local level 2): the W segment rows
// of the part meet in shared memory (CTA barrier), warp 0 reduces them to
// the part's two boundary rows (level 2), sends them into every part's row
// buffer with st.async (completing 32 bytes on that part's row mbarrier of
// the round's parity), waits (bounded) for all P parts' rows, solves the
// 2P-row system (level 3), and back-substitutes level 2 into shared memory
// for the caller's CTA barrier.  Slot reuse as for cluster_levels23: a part
// sends round r + 2 only after receiving every part's round r + 1 rows,
// each sent after that part read its round r rows.
template <int NT, int P, int NTS>
__device__ __forceinline__ void cluster_levels2_3(const Row &R0, const Row &R1,
                                                  Smem<NTS> &sm, Part &pc) {
    constexpr int W = NT / 32;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    if (lane == 0) sm.rows[warp].R0 = R0;
    if (lane == 31) sm.rows[warp].R1 = R1;
    __syncthreads();
    if (warp == 0) {
        Row S0{0.f, 0.f, 0.f}, S1{0.f, 0.f, 0.f};
        const int q2 = lane & (W - 1);
        if (lane < W) {
            S0 = sm.rows[lane].R0;
            S1 = sm.rows[lane].R1;
        }
        hier::seg_reduce_k<W>(S0, S1, q2);
        const unsigned par = pc.round & 1u;
        const float a0 = __shfl_sync(0xffffffffu, S0.a, 0);
        const float c0 = __shfl_sync(0xffffffffu, S0.c, 0);
        const float d0 = __shfl_sync(0xffffffffu, S0.d, 0);
        const float a1 = __shfl_sync(0xffffffffu, S1.a, W - 1);
        const float c1 = __shfl_sync(0xffffffffu, S1.c, W - 1);
        const float d1 = __shfl_sync(0xffffffffu, S1.d, W - 1);
        if (lane == 0) tma::mbar_expect_tx(pc.rbar + par, 32u * P);
        if (lane < P) {
            const uint32_t dst = cl::map(pc.crows + ((int)par * P + pc.p) * 2, (unsigned)lane);
            const uint32_t bar = cl::map(pc.rbar + par, (unsigned)lane);
            cl::st_async4(dst, make_float4(a0, c0, d0, 0.f), bar);
            cl::st_async4(dst + 16u, make_float4(a1, c1, d1, 0.f), bar);
        }
        const bool in = cl::mbar_wait(pc.rbar + par, (pc.round >> 1) & 1u, kRowWaitLimit);
        if (!in && lane == 0) {
            atomicCAS(&pc.cstatus[0], 0u, (unsigned)TPRGB_ETIMEOUT);
            pc.cstatus[1] = 4;
            pc.cstatus[2] = pc.round;
        }
        Row U0{0.f, 0.f, 0.f}, U1{0.f, 0.f, 0.f};
        if (lane < P) {
            const float4 *src = pc.crows + ((int)par * P + lane) * 2;
            const float4 v0 = src[0], v1 = src[1];
            U0 = Row{v0.x, v0.y, v0.z};
            U1 = Row{v1.x, v1.y, v1.z};
        }
        const int q3 = lane & (P - 1);
        hier::seg_reduce_k<P>(U0, U1, q3);
        float zf, zl, z0, z1;
        hier::seg_top_k<P>(U0, U1, zf, zl);
        hier::seg_back(U0, U1, q3, P, zf, zl, z0, z1);
        const float yf = __shfl_sync(0xffffffffu, z0, pc.p);
        const float yl = __shfl_sync(0xffffffffu, z1, pc.p);
        // the neighbouring parts' edge unknowns for the next residual
        const float pl = __shfl_sync(0xffffffffu, z1, pc.p > 0 ? pc.p - 1 : 0);
        const float nf = __shfl_sync(0xffffffffu, z0, pc.p < P - 1 ? pc.p + 1 : 0);
        if (lane == 0)
            sm.part_nb = make_float2(pc.p > 0 ? pl : 0.f, pc.p < P - 1 ? nf : 0.f);
        float y0, y1;
        hier::seg_back(S0, S1, q2, W, yf, yl, y0, y1);
        if (lane < W) sm.x[lane] = make_float2(y0, y1);
    }
    pc.round++;
}

// Which cluster exchange a (threads per CTA, parts) shape uses: the
// one-pass reduction up to 64 warp segments per system, two stages above.
template <int NT, int P>
constexpr bool cluster_one_pass() {
    return (NT / 32) * P <= 64;
}

// Hierarchical solve.  T: threads of this system inside the CTA (T <= NT;
// T == NT for a part of a multi-CTA system), a compile-time power of two so
// that segment widths and lane arithmetic fold to constants.  All threads
// of the CTA call this (it has CTA barriers when T > 32).
template <int L, int NT, int T, int PP = 0>
__device__ __forceinline__ void solve(const float (&a)[L], const float (&b)[L],
                                      const float (&c)[L], const float (&d)[L],
                                      float (&x)[L], Smem<NT> &sm, Part &pc) {
    constexpr int K = T < 32 ? T : 32;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int q = lane & (K - 1);
    Chunk<L> ck;
    hier::level0<L>(a, b, c, d, ck);
    Row R0 = ck.F, R1 = ck.E;
    hier::seg_reduce_k<K>(R0, R1, q);
    float xf, xl;
    if (T <= 32) {
        hier::seg_top_k<K>(R0, R1, xf, xl);
    } else if constexpr (PP > 0) {
        // a part of a system on a thread-block cluster of PP CTAs
        // (T == NT): levels 2 and 3 as one reduction
        if constexpr (cluster_one_pass<NT, PP>())
            cluster_levels23<NT, PP>(R0, R1, sm, pc);
        else
            cluster_levels2_3<NT, PP>(R0, R1, sm, pc);
        __syncthreads();
        const float2 v = sm.x[tid >> 5];
        xf = v.x;
        xl = v.y;
        const float2 nb = sm.part_nb;
        if (pc.nsolve == 0) {
            pc.nb_hm = nb.x;
            pc.nb_lm = 0.f;
            pc.nb_hp = nb.y;
            pc.nb_lp = 0.f;
        } else {
            pc.nb_lm += nb.x;
            pc.nb_lp += nb.y;
        }
        pc.nsolve++;
    } else {
        constexpr int W = T > 32 ? T / 32 : 1;
        const int warp = tid >> 5;
        const int sys_warp0 = warp & ~(W - 1);
        const int w = warp - sys_warp0;
        if (q == 0) sm.rows[warp].R0 = R0;
        if (q == 31) sm.rows[warp].R1 = R1;
        __syncthreads();
        Row S0{0.f, 0.f, 0.f}, S1{0.f, 0.f, 0.f};
        const int q2 = lane & (W - 1);
        if (!pc.on && W <= 4) {
            // every lane solves the system's 2W segment rows (unit
            // diagonal, in the order F_0, E_0, F_1, ...; outer couplings
            // zero) itself by one elimination sweep and back-substitution
            // from shared memory: no shuffles, no idle warps, no second
            // barrier (the rows buffer is rewritten only after a later one)
            constexpr int R = 2 * W;
            float ra[R], rc[R], rd[R];
#pragma unroll
            for (int g = 0; g < W; g++) {
                const SegRows sr = sm.rows[sys_warp0 + g];
                ra[2 * g] = sr.R0.a;
                rc[2 * g] = sr.R0.c;
                rd[2 * g] = sr.R0.d;
                ra[2 * g + 1] = sr.R1.a;
                rc[2 * g + 1] = sr.R1.c;
                rd[2 * g + 1] = sr.R1.d;
            }
#pragma unroll
            for (int k = 1; k < R; k++) {
                const float inv = hier::rcp(fmaf(-ra[k], rc[k - 1], 1.0f));
                rc[k] *= inv;
                rd[k] = fmaf(-ra[k], rd[k - 1], rd[k]) * inv;
            }
            float y[R];
            y[R - 1] = rd[R - 1];
#pragma unroll
            for (int k = R - 2; k >= 0; k--) y[k] = fmaf(-rc[k], y[k + 1], rd[k]);
            xf = y[0];
            xl = y[1];
#pragma unroll
            for (int g = 1; g < W; g++) {
                if (w == g) {
                    xf = y[2 * g];
                    xl = y[2 * g + 1];
                }
            }
        } else if (!pc.on) {
            // every warp of the system solves the 2W segment rows itself:
            // no idle warps and no second barrier (the rows buffer is
            // rewritten only after a later barrier)
            if (lane < W) {
                S0 = sm.rows[sys_warp0 + lane].R0;
                S1 = sm.rows[sys_warp0 + lane].R1;
            }
            hier::seg_reduce_k<W>(S0, S1, q2);
            float yf, yl, y0, y1;
            hier::seg_top_k<W>(S0, S1, yf, yl);
            hier::seg_back(S0, S1, q2, W, yf, yl, y0, y1);
            // the rows sit in lanes 0..W-1 only: read lane w of the whole
            // warp (a width-W shuffle would read other, empty segments)
            xf = __shfl_sync(0xffffffffu, y0, w);
            xl = __shfl_sync(0xffffffffu, y1, w);
        } else {
            float yf = 0.f, yl = 0.f;
            if (w == 0) {
                if (lane < W) {
                    S0 = sm.rows[sys_warp0 + lane].R0;
                    S1 = sm.rows[sys_warp0 + lane].R1;
                }
                hier::seg_reduce_k<W>(S0, S1, q2);
            }
            // level 3 (persistent queue kernel): this CTA's two boundary
            // rows -> global scratch, counter barrier, every part solves the
            // 2P-row system redundantly
            const unsigned par = pc.round & 1u;
            if (warp == 0 && lane == 0) {
                float4 *dst = reinterpret_cast<float4 *>(pc.rows + (par * 32 + pc.p) * 8);
                __stcg(dst, make_float4(S0.a, S0.c, S0.d, 0.f));
                writer_fence();
            }
            if (warp == 0 && lane == W - 1) {
                float4 *dst = reinterpret_cast<float4 *>(pc.rows + (par * 32 + pc.p) * 8 + 4);
                __stcg(dst, make_float4(S1.a, S1.c, S1.d, 0.f));
                writer_fence();
            }
            part_barrier<NT>(pc, sm, 1);
            if (warp == 0) {
                const int P = pc.P;
                Row U0{0.f, 0.f, 0.f}, U1{0.f, 0.f, 0.f};
                if (lane < P) {
                    const float4 *src =
                        reinterpret_cast<const float4 *>(pc.rows + (par * 32 + lane) * 8);
                    const float4 v0 = __ldcg(src), v1 = __ldcg(src + 1);
                    U0 = Row{v0.x, v0.y, v0.z};
                    U1 = Row{v1.x, v1.y, v1.z};
                }
                const int q3 = lane & (P - 1);
                hier::seg_reduce(U0, U1, q3, P);
                float zf, zl, z0, z1;
                hier::seg_top(U0, U1, q3, P, zf, zl);
                hier::seg_back(U0, U1, q3, P, zf, zl, z0, z1);
                yf = __shfl_sync(0xffffffffu, z0, pc.p);
                yl = __shfl_sync(0xffffffffu, z1, pc.p);
                // neighbours' edge unknowns for the next residual: no
                // separate exchange needed
                const float pl = __shfl_sync(0xffffffffu, z1, pc.p > 0 ? pc.p - 1 : 0);
                const float nf = __shfl_sync(0xffffffffu, z0, pc.p < P - 1 ? pc.p + 1 : 0);
                if (lane == 0)
                    sm.part_nb = make_float2(pc.p > 0 ? pl : 0.f,
                                             pc.p < P - 1 ? nf : 0.f);
                float y0, y1;
                hier::seg_back(S0, S1, q2, W, yf, yl, y0, y1);
                if (lane < W) sm.x[sys_warp0 + lane] = make_float2(y0, y1);
            }
            __syncthreads();
            float2 v = sm.x[warp];
            xf = v.x;
            xl = v.y;
            const float2 nb = sm.part_nb;
            if (pc.nsolve == 0) {
                pc.nb_hm = nb.x;
                pc.nb_lm = 0.f;
                pc.nb_hp = nb.y;
                pc.nb_lp = 0.f;
            } else {
                pc.nb_lm += nb.x;
                pc.nb_lp += nb.y;
            }
            pc.nsolve++;
        }
    }
    float x0, x1;
    hier::seg_back(R0, R1, q, K, xf, xl, x0, x1);
    hier::level0_back<L>(ck, x0, x1, x);
}

// x[-1] and x[L] of this thread's chunk (hi, lo pairs), zero outside the
// system.  t: thread index within the system's threads of this CTA.
template <int NT, int T>
__device__ __forceinline__ void neighbours(float hfirst, float hlast,
                                           float lfirst, float llast, int t,
                                           float &hm, float &lm, float &hp,
                                           float &lp, Smem<NT> &sm, Part &pc) {
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    constexpr int K = T < 32 ? T : 32;
    hm = __shfl_up_sync(0xffffffffu, hlast, 1, K);
    lm = __shfl_up_sync(0xffffffffu, llast, 1, K);
    hp = __shfl_down_sync(0xffffffffu, hfirst, 1, K);
    lp = __shfl_down_sync(0xffffffffu, lfirst, 1, K);
    if (T > 32) {
        const int warp = tid >> 5;
        if (lane == 0) sm.edge[2 * warp] = make_float4(hfirst, lfirst, 0.f, 0.f);
        if (lane == 31) sm.edge[2 * warp + 1] = make_float4(hlast, llast, 0.f, 0.f);
        __syncthreads();
        if (lane == 0 && t > 0) {
            float4 v = sm.edge[2 * (warp - 1) + 1];
            hm = v.x;
            lm = v.y;
        }
        if (lane == 31 && t < T - 1) {
            float4 v = sm.edge[2 * (warp + 1)];
            hp = v.x;
            lp = v.y;
        }
        // no second barrier: sm.edge is rewritten only in the next
        // refinement step, after the correction solve's barriers
    }
    if (pc.on) {
        // neighbouring parts' edge values from the level-3 solutions
        if (t == 0) {
            hm = pc.nb_hm;
            lm = pc.nb_lm;
        }
        if (t == T - 1) {
            hp = pc.nb_hp;
            lp = pc.nb_lp;
        }
    } else {
        if (t == 0) {
            hm = 0.f;
            lm = 0.f;
        }
        if (t == T - 1) {
            hp = 0.f;
            lp = 0.f;
        }
    }
}

// Residuals of a chunk's rows for x = xh + xlo (hm/lm, hp/lp: the
// neighbouring unknowns outside the chunk).  lo_terms = false in the first
// refinement step, where xlo is zero: one uniform branch per chunk picks
// the form without the lo products.
template <int L>
__device__ __forceinline__ void residuals(const float (&a)[L], const float (&b)[L],
                                          const float (&c)[L], const float (&d)[L],
                                          const float (&xh)[L], const float (&xlo)[L],
                                          float hm, float lm, float hp, float lp,
                                          bool lo_terms, float (&r)[L]) {
    if (lo_terms) {
#pragma unroll
        for (int i = 0; i < L; i++)
            r[i] = hier::residual_df<true>(a[i], b[i], c[i], d[i],
                                           i > 0 ? xh[i - 1] : hm,
                                           i > 0 ? xlo[i - 1] : lm, xh[i], xlo[i],
                                           i < L - 1 ? xh[i + 1] : hp,
                                           i < L - 1 ? xlo[i + 1] : lp);
    } else {
#pragma unroll
        for (int i = 0; i < L; i++)
            r[i] = hier::residual_df<false>(a[i], b[i], c[i], d[i],
                                            i > 0 ? xh[i - 1] : hm, 0.f, xh[i], 0.f,
                                            i < L - 1 ? xh[i + 1] : hp, 0.f);
    }
}

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

// Whole tile: load, solve, refine, store.  MODE: 0 plain FP32, 1 refine
// with compensated residual, 2 refine with native FP64 residual.
// first_eq / last_eq: this thread's chunk holds the system's first / last
// equation.  Returns true if every x of this thread is finite.
template <int L, int NT, int T, int MODE>
__device__ __forceinline__ bool run_tile(
    const float *__restrict__ ga, const float *__restrict__ gb,
    const float *__restrict__ gc, const float *__restrict__ gd,
    void *__restrict__ gx, long long base, bool active, int t, bool first_eq,
    bool last_eq, int refine_steps, int x_f64, Smem<NT> &sm, Part &pc) {
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
    if (first_eq) a[0] = 0.f;     // a[0] of a system takes no part
    if (last_eq) c[L - 1] = 0.f;  // nor does c[n-1]

    float xh[L];
    solve<L, NT, T>(a, b, c, d, xh, sm, pc);

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
            float hm, lm, hp, lp;
            if (MODE == 1) {
                neighbours<NT, T>(xh[0], xh[L - 1], xlo[0], xlo[L - 1], t, hm,
                                  lm, hp, lp, sm, pc);
                residuals<L>(a, b, c, d, xh, xlo, hm, lm, hp, lp, step > 0, r);
            } else {
                float fh = (float)xd[0], fl = (float)(xd[0] - (double)fh);
                float lh = (float)xd[L - 1], ll = (float)(xd[L - 1] - (double)lh);
                neighbours<NT, T>(fh, lh, fl, ll, t, hm, lm, hp, lp, sm, pc);
                const double xm = (double)hm + (double)lm;
                const double xp = (double)hp + (double)lp;
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
            solve<L, NT, T>(a, b, c, r, dx, sm, pc);
#pragma unroll
            for (int i = 0; i < L; i++) {
                if (MODE == 1)
                    xlo[i] += dx[i];
                else
                    xd[i] += (double)dx[i];
            }
        }
    }

    bool finite = true;
    if (!active) return true;
    if (x_f64 && MODE != 2) {
        finite = hier::store_pairs_f64<L>(xh, xlo, (double *)gx + base);
    } else if (x_f64) {
        double2 *o = reinterpret_cast<double2 *>((double *)gx + base);
#pragma unroll
        for (int i = 0; i < L / 2; i++) {
            finite = finite && isfinite(xh[2 * i]) && isfinite(xh[2 * i + 1]);
            o[i] = make_double2(xd[2 * i], xd[2 * i + 1]);
        }
    } else {
        float4 *o = reinterpret_cast<float4 *>((float *)gx + base);
#pragma unroll
        for (int i = 0; i < L / 4; i++) {
            float v[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                v[j] = MODE == 2 ? (float)xd[4 * i + j]
                                 : xh[4 * i + j] + xlo[4 * i + j];
                finite = finite && isfinite(v[j]);
            }
            o[i] = make_float4(v[0], v[1], v[2], v[3]);
        }
    }
    return finite;
}


// ---- tile runner with the raw system staged in shared memory ---------------
// A thread's chunk of one array is L/4 16-byte units at the byte offsets
// off[0..L/4) from the array's base: consecutive for a plain staged tile,
// permuted by the 128-byte swizzle of a tensor-map load (unit u of 128-byte
// row r sits at unit u ^ (r & 7)), which spreads the lanes of a warp over
// all 32 banks.
template <int L>
__device__ __forceinline__ void lds_chunk(const float *p, float (&v)[L]) {
    const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
    for (int i = 0; i < L / 4; i++) {
        float4 t = q[i];
        v[4 * i + 0] = t.x;
        v[4 * i + 1] = t.y;
        v[4 * i + 2] = t.z;
        v[4 * i + 3] = t.w;
    }
}

// Swizzled form: unit i of the chunk at byte offset off[i] from `base`.
template <int L>
__device__ __forceinline__ void lds_chunk_sw(const float *base,
                                             const unsigned (&off)[L / 4],
                                             float (&v)[L]) {
    const char *p = reinterpret_cast<const char *>(base);
#pragma unroll
    for (int i = 0; i < L / 4; i++) {
        float4 t = *reinterpret_cast<const float4 *>(p + off[i]);
        v[4 * i + 0] = t.x;
        v[4 * i + 1] = t.y;
        v[4 * i + 2] = t.z;
        v[4 * i + 3] = t.w;
    }
}

// Byte offsets of the 16-byte units of tile-thread `tid`'s chunk (L
// equations per thread) in an array region written by a tensor-map load
// with the 128-byte swizzle.
template <int L>
__device__ __forceinline__ void swizzled_offsets(int tid, unsigned (&off)[L / 4]) {
    const unsigned b0 = (unsigned)tid * L * 4u;
    const unsigned r7 = (b0 >> 7) & 7u;
#pragma unroll
    for (int j = 0; j < L / 4; j++) off[j] = b0 ^ ((((unsigned)j) ^ r7) << 4);
}

// Unit u (equations 4u .. 4u + 3) of this thread's chunk of one staged
// array: at byte offset off[u] from the region's base (swizzled), or the
// u-th float4 of the thread's contiguous chunk.
template <int L, bool SW>
__device__ __forceinline__ float4 unit_at(const float *base, const unsigned (&off)[L / 4],
                                          int u) {
    if (SW) return *reinterpret_cast<const float4 *>(reinterpret_cast<const char *>(base) + off[u]);
    return reinterpret_cast<const float4 *>(base)[u];
}

// No-op stage-free hook (run_tile_smem's default).
struct NoHook {
    __device__ __forceinline__ void operator()() const {}
};

// Same computation as run_tile, but a, b, c, d are re-read from shared
// memory each time they are needed instead of being held in registers
// through the refinement.  MODE: 0 plain FP32, 1 refinement with the
// compensated FP32 residual, 2 refinement with the native FP64 residual
// (x accumulated in FP64).  SW = false: sa..sd point at this thread's
// contiguous chunk; SW = true: sa..sd are the array regions' bases and off
// holds the chunk's swizzled unit offsets.  stage_free() is called by every
// thread right after the tile's last read of the staged arrays (before the
// last solve's reduction), so a one-stage kernel can start loading its next
// tile there; the hook synchronises the CTA itself.
template <int L, int NT, int T, int MODE, bool SW = false, typename Hook = NoHook,
          int PP = 0>
__device__ __forceinline__ bool run_tile_smem(
    const float *sa, const float *sb, const float *sc, const float *sd,
    const unsigned (&off)[L / 4], void *__restrict__ gx, long long base,
    bool active, int t, bool first_eq, bool last_eq, int refine_steps,
    int x_f64, Smem<NT> &sm, Part &pc, Hook stage_free = Hook()) {
    auto load4 = [&](float (&a)[L], float (&b)[L], float (&c)[L],
                     float (&d)[L]) {
        if (active) {
            if (SW) {
                lds_chunk_sw<L>(sa, off, a);
                lds_chunk_sw<L>(sb, off, b);
                lds_chunk_sw<L>(sc, off, c);
                lds_chunk_sw<L>(sd, off, d);
            } else {
                lds_chunk<L>(sa, a);
                lds_chunk<L>(sb, b);
                lds_chunk<L>(sc, c);
                lds_chunk<L>(sd, d);
            }
        } else {
#pragma unroll
            for (int i = 0; i < L; i++) {
                a[i] = 0.f;
                b[i] = 1.f;
                c[i] = 0.f;
                d[i] = 0.f;
            }
        }
        if (first_eq) a[0] = 0.f;
        if (last_eq) c[L - 1] = 0.f;
    };
    const bool refine = MODE != 0 && refine_steps > 0;
    float xh[L];
    {
        float a[L], b[L], c[L], d[L];
        load4(a, b, c, d);
        if (!refine) stage_free();
        solve<L, NT, T, PP>(a, b, c, d, xh, sm, pc);
    }
    if constexpr (MODE == 2) {
        // native FP64 residual: x accumulated in FP64, the residual
        // r = d - A x formed by three DFMAs on the exactly converted
        // coefficients and rounded once to FP32 for the correction solve
        double xd[L];
#pragma unroll
        for (int i = 0; i < L; i++) xd[i] = (double)xh[i];
        for (int step = 0; step < refine_steps; step++) {
            // the chunk's edge values as (hi, lo) FP32 pairs for the
            // neighbour exchange
            const float fh = (float)xd[0], fl = (float)(xd[0] - (double)fh);
            const float lh = (float)xd[L - 1], ll = (float)(xd[L - 1] - (double)lh);
            float hm, lm, hp, lp;
            neighbours<NT, T>(fh, lh, fl, ll, t, hm, lm, hp, lp, sm, pc);
            const double xm = (double)hm + (double)lm;
            const double xp = (double)hp + (double)lp;
            float r[L];
            // four equations at a time (one 16-byte unit of each array), so
            // that only one unit of the coefficients is live beside x
#pragma unroll
            for (int u = 0; u < L / 4; u++) {
                float4 ua = make_float4(0.f, 0.f, 0.f, 0.f), ub = make_float4(1.f, 1.f, 1.f, 1.f);
                float4 uc = ua, ud = ua;
                if (active) {
                    ua = unit_at<L, SW>(sa, off, u);
                    ub = unit_at<L, SW>(sb, off, u);
                    uc = unit_at<L, SW>(sc, off, u);
                    ud = unit_at<L, SW>(sd, off, u);
                }
                const float ea[4] = {ua.x, ua.y, ua.z, ua.w}, eb[4] = {ub.x, ub.y, ub.z, ub.w};
                const float ec[4] = {uc.x, uc.y, uc.z, uc.w}, ed[4] = {ud.x, ud.y, ud.z, ud.w};
                // the coefficients as doubles: bit-built on the integer
                // pipes, or converted on the FP64 pipe for a unit holding a
                // value that is not a normal float or zero
                bool odd = false;
#pragma unroll
                for (int j = 0; j < 4; j++)
                    odd = odd || hier::f32_odd(ea[j]) || hier::f32_odd(eb[j]) ||
                          hier::f32_odd(ec[j]) || hier::f32_odd(ed[j]);
                auto cv = [odd](float f) {
                    return odd ? (double)f : hier::f32_to_f64_bits(f);
                };
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int i = 4 * u + j;
                    const float ai = (i == 0 && first_eq) ? 0.f : ea[j];
                    const float ci = (i == L - 1 && last_eq) ? 0.f : ec[j];
                    double rr = fma(-cv(eb[j]), xd[i], cv(ed[j]));
                    rr = fma(-cv(ai), i > 0 ? xd[i - 1] : xm, rr);
                    rr = fma(-cv(ci), i < L - 1 ? xd[i + 1] : xp, rr);
                    r[i] = (float)rr;
                }
            }
            float dx[L];
            {
                float a[L], b[L], c[L], d[L];
                load4(a, b, c, d);
                if (step == refine_steps - 1) stage_free();
                solve<L, NT, T, PP>(a, b, c, r, dx, sm, pc);
            }
            bool odd = false;
#pragma unroll
            for (int i = 0; i < L; i++) odd = odd || hier::f32_odd(dx[i]);
            if (odd) {
#pragma unroll
                for (int i = 0; i < L; i++) xd[i] += (double)dx[i];
            } else {
#pragma unroll
                for (int i = 0; i < L; i++) xd[i] += hier::f32_to_f64_bits(dx[i]);
            }
        }
        if (!active) return true;
        bool finite = true;
#pragma unroll
        for (int i = 0; i < L; i++) finite = finite && isfinite(xd[i]);
        if (x_f64) {
            double2 *o = reinterpret_cast<double2 *>((double *)gx + base);
#pragma unroll
            for (int i = 0; i < L / 2; i++) o[i] = make_double2(xd[2 * i], xd[2 * i + 1]);
        } else {
            float4 *o = reinterpret_cast<float4 *>((float *)gx + base);
#pragma unroll
            for (int i = 0; i < L / 4; i++)
                o[i] = make_float4((float)xd[4 * i], (float)xd[4 * i + 1],
                                   (float)xd[4 * i + 2], (float)xd[4 * i + 3]);
        }
        return finite;
    } else {
        float xlo[L];
#pragma unroll
        for (int i = 0; i < L; i++) xlo[i] = 0.f;
        if (MODE == 1) {
            for (int step = 0; step < refine_steps; step++) {
                float hm, lm, hp, lp;
                neighbours<NT, T>(xh[0], xh[L - 1], xlo[0], xlo[L - 1], t, hm, lm,
                                  hp, lp, sm, pc);
                float r[L];
                {
                    float a[L], b[L], c[L], d[L];
                    load4(a, b, c, d);
                    residuals<L>(a, b, c, d, xh, xlo, hm, lm, hp, lp, step > 0, r);
                }
                float dx[L];
                {
                    float a[L], b[L], c[L], d[L];
                    load4(a, b, c, d);
                    if (step == refine_steps - 1) stage_free();
                    solve<L, NT, T, PP>(a, b, c, r, dx, sm, pc);
                }
#pragma unroll
                for (int i = 0; i < L; i++) xlo[i] += dx[i];
            }
        }
        bool finite = true;
        if (!active) return true;
        if (x_f64) {
            finite = hier::store_pairs_f64<L>(xh, xlo, (double *)gx + base);
        } else {
            float4 *o = reinterpret_cast<float4 *>((float *)gx + base);
#pragma unroll
            for (int i = 0; i < L / 4; i++) {
                float v[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    v[j] = xh[4 * i + j] + xlo[4 * i + j];
                    finite = finite && isfinite(v[j]);
                }
                o[i] = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
        return finite;
    }
}

}  // namespace tile
}  // namespace tprgb
