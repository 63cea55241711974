// Batches staged by swizzled 2D tensor-map loads: batch_sw (one CTA per
// tile of whole systems) and batch_cl (one thread-block cluster per system,
// the parts exchanging their level-3 rows in distributed shared memory).
//
// Each array's tile is one box of a 2D tensor map (rows of 128 bytes, 32
// floats) loaded with the 128-byte swizzle: unit u (16 bytes) of row r
// lands at unit u ^ (r & 7), so the lanes of a warp reading their own
// chunks' units spread over all 32 banks (a contiguous layout puts lanes
// whose chunks are 32 or 64 bytes apart on the same banks).  Persistent
// CTAs walk the batch with a one- or two-stage ring; 8 or 16 equations per
// thread.  Every mbarrier wait is bounded; a timeout is recorded in the
// status word.  A batch_sw CTA then stops after draining its copies; a
// batch_cl CTA keeps taking part in its cluster's row exchanges on
// placeholder rows, storing nothing.
#include <cuda.h>  // CUtensorMap and its enums (the encoder is fetched at run time)

#include <algorithm>

#include "batch.cuh"
#include "cluster.cuh"
#include "tile.cuh"
#include "tma.cuh"

namespace tprgb {

__device__ unsigned g_sw_status[4];  // code, where, tile, unused

namespace bt {

// polls of a load's mbarrier before giving up: 1.0 s on GB300 (a poll with
// its back-off sleep takes about 3.8 us; measured with
// tprgb_selftest_wait_timeout)
constexpr unsigned kWaitLimit = 1u << 18;

// ---- tensor-map (swizzled) staging ----------------------------------------
struct TensorMaps {
    CUtensorMap m[4];  // a, b, c, d as [rows][32 floats]
};

// Registers a thread may use so that the tile's CTAs fit the register file:
// 128 for 16 equations per thread, 80 below.
constexpr int sw_min_blocks(int L, int NT) {
    return (65536 / (NT * (L >= 16 ? 128 : 80))) < 1 ? 1
                                                      : 65536 / (NT * (L >= 16 ? 128 : 80));
}

// Stage-free hook of the one-stage uniform tile: after the tile's last read
// of the stage (every thread calls it there), thread 0 starts loading the
// next tile into the same stage, so the load overlaps the rest of the
// solve and the stores.  Plain values only: a hook that refers to the
// kernel's locals would put them in local memory.
struct NextTileLoad {
    const CUtensorMap *maps;  // a, b, c, d
    float *stage;
    uint64_t *bar;
    unsigned bytes;  // one tile of the four arrays
    int tile_elems;
    int row;         // first 128-byte row of the next tile
    bool use;        // the kernel takes this route (CTA-uniform)
    bool go;         // this thread issues (thread 0, a next tile exists)
    __device__ __forceinline__ void operator()() const {
        if (!use) return;
        __syncthreads();  // every thread is done reading the stage
        if (go) {
            tma::fence_proxy_async();
            tma::mbar_expect_tx(bar, bytes);
#pragma unroll
            for (int k = 0; k < 4; k++)
                tma::tensor_g2s_2d(stage + k * tile_elems, &maps[k], 0, row, bar);
        }
    }
};

// The same for systems at offsets (plans, serving steps): the next tile's
// systems are loaded by the lanes of warp 0, one box of N / 32 rows per
// system and array, as at the top of the tile loop.
template <int TILE, int N>
struct NextTileLoadOffsets {
    const CUtensorMap *maps;  // a, b, c, d
    float *stage;
    uint64_t *bar;
    const long long *sys_off;
    long long s0;  // first system of the next tile
    int gs;        // systems in the next tile
    bool go;       // this thread's warp issues: a next tile exists
    __device__ __forceinline__ void operator()() const {
        __syncthreads();  // every thread is done reading the stage
        if (!go) return;
        const int lane = threadIdx.x & 31;
        tma::fence_proxy_async();
        if (lane == 0) tma::mbar_expect_tx(bar, 4u * (unsigned)gs * N * 4u);
        __syncwarp();
        for (int g = lane; g < gs; g += 32) {
            const int r = (int)(sys_off[s0 + g] >> 5);
#pragma unroll
            for (int k = 0; k < 4; k++)
                tma::tensor_g2s_2d(stage + k * TILE + g * N, &maps[k], 0, r, bar);
        }
    }
};

// Systems at offsets: sys_off (element offsets, multiples of 32, n >= 256)
// gives system k's first equation; the tensor maps' box is then one system
// (n / 32 rows) and each tile is G box loads per array, issued by the
// lanes of warp 0.  sys_off == nullptr: system k at k * n, one box per tile.
// sys_status (may be null): word k |= 1 when system k's solution is not
// finite.  status: timeout record (code, site, detail), g_sw_status if null.
template <int L, int NT, int T, int MODE, bool OFFS_HOOK>
__global__ void __launch_bounds__(NT, sw_min_blocks(L, NT))
batch_sw(const __grid_constant__ TensorMaps tm, void *__restrict__ gx, int nsys,
         int refine_steps, int x_f64, int S, const long long *__restrict__ sys_off,
         unsigned *__restrict__ sys_status, unsigned *__restrict__ status) {
    constexpr int TILE = NT * L;     // equations per tile
    constexpr int ROWS = TILE / 32;  // 128-byte rows per array and tile
    constexpr int G = NT / T;
    constexpr int n = T * L;
    static_assert(ROWS % 8 == 0 && ROWS <= 256, "tile rows");
    extern __shared__ unsigned char dyn_sw[];
    // stage base on a 1024-byte boundary: the swizzle pattern spans 8 rows
    const unsigned pad = (1024u - (tma::smem_addr(dyn_sw) & 1023u)) & 1023u;
    float *stages = reinterpret_cast<float *>(dyn_sw + pad);  // [S][4][TILE]
    __shared__ __align__(8) uint64_t full[2];
    __shared__ tile::Smem<NT> sm;
    __shared__ int s_ok;
    const int tid = threadIdx.x;
    const long long ntiles = ((long long)nsys + G - 1) / G;
    unsigned *stw = status ? status : g_sw_status;

    if (tid == 0) {
        tma::mbar_init(&full[0], 1);
        tma::mbar_init(&full[1], 1);
        tma::fence_barrier_init();
    }
    __syncthreads();

    auto issue = [&](long long tl, int st) {  // the lanes of warp 0
        const int lane = tid & 31;
        tma::fence_proxy_async();
        if (!sys_off) {
            if (lane == 0) {
                // the whole box counts, rows past the end are zero-filled
                tma::mbar_expect_tx(&full[st], 4u * TILE * 4u);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    tma::tensor_g2s_2d(stages + (st * 4 + k) * TILE, &tm.m[k], 0,
                                       (int)(tl * ROWS), &full[st]);
            }
            return;
        }
        const long long s0 = tl * G;
        const int gs = (int)min((long long)G, (long long)nsys - s0);
        if (lane == 0) tma::mbar_expect_tx(&full[st], 4u * (unsigned)gs * n * 4u);
        __syncwarp();
        for (int g = lane; g < gs; g += 32) {
            const int row = (int)(sys_off[s0 + g] >> 5);
#pragma unroll
            for (int k = 0; k < 4; k++)
                tma::tensor_g2s_2d(stages + (st * 4 + k) * TILE + g * n, &tm.m[k], 0,
                                   row, &full[st]);
        }
    };

    const long long first = blockIdx.x, stride = gridDim.x;
    if (tid < 32) {
        if (first < ntiles) issue(first, 0);
        if (S == 2 && first + stride < ntiles) issue(first + stride, 1);
    }
    unsigned off[L / 4];
    tile::swizzled_offsets<L>(tid, off);
    const int g = tid / T, t = tid & (T - 1);
    int it = 0;
    for (long long tl = first; tl < ntiles; tl += stride, it++) {
        const int st = S == 2 ? (it & 1) : 0;
        const unsigned phase = (unsigned)(S == 2 ? (it >> 1) : it) & 1u;
        if (tid == 0) {
            s_ok = tma::mbar_wait(&full[st], phase, kWaitLimit) ? 1 : 0;
            if (!s_ok) {
                atomicCAS(&stw[0], 0u, (unsigned)TPRGB_ETIMEOUT);
                stw[1] = 2;
                stw[2] = (unsigned)tl;
            }
        }
        __syncthreads();
        if (!s_ok) {
            // Leave no copy in flight into this CTA's shared memory: thread 0
            // waits (bounded again) for the late copy into the stage that
            // timed out, then for the other stage's copy if one was issued.
            // The other threads may leave; the CTA stays resident until
            // thread 0 returns.
            if (tid == 0) {
                tma::mbar_wait(&full[st], phase, kWaitLimit);
                if (S == 2 && tl + stride < ntiles)
                    tma::mbar_wait(&full[st ^ 1], (unsigned)((it + 1) >> 1) & 1u,
                                   kWaitLimit);
            }
            return;
        }
        const long long sys = tl * G + g;
        const bool active = sys < nsys;
        tile::Part pc;
        pc.on = 0;
        pc.P = 1;
        pc.p = 0;
        pc.round = 0;
        const float *s0 = stages + st * 4 * TILE;
        const long long sbase = active ? (sys_off ? sys_off[sys] : sys * n) : 0;
        // one stage: the next tile loads as soon as this one's last read of
        // the stage is done (OFFS_HOOK: the instance for systems at offsets,
        // launched with S = 1 only; otherwise systems back to back)
        const bool early = OFFS_HOOK || (S == 1 && !sys_off);
        bool finite;
        if constexpr (OFFS_HOOK) {
            const long long nx = tl + stride;
            const NextTileLoadOffsets<TILE, n> hook{
                tm.m, stages, &full[0], sys_off, nx * G,
                (int)min((long long)G, (long long)nsys - nx * G), tid < 32 && nx < ntiles};
            finite = tile::run_tile_smem<L, NT, T, MODE, true>(
                s0, s0 + TILE, s0 + 2 * TILE, s0 + 3 * TILE, off, gx,
                active ? sbase + (long long)t * L : 0, active, t, t == 0,
                t == T - 1, refine_steps, x_f64, sm, pc, hook);
        } else {
            const NextTileLoad hook{tm.m, stages, &full[0], 4u * TILE * 4u, TILE,
                                    (int)((tl + stride) * ROWS), early,
                                    early && tid == 0 && tl + stride < ntiles};
            finite = tile::run_tile_smem<L, NT, T, MODE, true>(
                s0, s0 + TILE, s0 + 2 * TILE, s0 + 3 * TILE, off, gx,
                active ? sbase + (long long)t * L : 0, active, t, t == 0,
                t == T - 1, refine_steps, x_f64, sm, pc, hook);
        }
        if (sys_status && active && !finite) atomicOr(&sys_status[sys], 1u);
        if (!early) {
            __syncthreads();  // every thread is done reading this stage
            if (tid < 32 && tl + (long long)S * stride < ntiles)
                issue(tl + (long long)S * stride, st);
        }
    }
}

// ---- systems spanning a thread-block cluster --------------------------------
// One cluster of P CTAs per system of n = P * NT * L equations; CTA rank p
// stages rows [p * ROWS, (p + 1) * ROWS) of the system's 128-byte rows with
// a swizzled tensor-map load and solves its part; in each solve every warp
// sends its segment's two boundary rows into every part's shared memory
// (st.async onto a row mbarrier per parity) and warp 0 of each part solves
// the system's reduced rows (tile::cluster_levels23); above 64 warp
// segments per system each part first reduces its own rows to two and
// only those are exchanged (tile::cluster_levels2_3).  Clusters
// walk the batch with a stride of the number of clusters; every CTA of a
// cluster runs the same number of systems and solves, so their row
// exchanges pair up.  A load that times out is recorded in the status
// word, its CTA stores nothing for that system, and the CTA keeps taking
// part in the exchanges.  sys_off / sys_status / status as for batch_sw
// (offsets multiples of 32).
template <int L, int NT, int MODE, int P>
__global__ void __launch_bounds__(NT, sw_min_blocks(L, NT))
batch_cl(const __grid_constant__ TensorMaps tm, void *__restrict__ gx, int nsys,
         int refine_steps, int x_f64, const long long *__restrict__ sys_off,
         unsigned *__restrict__ sys_status, unsigned *__restrict__ status) {
    constexpr int TILE = NT * L;
    constexpr int ROWS = TILE / 32;
    static_assert(ROWS % 8 == 0 && ROWS <= 256, "tile rows");
    extern __shared__ unsigned char dyn_sw[];
    const unsigned pad = (1024u - (tma::smem_addr(dyn_sw) & 1023u)) & 1023u;
    float *stage = reinterpret_cast<float *>(dyn_sw + pad);  // [4][TILE]
    __shared__ __align__(8) uint64_t full;
    __shared__ tile::Smem<NT> sm;
    __shared__ float4 crows[tile::cluster_row_slots<NT, P>()];
    __shared__ __align__(8) uint64_t rbar[2];  // row barriers, one per parity
    __shared__ int s_ok;
    const int tid = threadIdx.x;
    const unsigned p = cl::rank();  // the cluster has P CTAs
    const long long nclusters = gridDim.x / P, c0 = blockIdx.x / P;
    const long long rows_per_sys = (long long)P * ROWS;
    unsigned *stw = status ? status : g_sw_status;
    auto sys_base = [&](long long sys) {  // first equation of a system
        return sys_off ? sys_off[sys] : sys * rows_per_sys * 32;
    };

    if (tid == 0) {
        tma::mbar_init(&full, 1);
        tma::mbar_init(&rbar[0], 1);
        tma::mbar_init(&rbar[1], 1);
        tma::fence_barrier_init();
    }
    __syncthreads();
    cl::sync();  // every CTA's row barriers exist before any part stores rows
    auto issue = [&](long long sys) {  // thread 0 only
        tma::fence_proxy_async();
        tma::mbar_expect_tx(&full, 4u * TILE * 4u);
#pragma unroll
        for (int k = 0; k < 4; k++)
            tma::tensor_g2s_2d(stage + k * TILE, &tm.m[k], 0,
                               (int)((sys_base(sys) >> 5) + (long long)p * ROWS), &full);
    };
    if (tid == 0 && c0 < nsys) issue(c0);
    unsigned off[L / 4];
    tile::swizzled_offsets<L>(tid, off);
    unsigned round = 0;
    // After a load times out, the CTA issues no more loads and solves its
    // remaining parts on placeholder rows (storing nothing), so that its
    // row exchanges still pair with the other CTAs'; before leaving it
    // waits, bounded, for the late copy.
    bool pending = false;
    unsigned pend_phase = 0;
    int it = 0;
    for (long long sys = c0; sys < nsys; sys += nclusters, it++) {
        bool ok = false;
        if (!pending) {
            if (tid == 0) {
                s_ok = tma::mbar_wait(&full, (unsigned)it & 1u, kWaitLimit) ? 1 : 0;
                if (!s_ok) {
                    atomicCAS(&stw[0], 0u, (unsigned)TPRGB_ETIMEOUT);
                    stw[1] = 3;
                    stw[2] = (unsigned)sys;
                }
            }
            __syncthreads();
            ok = s_ok != 0;
            if (!ok) {
                pending = true;
                pend_phase = (unsigned)it & 1u;
            }
        }
        tile::Part pc;
        pc.on = 2;
        pc.crows = crows;
        pc.rbar = rbar;
        pc.cstatus = stw;
        pc.P = P;
        pc.p = (int)p;
        pc.round = round;
        pc.nsolve = 0;
        const long long base = sys_base(sys) + (long long)p * TILE + tid * L;
        // the next system's part starts loading as soon as this one's last
        // read of the stage is done, overlapping the rest of the solve
        auto early = [&]() {
            __syncthreads();  // every thread is done reading the stage
            if (tid == 0 && !pending && sys + nclusters < nsys) issue(sys + nclusters);
        };
        const bool finite = tile::run_tile_smem<L, NT, NT, MODE, true, decltype(early), P>(
            stage, stage + TILE, stage + 2 * TILE, stage + 3 * TILE, off, gx,
            ok ? base : 0, ok, tid, p == 0 && tid == 0,
            p == P - 1 && tid == NT - 1, refine_steps, x_f64, sm, pc, early);
        if (sys_status && ok && !finite) atomicOr(&sys_status[sys], 1u);
        round = pc.round;
    }
    // no CTA leaves while a part of its cluster may still store rows into
    // its shared memory (possible only after a row wait timed out: every
    // part otherwise waits for all rows sent to it)
    cl::sync();
    if (pending && tid == 0) tma::mbar_wait(&full, pend_phase, kWaitLimit);
}

}  // namespace bt

// ---- swizzled variant: host side -------------------------------------------
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t,
                                 void *, const cuuint64_t *, const cuuint64_t *,
                                 const cuuint32_t *, const cuuint32_t *,
                                 CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int tensor_encoder(EncodeTiled *out) {
    static std::atomic<EncodeTiled> fn{nullptr};
    EncodeTiled f = fn.load(std::memory_order_acquire);
    if (!f) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p,
                                                         12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
            return fail(TPRGB_EUNSUPPORTED, "cuTensorMapEncodeTiled is not available");
        f = reinterpret_cast<EncodeTiled>(p);
        fn.store(f, std::memory_order_release);
    }
    *out = f;
    return TPRGB_OK;
}

// The four tensor maps of a launch (a, b, c, d as rows of 32 floats, boxes
// of `rows` rows, 128-byte swizzle).  A map is a plain descriptor of the
// address, extents and box, so repeated launches on the same buffers reuse
// the last encodings: each host thread keeps its own few, looked up by
// (device, pointers, extent, box); the encode calls then leave the
// back-to-back launch path.
static int tile_maps(const BatchArgs &A, int dev, unsigned rows, bt::TensorMaps *out) {
    struct Entry {
        const float *p[4];
        unsigned long long total;
        unsigned rows;
        int dev;
        bool used;
        bt::TensorMaps tm;
    };
    static thread_local Entry cache[4];
    static thread_local unsigned next = 0;
    const unsigned long long total =
        A.total_eq ? (unsigned long long)A.total_eq
                   : (unsigned long long)A.nsys * (unsigned long long)A.n;
    const float *src[4] = {A.a, A.b, A.c, A.d};
    for (Entry &e : cache) {
        if (e.used && e.dev == dev && e.total == total && e.rows == rows &&
            e.p[0] == src[0] && e.p[1] == src[1] && e.p[2] == src[2] && e.p[3] == src[3]) {
            *out = e.tm;
            return TPRGB_OK;
        }
    }
    EncodeTiled enc = nullptr;
    int rc = tensor_encoder(&enc);
    if (rc) return rc;
    bt::TensorMaps tm;
    const cuuint64_t dims[2] = {32, (cuuint64_t)(total / 32)};
    const cuuint64_t strides[1] = {128};
    const cuuint32_t box[2] = {32, (cuuint32_t)rows};
    const cuuint32_t es[2] = {1, 1};
    for (int i = 0; i < 4; i++) {
        CUresult r = enc(&tm.m[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                         const_cast<float *>(src[i]), dims, strides, box, es,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return fail(TPRGB_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    }
    Entry &e = cache[next++ & 3u];
    for (int i = 0; i < 4; i++) e.p[i] = src[i];
    e.total = total;
    e.rows = rows;
    e.dev = dev;
    e.tm = tm;
    e.used = true;
    *out = tm;
    return TPRGB_OK;
}

template <int L, int NT, int T, int MODE, bool OFFS_HOOK>
static int launch_sw_k(const BatchArgs &A, int S, cudaStream_t st) {
    constexpr int G = NT / T;
    constexpr int ROWS = NT * L / 32;
    const size_t smem = (size_t)S * 4 * NT * L * sizeof(float) + 1024;
    auto k = bt::batch_sw<L, NT, T, MODE, OFFS_HOOK>;
    static DeviceOnce grid_cap[3];  // by stage count
    int dev = 0;
    TPRGB_CUDA(cudaGetDevice(&dev));
    int cap = grid_cap[S].get(dev);
    if (!cap) {
        const size_t smax = 2ull * 4 * NT * L * sizeof(float) + 1024;
        TPRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smax));
        int sms = 0, per = 0;
        TPRGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        TPRGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, NT, smem));
        cap = std::max(1, sms * std::max(per, 1));
        grid_cap[S].set(dev, cap);
    }
    bt::TensorMaps tm;
    int rc = tile_maps(A, dev, (unsigned)(A.sys_off ? A.n / 32 : ROWS), &tm);
    if (rc) return rc;
    const long long ntiles = (A.nsys + G - 1) / G;
    const int grid = (int)std::min<long long>(ntiles, cap);
    k<<<grid, NT, smem, st>>>(tm, A.x, A.nsys, A.refine_steps, A.x_f64, S, A.sys_off,
                              A.sys_status, A.status);
    TPRGB_CUDA(cudaGetLastError());
    return TPRGB_OK;
}

// Systems at offsets with one stage get the instance that loads the next
// tile early where plans and serving steps use it: 16 equations per
// thread, one system per CTA (n = 1024, 2048, 4096 on 64, 128, 256
// threads), refined.  Other shapes load after the tile (with several
// systems per CTA the early-load instance spilled 4-24 bytes).
template <int L, int NT, int T, int MODE>
static int launch_sw_t(const BatchArgs &A, int S, cudaStream_t st) {
    if constexpr (L == 16 && T == NT && MODE == 1) {
        if (A.sys_off && S == 1) return launch_sw_k<L, NT, T, MODE, true>(A, S, st);
    }
    return launch_sw_k<L, NT, T, MODE, false>(A, S, st);
}

template <int L, int NT, int T>
static int launch_sw_mode(const BatchArgs &A, int S, cudaStream_t st) {
    if (A.refine_steps <= 0) return launch_sw_t<L, NT, T, 0>(A, S, st);
    return launch_sw_t<L, NT, T, 1>(A, S, st);
}

template <int L, int NT>
static int launch_sw_T(const BatchArgs &A, int S, cudaStream_t st) {
    switch (A.n / L) {
        case 2: return launch_sw_mode<L, NT, 2>(A, S, st);
        case 4: return launch_sw_mode<L, NT, 4>(A, S, st);
        case 8: return launch_sw_mode<L, NT, 8>(A, S, st);
        case 16: return launch_sw_mode<L, NT, 16>(A, S, st);
        case 32: return launch_sw_mode<L, NT, 32>(A, S, st);
        case 64: return launch_sw_mode<L, NT, 64>(A, S, st);
        case 128: return launch_sw_mode<L, NT, (NT >= 128 ? 128 : NT)>(A, S, st);
        case 256: return launch_sw_mode<L, NT, (NT >= 256 ? 256 : NT)>(A, S, st);
        default: return fail(TPRGB_EINVAL, "unsupported threads per system");
    }
}

// Swizzled staged batch: L in {8, 16}, nt in {64, 128, 256}, n >= 32,
// compensated residual; S = 2 (two-stage ring) or 1 (one stage, more
// resident CTAs).
int launch_batch_sw(const BatchArgs &A, const TileConfig &cfg, cudaStream_t st) {
    int rc = batch_config_check(A.n, cfg);
    if (rc) return rc;
    if (A.residual == TPRGB_RESID_F64 && A.refine_steps > 0)
        return fail(TPRGB_EUNSUPPORTED, "staged kernel has no FP64 residual mode");
    if (cfg.nt != 64 && cfg.nt != 128 && cfg.nt != 256)
        return fail(TPRGB_EINVAL, "swizzled tiles use 64, 128 or 256 threads");
    if (A.n < 32)
        return fail(TPRGB_EUNSUPPORTED, "swizzled tiles need n >= 32");
    if (A.nsys == 0) return TPRGB_OK;
    const int S = cfg.staged == 2 ? 2 : 1;
    if (cfg.L == 16) {
        if (cfg.nt == 64) return launch_sw_T<16, 64>(A, S, st);
        return cfg.nt == 128 ? launch_sw_T<16, 128>(A, S, st)
                             : launch_sw_T<16, 256>(A, S, st);
    }
    if (cfg.L != 8) return fail(TPRGB_EINVAL, "swizzled tiles use 8 or 16 equations per thread");
    if (cfg.nt == 64) return launch_sw_T<8, 64>(A, S, st);
    return cfg.nt == 128 ? launch_sw_T<8, 128>(A, S, st) : launch_sw_T<8, 256>(A, S, st);
}

// ---- cluster variant: host side ---------------------------------------------
template <int L, int NT, int MODE, int P>
static int launch_cl_t(const BatchArgs &A, cudaStream_t st) {
    constexpr int TILE = NT * L;
    constexpr int ROWS = TILE / 32;
    const size_t smem = 4ull * TILE * sizeof(float) + 1024;
    auto k = bt::batch_cl<L, NT, MODE, P>;
    static DeviceOnce attrs, max_clusters;
    int dev = 0;
    TPRGB_CUDA(cudaGetDevice(&dev));
    if (!attrs.get(dev)) {
        TPRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
        TPRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        // load-balancing placement packs one more 16-CTA cluster onto the
        // GPCs than the default (15 against 14 resident at n = 65536; 152
        // against 148 four-CTA clusters of 128 threads)
        TPRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeClusterSchedulingPolicyPreference,
                                        cudaClusterSchedulingPolicyLoadBalancing));
        attrs.set(dev, 1);
    }
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)P;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)P, 1, 1);
    cfg.blockDim = dim3(NT, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int ncl_max = max_clusters.get(dev);
    if (!ncl_max) {
        TPRGB_CUDA(cudaOccupancyMaxActiveClusters(&ncl_max, k, &cfg));
        if (ncl_max < 1)
            return fail(TPRGB_EUNSUPPORTED, "a cluster of %d CTAs of %d threads does not fit",
                        P, NT);
        max_clusters.set(dev, ncl_max);
    }
    bt::TensorMaps tm;
    int rc = tile_maps(A, dev, (unsigned)ROWS, &tm);
    if (rc) return rc;
    const int ncl = (int)std::min<long long>(A.nsys, ncl_max);
    cfg.gridDim = dim3((unsigned)(ncl * P), 1, 1);
    TPRGB_CUDA(cudaLaunchKernelEx(&cfg, k, tm, A.x, A.nsys, A.refine_steps, A.x_f64,
                                  A.sys_off, A.sys_status, A.status));
    return TPRGB_OK;
}

template <int NT, int P>
static int launch_cl_mode(const BatchArgs &A, cudaStream_t st) {
    if (A.refine_steps <= 0) return launch_cl_t<16, NT, 0, P>(A, st);
    if (A.residual == TPRGB_RESID_F64) return launch_cl_t<16, NT, 2, P>(A, st);
    return launch_cl_t<16, NT, 1, P>(A, st);
}

template <int NT>
static int launch_cl_p(const BatchArgs &A, int P, cudaStream_t st) {
    switch (P) {
        case 2: return launch_cl_mode<NT, 2>(A, st);
        case 4: return launch_cl_mode<NT, 4>(A, st);
        case 8: return launch_cl_mode<NT, 8>(A, st);
        case 16: return launch_cl_mode<NT, 16>(A, st);
        default: return fail(TPRGB_EINVAL, "cluster of %d CTAs", P);
    }
}

// Cluster batch: 16 equations per thread, nt in {64, 128, 256, 512} threads per
// CTA, P = n / (16 nt) CTAs per system with P in {2, 4, 8, 16}; plain FP32,
// compensated FP32 residual or native FP64 residual.
int launch_batch_cl(const BatchArgs &A, const TileConfig &cfg, cudaStream_t st) {
    int P = 0;
    int rc = cluster_parts(A.n, cfg, &P);
    if (rc) return rc;
    if (A.nsys == 0) return TPRGB_OK;
    if (cfg.nt == 64) return launch_cl_p<64>(A, P, st);
    if (cfg.nt == 512) return launch_cl_p<512>(A, P, st);
    return cfg.nt == 128 ? launch_cl_p<128>(A, P, st) : launch_cl_p<256>(A, P, st);
}

int cluster_parts(int n, const TileConfig &cfg, int *P) {
    if (cfg.L != 16 || (cfg.nt != 64 && cfg.nt != 128 && cfg.nt != 256 && cfg.nt != 512))
        return fail(TPRGB_EINVAL, "cluster tiles use 16 equations per thread and 64, "
                                  "128, 256 or 512 threads");
    if (!is_pow2(n) || n < 2 * 16 * cfg.nt || n > 16 * 16 * cfg.nt)
        return fail(TPRGB_EINVAL, "n=%d needs 2..16 CTAs of %d equations", n, 16 * cfg.nt);
    *P = n / (16 * cfg.nt);
    return TPRGB_OK;
}

int sw_status(unsigned (&v)[4], bool reset) {
    TPRGB_CUDA(cudaMemcpyFromSymbol(v, g_sw_status, sizeof(v)));
    if (reset) {
        unsigned z[4] = {0, 0, 0, 0};
        TPRGB_CUDA(cudaMemcpyToSymbol(g_sw_status, z, sizeof(z)));
    }
    return TPRGB_OK;
}

}  // namespace tprgb
