// Uniform batches with the inputs staged by TMA bulk copies.
//
// Persistent CTAs walk the batch in tiles of NT*L equations (G = NT/T whole
// systems, contiguous in memory).  A two-stage shared-memory ring is fed by
// cp.async.bulk copies (four per tile: a, b, c, d) that complete on one
// mbarrier per stage; while a CTA solves the tile in one stage, the next
// tile streams into the other, so HBM reads overlap the elimination even
// at 2-3 CTAs per SM.  The refinement re-reads a, b, c, d from shared
// memory instead of holding them in registers.  Every mbarrier wait is
// bounded; a timeout is recorded in the batch status word and the CTA
// stops after draining its in-flight copies.
#include <algorithm>

#include "batch.cuh"
#include "tile.cuh"
#include "tma.cuh"

namespace tprgb {

__device__ unsigned g_batch_status[4];  // code, where, tile, unused

namespace bt {

// polls of a load's mbarrier before giving up: 1.0 s on GB300 (a poll with
// its back-off sleep takes about 3.8 us; measured with
// tprgb_selftest_wait_timeout)
constexpr unsigned kWaitLimit = 1u << 18;

template <int L, int NT, int T, int MODE>
__global__ void __launch_bounds__(NT, (NT <= 128 ? 6 : (NT <= 256 ? 3 : 1)))
batch_tma(const float *__restrict__ ga, const float *__restrict__ gb,
          const float *__restrict__ gc, const float *__restrict__ gd,
          void *__restrict__ gx, int nsys, int refine_steps, int x_f64) {
    constexpr int TILE = NT * L;  // equations per tile
    constexpr int G = NT / T;     // systems per tile
    constexpr int n = T * L;
    extern __shared__ __align__(128) unsigned char dyn[];
    float *stages = reinterpret_cast<float *>(dyn);  // [2][4][TILE]
    __shared__ __align__(8) uint64_t full[2];
    __shared__ tile::Smem<NT> sm;
    __shared__ int s_ok;
    const int tid = threadIdx.x;
    const long long ntiles = ((long long)nsys + G - 1) / G;
    const float *src[4] = {ga, gb, gc, gd};

    if (tid == 0) {
        tma::mbar_init(&full[0], 1);
        tma::mbar_init(&full[1], 1);
        tma::fence_barrier_init();
    }
    __syncthreads();

    auto issue = [&](long long tl, int st) {  // thread 0 only
        const long long s0 = tl * G;
        const int gs = (int)min((long long)G, (long long)nsys - s0);
        const unsigned bytes = (unsigned)gs * n * 4u;
        tma::fence_proxy_async();
        tma::mbar_expect_tx(&full[st], 4u * bytes);
#pragma unroll
        for (int k = 0; k < 4; k++)
            tma::bulk_g2s(stages + (st * 4 + k) * TILE, src[k] + s0 * n, bytes,
                          &full[st]);
    };

    const long long first = blockIdx.x, stride = gridDim.x;
    if (tid == 0) {
        if (first < ntiles) issue(first, 0);
        if (first + stride < ntiles) issue(first + stride, 1);
    }
    int it = 0;
    for (long long tl = first; tl < ntiles; tl += stride, it++) {
        const int st = it & 1;
        const unsigned phase = (unsigned)(it >> 1) & 1u;
        if (tid == 0) {
            s_ok = tma::mbar_wait(&full[st], phase, kWaitLimit) ? 1 : 0;
            if (!s_ok) {
                atomicCAS(&g_batch_status[0], 0u, (unsigned)TPRGB_ETIMEOUT);
                g_batch_status[1] = 1;
                g_batch_status[2] = (unsigned)tl;
            }
        }
        __syncthreads();
        if (!s_ok) {
            // leave no copy in flight: thread 0 waits (bounded again) for
            // the late copies into the stage that timed out, then for the
            // other stage's copies if they were issued
            if (tid == 0) {
                tma::mbar_wait(&full[st], phase, kWaitLimit);
                if (tl + stride < ntiles)
                    tma::mbar_wait(&full[st ^ 1], (unsigned)((it + 1) >> 1) & 1u,
                                   kWaitLimit);
            }
            return;
        }
        const int g = tid / T, t = tid & (T - 1);
        const long long sys = tl * G + g;
        const bool active = sys < nsys;
        const float *base_s = stages + st * 4 * TILE + g * n + t * L;
        const unsigned no_off[L / 4] = {};
        tile::Part pc;
        pc.on = 0;
        pc.P = 1;
        pc.p = 0;
        pc.round = 0;
        tile::run_tile_smem<L, NT, T, MODE>(
            base_s, base_s + TILE, base_s + 2 * TILE, base_s + 3 * TILE, no_off,
            gx, active ? sys * n + (long long)t * L : 0, active, t, t == 0,
            t == T - 1, refine_steps, x_f64, sm, pc);
        __syncthreads();  // every thread is done reading this stage
        if (tid == 0 && tl + 2 * stride < ntiles) issue(tl + 2 * stride, st);
    }
}

}  // namespace bt

template <int L, int NT, int T, int MODE>
static int launch_tma_t(const BatchArgs &A, cudaStream_t st) {
    constexpr int G = NT / T;
    const size_t smem = 2ull * 4 * NT * L * sizeof(float);
    auto k = bt::batch_tma<L, NT, T, MODE>;
    static DeviceOnce grid_cap;
    int dev = 0;
    TPRGB_CUDA(cudaGetDevice(&dev));
    int cap = grid_cap.get(dev);
    if (!cap) {
        TPRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
        int sms = 0, per = 0;
        TPRGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        TPRGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, NT, smem));
        cap = std::max(1, sms * std::max(per, 1));
        grid_cap.set(dev, cap);
    }
    const long long ntiles = (A.nsys + G - 1) / G;
    const int grid = (int)std::min<long long>(ntiles, cap);
    k<<<grid, NT, smem, st>>>(A.a, A.b, A.c, A.d, A.x, A.nsys, A.refine_steps,
                              A.x_f64);
    TPRGB_CUDA(cudaGetLastError());
    return TPRGB_OK;
}

template <int L, int NT, int T>
static int launch_tma_mode(const BatchArgs &A, cudaStream_t st) {
    if (A.refine_steps <= 0) return launch_tma_t<L, NT, T, 0>(A, st);
    return launch_tma_t<L, NT, T, 1>(A, st);
}

template <int L, int NT>
static int launch_tma_T(const BatchArgs &A, cudaStream_t st) {
    switch (A.n / L) {
        case 2: return launch_tma_mode<L, NT, 2>(A, st);
        case 4: return launch_tma_mode<L, NT, 4>(A, st);
        case 8: return launch_tma_mode<L, NT, 8>(A, st);
        case 16: return launch_tma_mode<L, NT, 16>(A, st);
        case 32: return launch_tma_mode<L, NT, 32>(A, st);
        case 64: return launch_tma_mode<L, NT, (NT >= 64 ? 64 : NT)>(A, st);
        case 128: return launch_tma_mode<L, NT, (NT >= 128 ? 128 : NT)>(A, st);
        case 256: return launch_tma_mode<L, NT, (NT >= 256 ? 256 : NT)>(A, st);
        case 512: return launch_tma_mode<L, NT, (NT >= 512 ? 512 : NT)>(A, st);
        default: return fail(TPRGB_EINVAL, "unsupported threads per system");
    }
}

// TMA-staged uniform batch (FP64 residual mode not provided: use the
// register kernel).  Tiles: L in {4, 8}, nt in {128, 256, 512}.
int launch_batch_tma(const BatchArgs &A, const TileConfig &cfg, cudaStream_t st) {
    int rc = batch_config_check(A.n, cfg);
    if (rc) return rc;
    if (A.residual == TPRGB_RESID_F64 && A.refine_steps > 0)
        return fail(TPRGB_EUNSUPPORTED, "staged kernel has no FP64 residual mode");
    if (cfg.nt != 128 && cfg.nt != 256 && cfg.nt != 512)
        return fail(TPRGB_EINVAL, "staged kernel tiles use 128, 256 or 512 threads");
    if (A.nsys == 0) return TPRGB_OK;
    if (cfg.L == 4) {
        if (cfg.nt == 128) return launch_tma_T<4, 128>(A, st);
        return cfg.nt == 256 ? launch_tma_T<4, 256>(A, st) : launch_tma_T<4, 512>(A, st);
    }
    if (cfg.nt == 128) return launch_tma_T<8, 128>(A, st);
    return cfg.nt == 256 ? launch_tma_T<8, 256>(A, st) : launch_tma_T<8, 512>(A, st);
}

}  // namespace tprgb

extern "C" TPRGB_API int tprgb_batch_status(unsigned *code, int reset) {
    using namespace tprgb;
    unsigned v[4], w[4];
    TPRGB_CUDA(cudaMemcpyFromSymbol(v, g_batch_status, sizeof(v)));
    int rc = sw_status(w, reset != 0);
    if (rc) return rc;
    if (v[0] == 0 && w[0] != 0)
        for (int i = 0; i < 4; i++) v[i] = w[i];
    if (code) *code = v[0];
    if (reset) {
        unsigned z[4] = {0, 0, 0, 0};
        TPRGB_CUDA(cudaMemcpyToSymbol(g_batch_status, z, sizeof(z)));
    }
    if (v[0] == TPRGB_ETIMEOUT)
        return fail(TPRGB_ETIMEOUT, "a staged-kernel wait gave up at tile %u", v[2]);
    return TPRGB_OK;
}
