// Internal interface of the batched solver (batch_kernels.cu, batch_api.cu).
#pragma once

#include "common.cuh"

namespace tprgb {

struct BatchArgs {
    const float *a, *b, *c, *d;
    void *x;
    int nsys, n;
    int refine_steps;
    int residual;  // TPRGB_RESID_*
    int x_f64;
    // swizzled and cluster kernels only: systems at element offsets sys_off
    // (device; null: system k at k * n), non-finite flags per system
    // (device, may be null), timeout record (device, null: the batch word)
    const long long *sys_off = nullptr;
    unsigned *sys_status = nullptr;
    unsigned *status = nullptr;
    long long total_eq = 0;  // elements of each array (0: nsys * n)
};

// Tile shape: L equations per thread, nt threads per CTA, and the kernel
// variant (0: inputs loaded straight to registers; 1: TMA-staged ring of
// bulk copies; 2: swizzled tensor-map staging, two stages; 3: the same with
// one stage; 4: one system per thread-block cluster).  The C ABI numbers
// these variants 1..5.
struct TileConfig {
    int L;
    int nt;
    int staged = 0;
};

int batch_config_check(int n, const TileConfig &cfg);
int launch_batch_uniform(const BatchArgs &A, const TileConfig &cfg,
                         cudaStream_t st);
int launch_batch_tma(const BatchArgs &A, const TileConfig &cfg, cudaStream_t st);
int launch_batch_sw(const BatchArgs &A, const TileConfig &cfg, cudaStream_t st);
int launch_batch_cl(const BatchArgs &A, const TileConfig &cfg, cudaStream_t st);

// A size group of a plan solved by the staged (kind 1) or cluster (kind 2)
// kernel: sorted systems [first, first + count) of size n.
struct Route {
    int kind = 0;
    int n = 0, first = 0, count = 0;
    TileConfig cfg{16, 64, 3};
};
// CTAs per system of the cluster variant for size n (error if invalid)
int cluster_parts(int n, const TileConfig &cfg, int *P);
// status word of the swizzled kernels (code, where, tile); reset clears it
int sw_status(unsigned (&v)[4], bool reset);

}  // namespace tprgb
