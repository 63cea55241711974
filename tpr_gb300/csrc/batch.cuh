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
};

// Tile shape: L equations per thread, nt threads per CTA, and the kernel
// variant (0: inputs loaded straight to registers; 1: TMA-staged ring of
// bulk copies; 2: swizzled tensor-map staging, two stages; 3: the same with
// one stage).  The C ABI numbers these variants 1..4.
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
// status word of the swizzled kernels (code, where, tile); reset clears it
int sw_status(unsigned (&v)[4], bool reset);

}  // namespace tprgb
