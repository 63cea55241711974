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
// variant (0: inputs loaded straight to registers; 1: TMA-staged ring).
struct TileConfig {
    int L;
    int nt;
    int staged = 0;
};

int batch_config_check(int n, const TileConfig &cfg);
int launch_batch_uniform(const BatchArgs &A, const TileConfig &cfg,
                         cudaStream_t st);
int launch_batch_tma(const BatchArgs &A, const TileConfig &cfg, cudaStream_t st);

}  // namespace tprgb
