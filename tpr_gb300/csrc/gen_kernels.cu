// Seeded synthetic systems generated directly in device memory (the serving
// loop's "state kept on device" mode, and fast workload set-up).
//
// Counter-based: every value is a hash of (seed, equation index, stream id)
// with the SplitMix64 finaliser (Steele, Lea & Flood, OOPSLA 2014), so any
// equation can be produced independently and the host can reproduce the
// same bits (tpr_gb300/devgen.py).
//   a[i] = 2u - 1 (a[0] = 0), c[i] = 2u - 1 (c[n-1] = 0)
//   b[i] = |a[i]| + |c[i]| + margin(u), margin per kind:
//          dominant U(1,2) | uneven U(0.1,1) | weak 10^U(-4,-1)
//   x_t[i] = 2u - 1;  d[i] = a[i] x_t[i-1] + b[i] x_t[i] + c[i] x_t[i+1]
// All FP32 arithmetic is explicitly rounded (no contraction) so the host
// mirror is bit-exact.
#include "common.cuh"

namespace tprgb {
namespace gen {

__host__ __device__ inline unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// uniform in [0, 1) with 24 random bits
__device__ __forceinline__ float u01(unsigned long long seed, long long i,
                                     unsigned which) {
    unsigned long long k = mix64(seed ^ mix64(((unsigned long long)i << 2) | which));
    return (float)(k >> 40) * 5.9604644775390625e-08f;  // 2^-24
}

__device__ __forceinline__ float coef(unsigned long long seed, long long i,
                                      unsigned which) {
    return __fsub_rn(__fmul_rn(2.0f, u01(seed, i, which)), 1.0f);
}

__device__ __forceinline__ float xtrue(unsigned long long seed, long long i,
                                       int n) {
    return (i < 0 || i >= n) ? 0.0f : coef(seed, i, 3);
}

__global__ void generate_kernel(int nsys, const long long *__restrict__ off,
                                const int *__restrict__ ns,
                                const unsigned long long *__restrict__ seeds,
                                int kind, float *__restrict__ ga,
                                float *__restrict__ gb, float *__restrict__ gc,
                                float *__restrict__ gd) {
    for (int s = blockIdx.x; s < nsys; s += gridDim.x) {
        const int n = ns[s];
        const long long o = off[s];
        const unsigned long long seed = seeds[s];
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            float a = i == 0 ? 0.0f : coef(seed, i, 0);
            float c = i == n - 1 ? 0.0f : coef(seed, i, 1);
            float u = u01(seed, i, 2), m;
            if (kind == 0)
                m = __fadd_rn(1.0f, u);
            else if (kind == 1)
                m = __fadd_rn(0.1f, __fmul_rn(0.9f, u));
            else
                m = exp10f(__fsub_rn(__fmul_rn(3.0f, u), 4.0f));
            float b = __fadd_rn(__fadd_rn(fabsf(a), fabsf(c)), m);
            float d = __fadd_rn(__fadd_rn(__fmul_rn(a, xtrue(seed, i - 1, n)),
                                          __fmul_rn(b, xtrue(seed, i, n))),
                                __fmul_rn(c, xtrue(seed, i + 1, n)));
            ga[o + i] = a;
            gb[o + i] = b;
            gc[o + i] = c;
            gd[o + i] = d;
        }
    }
}

}  // namespace gen

int launch_generate(int nsys, const long long *off, const int *ns,
                    const unsigned long long *seeds, int kind, float *a,
                    float *b, float *c, float *d, cudaStream_t st) {
    if (nsys <= 0) return TPRGB_OK;
    int blocks = nsys < 152 * 32 ? nsys : 152 * 32;
    gen::generate_kernel<<<blocks, 256, 0, st>>>(nsys, off, ns, seeds, kind, a,
                                                 b, c, d);
    TPRGB_CUDA(cudaGetLastError());
    return TPRGB_OK;
}

}  // namespace tprgb

extern "C" TPRGB_API int tprgb_generate_device(
    int nsys, const int64_t *d_offsets, const int *d_ns,
    const uint64_t *d_seeds, int kind, float *d_a, float *d_b, float *d_c,
    float *d_d, void *stream) {
    using namespace tprgb;
    if (nsys < 0) return fail(TPRGB_EINVAL, "nsys < 0");
    if (kind < 0 || kind > 2) return fail(TPRGB_EINVAL, "kind %d not in 0..2", kind);
    if (nsys > 0 && (!d_offsets || !d_ns || !d_seeds || !d_a || !d_b || !d_c || !d_d))
        return fail(TPRGB_EINVAL, "null device pointer");
    return launch_generate(nsys, (const long long *)d_offsets, d_ns,
                           (const unsigned long long *)d_seeds, kind, d_a, d_b,
                           d_c, d_d, (cudaStream_t)stream);
}
