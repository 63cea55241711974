// Persistent queue kernel for uneven batches (and systems larger than one
// CTA's tile).  A cooperative launch keeps every CTA resident; CTAs pull
// work items from a device counter in queue order (largest systems first).
//
// Work item (int4):
//   x  first system (index into the plan's size-sorted system table)
//   y  small item: number of systems; multi-CTA item: part index p
//   z  n
//   w  bits 0-3 log2(L) | bit 4 multi-CTA | bits 8-13 log2(P) |
//      bits 16-31 scratch slot of the multi-CTA system
//
// Multi-CTA systems are split into P consecutive items.  Deadlock freedom:
// items are pulled in increasing order, so whenever a CTA waits on a part
// that is not yet pulled, every item before it is held by a running CTA
// that does not wait on a later system; with more resident CTAs than
// parts per system (checked on the host) the missing parts are always
// pulled.  Every wait is bounded (tile::part_barrier) and reports
// TPRGB_ETIMEOUT instead of hanging.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "batch.cuh"
#include "tile.cuh"

namespace tprgb {
namespace pk {

// run_tile with the item's threads-per-system T as a compile-time value
template <int L, int NT, int MODE>
__device__ __forceinline__ bool dispatch_T(
    int T, const float *ga, const float *gb, const float *gc, const float *gd,
    void *gx, long long base, bool active, int t, bool first_eq, bool last_eq,
    int refine_steps, int x_f64, tile::Smem<NT> &sm, tile::Part &pc) {
#define TPRGB_CASE(TT)                                                       \
    case TT:                                                                 \
        return tile::run_tile<L, NT, (TT <= NT ? TT : NT), MODE>(            \
            ga, gb, gc, gd, gx, base, active, t, first_eq, last_eq,          \
            refine_steps, x_f64, sm, pc);
    switch (T) {
        TPRGB_CASE(2)
        TPRGB_CASE(4)
        TPRGB_CASE(8)
        TPRGB_CASE(16)
        TPRGB_CASE(32)
        TPRGB_CASE(64)
        TPRGB_CASE(128)
        TPRGB_CASE(256)
        TPRGB_CASE(512)
        default:
            return true;
    }
#undef TPRGB_CASE
}

template <int NT, int MODE>
__global__ void __launch_bounds__(NT, (NT <= 256 ? 2 : 1))
plan_persistent(const float *__restrict__ ga, const float *__restrict__ gb,
                const float *__restrict__ gc, const float *__restrict__ gd,
                void *__restrict__ gx, const int4 *__restrict__ items,
                int nitems, const long long *__restrict__ sys_off,
                unsigned *__restrict__ ctl, float *__restrict__ part_scratch,
                int refine_steps, int x_f64) {
    __shared__ tile::Smem<NT> sm;
    __shared__ int s_item;
    // ctl layout: [0] queue head, [4..7] DeviceStatus, [16..16+nlarge)
    // part counters, then one status word per system (after the counters;
    // offset passed in ctl[1])
    unsigned *head = ctl;
    DeviceStatus *status = reinterpret_cast<DeviceStatus *>(ctl + 4);
    unsigned *counters = ctl + 16;
    unsigned *sys_status = ctl + ctl[1];
    const int tid = threadIdx.x;
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(head, 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= nitems) break;
        const int4 w = items[it];
        const int lg = w.w & 15;
        const int L = 1 << lg;
        const bool multi = (w.w >> 4) & 1;
        const int n = w.z;
        tile::Part pc;
        pc.on = 0;
        pc.P = 1;
        pc.p = 0;
        pc.round = 0;
        pc.status = status;
        pc.item = it;
        pc.nsolve = 0;
        pc.nb_hm = pc.nb_lm = pc.nb_hp = pc.nb_lp = 0.f;
        int T, t, sys;
        bool active, first_eq, last_eq;
        long long base;
        if (!multi) {
            T = n >> lg;
            const int g = tid / T;
            t = tid - g * T;
            active = g < w.y;
            sys = w.x + (active ? g : 0);
            base = active ? sys_off[sys] + (long long)t * L : 0;
            first_eq = t == 0;
            last_eq = t == T - 1;
        } else {
            const int P = 1 << ((w.w >> 8) & 63);
            const int slot = (int)((unsigned)w.w >> 16);
            T = NT;
            t = tid;
            sys = w.x;
            active = true;
            pc.on = 1;
            pc.P = P;
            pc.p = w.y;
            pc.counter = counters + slot;
            pc.rows = part_scratch + (long long)slot * tile::kScratchFloats;
            pc.edges = pc.rows + 2 * 32 * 8;
            base = sys_off[sys] + ((long long)pc.p * NT + t) * L;
            first_eq = pc.p == 0 && t == 0;
            last_eq = pc.p == P - 1 && t == NT - 1;
        }
        bool finite = true;
        if (L == 4)
            finite = dispatch_T<4, NT, MODE>(T, ga, gb, gc, gd, gx, base, active,
                                             t, first_eq, last_eq, refine_steps,
                                             x_f64, sm, pc);
        else
            finite = dispatch_T<8, NT, MODE>(T, ga, gb, gc, gd, gx, base, active,
                                             t, first_eq, last_eq, refine_steps,
                                             x_f64, sm, pc);
        if (active && !finite) atomicOr(&sys_status[sys], 1u);
    }
}

}  // namespace pk

// ---- plan (host) -------------------------------------------------------------

struct Plan {
    int nsys = 0, nitems = 0, nlarge = 0;
    std::vector<Route> routes;  // size groups on the staged / cluster kernels
    long long total_eq = 0;     // extent of the arrays the systems cover
    int nt = 256, refine_steps = 1, residual = TPRGB_RESID_DF, x_f64 = 1;
    int grid = 0;
    std::vector<int> order;  // sorted position -> caller's system index
    std::vector<int> bucket_L;
    int4 *d_items = nullptr;
    long long *d_off = nullptr;
    unsigned *d_ctl = nullptr;    // head, status, counters, per-system status
    size_t ctl_words = 0;
    float *d_scratch = nullptr;   // rows / edges of multi-CTA systems
    // graph replay
    bool use_graph = false, graph_failed = false;
    cudaGraphExec_t gexec = nullptr;
    const void *g_ptrs[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaStream_t cap_stream = nullptr;
    // routed size groups run on kPlanSides side streams forked from the
    // caller's stream (joined before the queue kernel)
    static constexpr int kPlanSides = 3;
    cudaStream_t side[kPlanSides] = {};
    cudaEvent_t fork = nullptr, join[kPlanSides] = {};
};

TileConfig tuned_tile(int n);  // batch_api.cu

template <int NT, int MODE>
static const void *plan_kernel_ptr() {
    return (const void *)pk::plan_persistent<NT, MODE>;
}

static const void *plan_kernel(int nt, int mode) {
    if (nt == 256) {
        if (mode == 0) return plan_kernel_ptr<256, 0>();
        if (mode == 1) return plan_kernel_ptr<256, 1>();
        return plan_kernel_ptr<256, 2>();
    }
    if (mode == 0) return plan_kernel_ptr<512, 0>();
    if (mode == 1) return plan_kernel_ptr<512, 1>();
    return plan_kernel_ptr<512, 2>();
}

// Staged or cluster kernel for the sorted systems [k, e) of size n, if one
// serves them: offsets multiples of 32 equations (rows of the tensor-map
// loads); the tile table's cluster tile where it names one, else
// 256 <= n <= 4096 one CTA per system (swizzled staging) and
// 8192 <= n <= 65536 one thread-block cluster per system.
static bool route_for(int n, const std::vector<long long> &off, int k, int e,
                      Route &r) {
    for (int i = k; i < e; i++)
        if (off[i] & 31) return false;
    TileConfig c = tuned_tile(n);
    // the table's cluster tile wherever it names one (n = 2048 ... 65536)
    if (c.staged == 4 && c.L == 16 &&
        (c.nt == 64 || c.nt == 128 || c.nt == 256 || c.nt == 512) && n % (16 * c.nt) == 0 && n / (16 * c.nt) >= 2 && n / (16 * c.nt) <= 16) {
        r = Route{2, n, k, e - k, c};
        return true;
    }
    if (n >= 256 && n <= 4096) {
        const bool sw = (c.staged == 2 || c.staged == 3) && (c.L == 8 || c.L == 16) &&
                        (c.nt == 64 || c.nt == 128 || c.nt == 256) && n / c.L <= c.nt;
        if (!sw) c = TileConfig{16, std::max(64, n / 16), 3};
        r = Route{1, n, k, e - k, c};
        return true;
    }
    if (n >= 8192 && n <= 65536) {
        if (c.staged != 4) c = TileConfig{16, 256, 4};
        const int P = n / (16 * c.nt);
        if (n % (16 * c.nt) || P < 2 || P > 16) return false;
        r = Route{2, n, k, e - k, c};
        return true;
    }
    return false;
}

// Work items for a batch: systems sorted by decreasing n (order[k] = the
// caller's index of sorted system k, off[k] its offset); small systems
// packed per CTA, larger ones split into P parts (slot = multi-CTA
// systems so far, incremented).  With `routes`, size groups that a staged
// or cluster kernel serves are listed there instead of becoming items.
int build_items(int nsys, const int64_t *offsets, const int *ns, int nt,
                std::vector<int> &order, std::vector<int4> &items,
                std::vector<long long> &off, int &slot,
                std::vector<Route> *routes) {
    order.resize(nsys);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int i, int j) { return ns[i] > ns[j]; });
    items.clear();
    off.resize(nsys);
    for (int k = 0; k < nsys; k++) off[k] = offsets[order[k]];
    int k = 0;
    while (k < nsys) {
        const int n = ns[order[k]];
        int e = k;
        while (e < nsys && ns[order[e]] == n) e++;
        Route r;
        if (routes && route_for(n, off, k, e, r)) {
            routes->push_back(r);
            k = e;
            continue;
        }
        TileConfig tc = tuned_tile(n);
        int L = tc.L == 4 ? 4 : 8;
        if (n < 2 * L) L = 4;
        const int lg = L == 4 ? 2 : 3;
        const long long cap = (long long)nt * L;  // equations per CTA
        if (n <= cap) {
            const int per = (int)(cap / n);
            for (int s0 = k; s0 < e; s0 += per)
                items.push_back(make_int4(s0, std::min(per, e - s0), n, lg));
        } else {
            const long long P = n / cap;
            if (P > 32)
                return fail(TPRGB_EUNSUPPORTED,
                            "n=%d needs %lld CTAs per system (max 32)", n, P);
            const int lp = ilog2(P);
            for (int s = k; s < e; s++, slot++) {
                if (slot > 0xffff)
                    return fail(TPRGB_EUNSUPPORTED, "too many multi-CTA systems");
                for (int q = 0; q < P; q++)
                    items.push_back(
                        make_int4(s, q, n, lg | 16 | (lp << 8) | (slot << 16)));
            }
        }
        k = e;
    }
    return TPRGB_OK;
}

// Resident CTAs of the persistent kernel for (nt, mode).
int persistent_capacity(int nt, int mode, int *resident) {
    const void *kern = plan_kernel(nt, mode);
    int dev = 0, sms = 0, per_sm = 0;
    TPRGB_CUDA(cudaGetDevice(&dev));
    TPRGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TPRGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, 0));
    *resident = sms * per_sm;
    return TPRGB_OK;
}

// Cooperative launch of the persistent kernel.
int launch_persistent(int nt, int mode, int grid, const float *a,
                      const float *b, const float *c, const float *d, void *x,
                      const int4 *items, int nitems, const long long *off,
                      unsigned *ctl, float *scratch, int refine_steps,
                      int x_f64, cudaStream_t st) {
    if (nitems == 0) return TPRGB_OK;
    const void *kern = plan_kernel(nt, mode);
    void *args[] = {(void *)&a, (void *)&b, (void *)&c, (void *)&d, (void *)&x,
                    (void *)&items, (void *)&nitems, (void *)&off,
                    (void *)&ctl, (void *)&scratch, (void *)&refine_steps,
                    (void *)&x_f64};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(nt);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    TPRGB_CUDA(cudaLaunchKernelExC(&cfg, kern, args));
    return TPRGB_OK;
}

static int plan_mode(const Plan &p) {
    if (p.refine_steps <= 0) return 0;
    return p.residual == TPRGB_RESID_F64 ? 2 : 1;
}

static void plan_free(Plan *p) {
    if (!p) return;
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
    for (int i = 0; i < Plan::kPlanSides; i++) {
        if (p->side[i]) cudaStreamDestroy(p->side[i]);
        if (p->join[i]) cudaEventDestroy(p->join[i]);
    }
    if (p->fork) cudaEventDestroy(p->fork);
    cudaFree(p->d_items);
    cudaFree(p->d_off);
    cudaFree(p->d_ctl);
    cudaFree(p->d_scratch);
    delete p;
}

int plan_create(int nsys, const int64_t *offsets, const int *ns,
                const tprgb_batch_opts &o, int nt, Plan **out) {
    *out = nullptr;
    if (nsys < 0) return fail(TPRGB_EINVAL, "nsys < 0");
    if (nsys > 0 && (!offsets || !ns)) return fail(TPRGB_EINVAL, "null host array");
    if (nt != 256 && nt != 512)
        return fail(TPRGB_EINVAL, "plan threads per CTA %d not in {256, 512}", nt);
    for (int k = 0; k < nsys; k++) {
        if (!is_pow2(ns[k]) || ns[k] < 16)
            return fail(TPRGB_EINVAL, "system %d: n=%d must be a power of two >= 16",
                        k, ns[k]);
        if (offsets[k] < 0 || (offsets[k] & 3))
            return fail(TPRGB_EINVAL, "system %d: offset %lld must be a multiple of 4",
                        k, (long long)offsets[k]);
    }
    Plan *p = new Plan();
    p->nsys = nsys;
    p->nt = nt;
    p->refine_steps = o.refine_steps;
    p->residual = o.residual;
    p->x_f64 = o.x_f64;

    std::vector<int4> items;
    std::vector<long long> off;
    int slot = 0;
    // staged / cluster routes unless the caller asks for the register
    // kernel (variant 1) or the FP64 residual (queue kernel only)
    const bool use_routes = o.variant != 1 &&
                            !(o.residual == TPRGB_RESID_F64 && o.refine_steps > 0);
    int rc = build_items(nsys, offsets, ns, nt, p->order, items, off, slot,
                         use_routes ? &p->routes : nullptr);
    for (int k = 0; k < nsys; k++)
        p->total_eq = std::max<long long>(p->total_eq, offsets[k] + ns[k]);
    if (rc) {
        plan_free(p);
        return rc;
    }
    p->nitems = (int)items.size();
    p->nlarge = slot;

    int resident = 0;
    rc = persistent_capacity(nt, plan_mode(*p), &resident);
    if (rc) {
        plan_free(p);
        return rc;
    }
    if (resident < 33) {
        plan_free(p);
        return fail(TPRGB_EUNSUPPORTED, "only %d resident CTAs", resident);
    }
    p->grid = std::max(1, std::min(resident, std::max(p->nitems, 1)));

    p->ctl_words = 16 + (size_t)p->nlarge + (size_t)nsys;
    std::vector<unsigned> ctl_init(16, 0u);
    ctl_init[1] = (unsigned)(16 + p->nlarge);  // start of per-system status
    cudaError_t e = cudaMalloc(&p->d_ctl, sizeof(unsigned) * p->ctl_words);
    if (e == cudaSuccess && p->nitems)
        e = cudaMalloc(&p->d_items, sizeof(int4) * items.size());
    if (e == cudaSuccess && nsys) e = cudaMalloc(&p->d_off, sizeof(long long) * nsys);
    if (e == cudaSuccess && p->nlarge)
        e = cudaMalloc(&p->d_scratch, sizeof(float) * tile::kScratchFloats * (size_t)p->nlarge);
    if (e == cudaSuccess && p->nitems)
        e = cudaMemcpy(p->d_items, items.data(), sizeof(int4) * items.size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nsys)
        e = cudaMemcpy(p->d_off, off.data(), sizeof(long long) * nsys,
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(p->d_ctl, 0, sizeof(unsigned) * p->ctl_words);
    if (e == cudaSuccess)
        e = cudaMemcpy(p->d_ctl, ctl_init.data(), sizeof(unsigned) * 16,
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        plan_free(p);
        return cuda_fail(e, "plan buffers");
    }
    *out = p;
    return TPRGB_OK;
}

// Reset the queue head, the device status, the part counters and the
// per-system status; keep ctl[1] (status offset).
static int plan_reset(Plan *p, cudaStream_t st) {
    TPRGB_CUDA(cudaMemsetAsync(p->d_ctl, 0, sizeof(unsigned), st));
    TPRGB_CUDA(cudaMemsetAsync(p->d_ctl + 2, 0, sizeof(unsigned) * (p->ctl_words - 2), st));
    return TPRGB_OK;
}

// One launch per routed size group, largest first, dealt round-robin onto
// the side streams, so that groups of different sizes (cluster sizes that
// leave SMs idle, staged groups, the kernels' tails) run side by side;
// then, after the side streams join the caller's stream, the queue kernel
// for the remaining systems (its multi-CTA barriers assume all of its CTAs
// become resident, so it runs alone).
static int plan_launch(Plan *p, const float *a, const float *b, const float *c,
                       const float *d, void *x, cudaStream_t st) {
    int rc = plan_reset(p, st);
    if (rc) return rc;
    unsigned *sys_status = p->d_ctl + 16 + p->nlarge;
    const int nsides = std::min<int>(Plan::kPlanSides, (int)p->routes.size());
    const bool fork = nsides > 1;
    if (fork) {
        for (int i = 0; i < nsides; i++) {
            if (!p->side[i])
                TPRGB_CUDA(cudaStreamCreateWithFlags(&p->side[i], cudaStreamNonBlocking));
            if (!p->join[i])
                TPRGB_CUDA(cudaEventCreateWithFlags(&p->join[i], cudaEventDisableTiming));
        }
        if (!p->fork) TPRGB_CUDA(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming));
        TPRGB_CUDA(cudaEventRecord(p->fork, st));
        for (int i = 0; i < nsides; i++)
            TPRGB_CUDA(cudaStreamWaitEvent(p->side[i], p->fork, 0));
    }
    int ri = 0;
    for (const Route &r : p->routes) {
        BatchArgs A{a, b, c, d, x, r.count, r.n, p->refine_steps, p->residual, p->x_f64};
        A.sys_off = p->d_off + r.first;
        A.sys_status = sys_status + r.first;
        A.status = p->d_ctl + 4;
        A.total_eq = p->total_eq;
        cudaStream_t rs = fork ? p->side[ri++ % nsides] : st;
        rc = r.kind == 2 ? launch_batch_cl(A, r.cfg, rs) : launch_batch_sw(A, r.cfg, rs);
        if (rc) break;
    }
    // join even after a failed launch, so the caller's stream still orders
    // after whatever was launched on the side streams
    if (fork) {
        for (int i = 0; i < nsides; i++) {
            TPRGB_CUDA(cudaEventRecord(p->join[i], p->side[i]));
            TPRGB_CUDA(cudaStreamWaitEvent(st, p->join[i], 0));
        }
    }
    if (rc) return rc;
    return launch_persistent(p->nt, plan_mode(*p), p->grid, a, b, c, d, x,
                             p->d_items, p->nitems, p->d_off, p->d_ctl,
                             p->d_scratch, p->refine_steps, p->x_f64, st);
}

int plan_execute(Plan *p, const float *a, const float *b, const float *c,
                 const float *d, void *x, cudaStream_t st) {
    if (!p) return fail(TPRGB_EINVAL, "plan is NULL");
    if (p->nsys > 0 && (!a || !b || !c || !d || !x))
        return fail(TPRGB_EINVAL, "null device pointer");
    for (const void *q : {(const void *)a, (const void *)b, (const void *)c,
                          (const void *)d, (const void *)x})
        if (((uintptr_t)q & 15) != 0)
            return fail(TPRGB_EINVAL, "device arrays must be 16-byte aligned");
    if (!p->use_graph || p->graph_failed) return plan_launch(p, a, b, c, d, x, st);
    const void *ptrs[5] = {a, b, c, d, x};
    bool same = p->gexec && std::equal(ptrs, ptrs + 5, p->g_ptrs);
    if (!same) {
        if (p->gexec) {
            cudaGraphExecDestroy(p->gexec);
            p->gexec = nullptr;
        }
        if (!p->cap_stream)
            TPRGB_CUDA(cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        TPRGB_CUDA(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
        int rc = plan_launch(p, a, b, c, d, x, p->cap_stream);
        cudaError_t ce = cudaStreamEndCapture(p->cap_stream, &g);
        if (rc || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            p->graph_failed = true;  // fall back to direct launches
            return plan_launch(p, a, b, c, d, x, st);
        }
        ce = cudaGraphInstantiate(&p->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            cudaGetLastError();
            p->gexec = nullptr;
            p->graph_failed = true;
            return plan_launch(p, a, b, c, d, x, st);
        }
        std::copy(ptrs, ptrs + 5, p->g_ptrs);
    }
    TPRGB_CUDA(cudaGraphLaunch(p->gexec, st));
    return TPRGB_OK;
}

}  // namespace tprgb

using namespace tprgb;

struct tprgb_plan {
    Plan *p;
};

extern "C" {

TPRGB_API int tprgb_plan_create(int nsys, const int64_t *offsets,
                                const int *ns, const tprgb_batch_opts *opts,
                                tprgb_plan **out) {
    if (!out) return fail(TPRGB_EINVAL, "out is NULL");
    tprgb_batch_opts o;
    if (opts)
        o = *opts;
    else
        tprgb_batch_opts_default(&o);
    if (o.refine_steps < 0 || o.refine_steps > 8)
        return fail(TPRGB_EINVAL, "refine_steps=%d outside [0, 8]", o.refine_steps);
    if (o.residual != TPRGB_RESID_DF && o.residual != TPRGB_RESID_F64)
        return fail(TPRGB_EINVAL, "unknown residual mode %d", o.residual);
    int nt = o.threads_per_cta ? o.threads_per_cta : 256;
    Plan *p = nullptr;
    int rc = plan_create(nsys, offsets, ns, o, nt, &p);
    if (rc) return rc;
    *out = new tprgb_plan{p};
    return TPRGB_OK;
}

TPRGB_API int tprgb_plan_destroy(tprgb_plan *plan) {
    if (!plan) return fail(TPRGB_EINVAL, "plan is NULL");
    cudaDeviceSynchronize();
    plan_free(plan->p);
    delete plan;
    return TPRGB_OK;
}

TPRGB_API int tprgb_plan_use_graph(tprgb_plan *plan, int enable) {
    if (!plan) return fail(TPRGB_EINVAL, "plan is NULL");
    plan->p->use_graph = enable != 0;
    return TPRGB_OK;
}

TPRGB_API int tprgb_plan_execute(tprgb_plan *plan, const float *d_a,
                                 const float *d_b, const float *d_c,
                                 const float *d_d, void *d_x, void *stream) {
    if (!plan) return fail(TPRGB_EINVAL, "plan is NULL");
    return plan_execute(plan->p, d_a, d_b, d_c, d_d, d_x, (cudaStream_t)stream);
}

TPRGB_API int tprgb_plan_info(const tprgb_plan *plan, int *nitems, int *grid,
                              int *nlarge, int *graph_active) {
    if (!plan) return fail(TPRGB_EINVAL, "plan is NULL");
    if (nitems) *nitems = plan->p->nitems;
    if (grid) *grid = plan->p->grid;
    if (nlarge) *nlarge = plan->p->nlarge;
    if (graph_active) *graph_active = plan->p->gexec != nullptr;
    return TPRGB_OK;
}

TPRGB_API int tprgb_plan_routes(const tprgb_plan *plan, int *staged_systems,
                                int *cluster_systems, int *queue_systems,
                                int *launches) {
    if (!plan) return fail(TPRGB_EINVAL, "plan is NULL");
    const Plan *p = plan->p;
    int st = 0, clu = 0;
    for (const Route &r : p->routes) (r.kind == 2 ? clu : st) += r.count;
    if (staged_systems) *staged_systems = st;
    if (cluster_systems) *cluster_systems = clu;
    if (queue_systems) *queue_systems = p->nsys - st - clu;
    if (launches) *launches = (int)p->routes.size() + (p->nitems > 0 ? 1 : 0);
    return TPRGB_OK;
}

TPRGB_API int tprgb_plan_status(tprgb_plan *plan, unsigned *sys_status,
                                unsigned *device_code, void *stream) {
    if (!plan) return fail(TPRGB_EINVAL, "plan is NULL");
    Plan *p = plan->p;
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<unsigned> ctl(8), per(p->nsys);
    TPRGB_CUDA(cudaMemcpyAsync(ctl.data(), p->d_ctl, sizeof(unsigned) * 8,
                               cudaMemcpyDeviceToHost, st));
    if (p->nsys)
        TPRGB_CUDA(cudaMemcpyAsync(per.data(), p->d_ctl + 16 + p->nlarge,
                                   sizeof(unsigned) * p->nsys,
                                   cudaMemcpyDeviceToHost, st));
    TPRGB_CUDA(cudaStreamSynchronize(st));
    if (device_code) *device_code = ctl[4];
    int bad = 0;
    for (int k = 0; k < p->nsys; k++) {
        if (sys_status) sys_status[p->order[k]] = per[k];
        bad += per[k] != 0;
    }
    if (ctl[4] == TPRGB_ETIMEOUT)
        return fail(TPRGB_ETIMEOUT, "a multi-CTA wait gave up (site %u, item %u)",
                    ctl[5], ctl[6]);
    if (bad) return fail(TPRGB_ENONFINITE, "%d systems have non-finite solutions", bad);
    return TPRGB_OK;
}

}  // extern "C"
