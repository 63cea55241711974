// Serving loop: continuous batching of solve requests on one GPU.
//
// Device memory: one arena of `budget_bytes`, split into five parallel
// arrays a, b, c, d (FP32) and x (FP64) indexed by the same equation
// number, so one equation range [e0, e0 + neq) holds a request's whole
// state.  An equation-range allocator (first fit, 4-equation alignment)
// admits requests against the budget; a request that does not fit waits in
// FIFO order.  State stays resident from admission to release.
//
// Scheduler thread: admits pending requests (uploading host arrays or
// generating seeded systems into their ranges on a preparation stream),
// merges every admitted, not yet solved request into the next step -- one
// cooperative launch of the persistent queue kernel over the union of
// their systems -- and queues that step behind the running one on the
// compute stream, so requests that arrive while a step runs are solved in
// the next step without an idle gap.  At most two steps are in flight.
// Per-request latency = completion of its step (event) - submission.
#include <algorithm>
#include <atomic>
#include <climits>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.cuh"
#include "tile.cuh"

namespace tprgb {

// plan_kernels.cu / gen_kernels.cu
int build_items(int nsys, const int64_t *offsets, const int *ns, int nt,
                std::vector<int> &order, std::vector<int4> &items,
                std::vector<long long> &off, int &slot,
                std::vector<Route> *routes);
int persistent_capacity(int nt, int mode, int *resident);
int launch_persistent(int nt, int mode, int grid, const float *a,
                      const float *b, const float *c, const float *d, void *x,
                      const int4 *items, int nitems, const long long *off,
                      unsigned *ctl, float *scratch, int refine_steps,
                      int x_f64, cudaStream_t st);
int launch_generate(int nsys, const long long *off, const int *ns,
                    const unsigned long long *seeds, int kind, float *a,
                    float *b, float *c, float *d, cudaStream_t st);

using Clock = std::chrono::steady_clock;

// Equation-range allocator.
class RangeAlloc {
   public:
    explicit RangeAlloc(long long cap) : cap_(cap) { free_[0] = cap; }
    // ranges start at multiples of 32 equations (128-byte rows of the
    // staged kernels' tensor-map loads)
    long long alloc(long long n) {
        n = (n + 31) & ~31LL;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                long long at = it->first, rest = it->second - n;
                free_.erase(it);
                if (rest) free_[at + n] = rest;
                used_ += n;
                return at;
            }
        }
        return -1;
    }
    void release(long long at, long long n) {
        n = (n + 31) & ~31LL;
        used_ -= n;
        auto it = free_.emplace(at, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    long long used() const { return used_; }
    long long cap() const { return cap_; }

   private:
    long long cap_, used_ = 0;
    std::map<long long, long long> free_;
};

struct Request {
    uint64_t ticket = 0;
    int nsys = 0;
    long long neq = 0, at = -1;
    std::vector<int> ns;
    std::vector<long long> rel;  // offsets inside the request
    // seeded
    std::vector<unsigned long long> seeds;
    int kind = 0;
    // host arrays
    const float *ha = nullptr, *hb = nullptr, *hc = nullptr, *hd = nullptr;
    double *hx = nullptr;
    Clock::time_point t_submit, t_done;
    double queue_us = 0.0;  // submission -> the finishing step was enqueued
    float step_us = 0.f;    // device time of the finishing step
    int state = 0;  // 0 pending, 1 admitted, 2 in step, 3 done, 4 failed
    int status = TPRGB_OK;
    unsigned nonfinite = 0;
    long long step = -1;     // the step that solved its last system
    int next_sys = 0;        // first system not yet given to a step
    int unfinished = 0;      // systems given to steps and not yet solved
    int timed_out = 0;
};

struct Step {
    long long id;
    // systems [first, first + count) of each request in this step
    struct Part {
        std::shared_ptr<Request> req;
        int first, count;
    };
    std::vector<Part> parts;
    std::vector<int> order;  // sorted system -> flattened index
    std::vector<int> owner;  // flattened index -> entry of parts
    int nsys = 0;
    cudaEvent_t start = nullptr, done = nullptr;
    Clock::time_point t_launch;
    int buf = 0;
};

struct Server {
    tprgb_server_opts o;
    long long cap_eq = 0;
    float *A = nullptr, *B = nullptr, *Cc = nullptr, *D = nullptr;
    double *X = nullptr;
    RangeAlloc *alloc = nullptr;
    cudaStream_t prep = nullptr, comp = nullptr;
    cudaEvent_t prep_ev[2] = {nullptr, nullptr};
    // a step's routed size groups run on kSides side streams forked from
    // comp and joined before its queue kernel
    static constexpr int kSides = 3;
    cudaStream_t side[kSides] = {};
    cudaEvent_t fork_ev = nullptr, join_ev[kSides] = {};
    // per step buffers (double-buffered): items, offsets, ctl, scratch,
    // generator tables
    struct Buf {
        int4 *items = nullptr;
        long long *off = nullptr;
        unsigned *ctl = nullptr;
        float *scratch = nullptr;
        int4 *h_items = nullptr;
        long long *h_off = nullptr;
        unsigned *h_ctl = nullptr;
        size_t cap_items = 0, cap_sys = 0, cap_large = 0;
    } buf[2];
    // generator tables for seeded requests, double-buffered: pinned host
    // staging + device copy; gen_ev[i] marks when table i may be reused
    struct Gen {
        long long *off = nullptr, *h_off = nullptr;
        int *n = nullptr, *h_n = nullptr;
        unsigned long long *seed = nullptr, *h_seed = nullptr;
        size_t cap = 0;
        cudaEvent_t ev = nullptr;
        bool used = false;
    } gen[2];
    int gen_next = 0;
    cudaEvent_t step_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t start_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    int mode = 1, grid = 0;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> pending;
    std::vector<std::shared_ptr<Request>> ready;  // admitted, not in a step
    std::deque<Step> inflight;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> all;
    uint64_t next_ticket = 1;
    long long next_step = 0;
    std::atomic<bool> stop{false};
    std::thread thr;
    int fatal = TPRGB_OK;
    // stats
    long long steps = 0, systems_done = 0, requests_done = 0, eq_done = 0;
    double busy_ms = 0;
};

static int ensure_buf(Server *s, Server::Buf &b, size_t nitems, size_t nsys,
                      size_t nlarge) {
    if (nitems > b.cap_items) {
        cudaFree(b.items);
        cudaFreeHost(b.h_items);
        size_t c = std::max(nitems, b.cap_items * 2);
        TPRGB_CUDA(cudaMalloc(&b.items, sizeof(int4) * c));
        TPRGB_CUDA(cudaHostAlloc(&b.h_items, sizeof(int4) * c, 0));
        b.cap_items = c;
    }
    if (nsys + nlarge + 16 > b.cap_sys) {
        cudaFree(b.off);
        cudaFree(b.ctl);
        cudaFreeHost(b.h_off);
        cudaFreeHost(b.h_ctl);
        size_t c = std::max(nsys + nlarge + 16, b.cap_sys * 2);
        TPRGB_CUDA(cudaMalloc(&b.off, sizeof(long long) * c));
        TPRGB_CUDA(cudaMalloc(&b.ctl, sizeof(unsigned) * (c + 16)));
        TPRGB_CUDA(cudaHostAlloc(&b.h_off, sizeof(long long) * c, 0));
        TPRGB_CUDA(cudaHostAlloc(&b.h_ctl, sizeof(unsigned) * (c + 16), 0));
        b.cap_sys = c;
    }
    if (nlarge > b.cap_large) {
        cudaFree(b.scratch);
        size_t c = std::max(nlarge, b.cap_large * 2);
        TPRGB_CUDA(cudaMalloc(&b.scratch, sizeof(float) * tile::kScratchFloats * c));
        b.cap_large = c;
    }
    (void)s;
    return TPRGB_OK;
}

// Upload an admitted host-array request into its range (async).
static int prepare_host(Server *s, Request &r) {
    const long long at = r.at;
    size_t bytes = sizeof(float) * (size_t)r.neq;
    TPRGB_CUDA(cudaMemcpyAsync(s->A + at, r.ha, bytes, cudaMemcpyHostToDevice, s->prep));
    TPRGB_CUDA(cudaMemcpyAsync(s->B + at, r.hb, bytes, cudaMemcpyHostToDevice, s->prep));
    TPRGB_CUDA(cudaMemcpyAsync(s->Cc + at, r.hc, bytes, cudaMemcpyHostToDevice, s->prep));
    TPRGB_CUDA(cudaMemcpyAsync(s->D + at, r.hd, bytes, cudaMemcpyHostToDevice, s->prep));
    return TPRGB_OK;
}

static int gen_reserve(Server::Gen &g, size_t nsys) {
    if (nsys <= g.cap) return TPRGB_OK;
    if (g.used) TPRGB_CUDA(cudaEventSynchronize(g.ev));
    cudaFree(g.off);
    cudaFree(g.n);
    cudaFree(g.seed);
    cudaFreeHost(g.h_off);
    cudaFreeHost(g.h_n);
    cudaFreeHost(g.h_seed);
    size_t c = std::max(nsys, 2 * g.cap);
    TPRGB_CUDA(cudaMalloc(&g.off, sizeof(long long) * c));
    TPRGB_CUDA(cudaMalloc(&g.n, sizeof(int) * c));
    TPRGB_CUDA(cudaMalloc(&g.seed, sizeof(unsigned long long) * c));
    TPRGB_CUDA(cudaHostAlloc(&g.h_off, sizeof(long long) * c, 0));
    TPRGB_CUDA(cudaHostAlloc(&g.h_n, sizeof(int) * c, 0));
    TPRGB_CUDA(cudaHostAlloc(&g.h_seed, sizeof(unsigned long long) * c, 0));
    g.cap = c;
    return TPRGB_OK;
}

// Generate every seeded request admitted in this round with one table
// upload and one generator launch on the preparation stream.
static int prepare_seeded(Server *s, std::vector<Request *> &rs) {
    size_t total = 0;
    for (Request *r : rs) total += (size_t)r->nsys;
    if (!total) return TPRGB_OK;
    Server::Gen &g = s->gen[s->gen_next];
    s->gen_next ^= 1;
    if (g.used) TPRGB_CUDA(cudaEventSynchronize(g.ev));  // table free again
    int rc = gen_reserve(g, total);
    if (rc) return rc;
    size_t k = 0;
    for (Request *r : rs)
        for (int j = 0; j < r->nsys; j++, k++) {
            g.h_off[k] = r->at + r->rel[j];
            g.h_n[k] = r->ns[j];
            g.h_seed[k] = r->seeds[j];
        }
    TPRGB_CUDA(cudaMemcpyAsync(g.off, g.h_off, sizeof(long long) * total,
                               cudaMemcpyHostToDevice, s->prep));
    TPRGB_CUDA(cudaMemcpyAsync(g.n, g.h_n, sizeof(int) * total,
                               cudaMemcpyHostToDevice, s->prep));
    TPRGB_CUDA(cudaMemcpyAsync(g.seed, g.h_seed, sizeof(unsigned long long) * total,
                               cudaMemcpyHostToDevice, s->prep));
    // one generator launch per run of consecutive requests of one kind
    size_t b = 0;
    for (size_t i = 0; i < rs.size();) {
        size_t j = i, e = b;
        while (j < rs.size() && rs[j]->kind == rs[i]->kind) e += (size_t)rs[j++]->nsys;
        rc = launch_generate((int)(e - b), g.off + b, g.n + b, g.seed + b,
                             rs[i]->kind, s->A, s->B, s->Cc, s->D, s->prep);
        if (rc) return rc;
        b = e;
        i = j;
    }
    TPRGB_CUDA(cudaEventRecord(g.ev, s->prep));
    g.used = true;
    return TPRGB_OK;
}

// Build and enqueue one step over all ready requests.  Called with mu held.
static int launch_step(Server *s) {
    Step st;
    st.id = s->next_step++;
    std::vector<int64_t> off;
    std::vector<int> ns;
    // whole systems from the ready requests in FIFO order, up to the step's
    // equation cap (a request larger than the cap spans several steps; the
    // first system is always taken so every step makes progress)
    const long long cap = s->o.max_step_eq > 0 ? s->o.max_step_eq : LLONG_MAX;
    long long eq = 0;
    size_t keep_from = 0;
    for (size_t q = 0; q < s->ready.size(); q++) {
        auto &rp = s->ready[q];
        Request &r = *rp;
        const int first = r.next_sys;
        int k = first;
        while (k < r.nsys && (eq == 0 || eq + r.ns[k] <= cap)) {
            off.push_back(r.at + r.rel[k]);
            ns.push_back(r.ns[k]);
            st.owner.push_back((int)st.parts.size());
            eq += r.ns[k];
            k++;
        }
        if (k > first) {
            st.parts.push_back(Step::Part{rp, first, k - first});
            r.next_sys = k;
            r.unfinished += k - first;
            r.state = 2;
        }
        if (r.next_sys < r.nsys) {  // cap reached inside this request
            keep_from = q;
            break;
        }
        keep_from = q + 1;
    }
    s->ready.erase(s->ready.begin(), s->ready.begin() + keep_from);
    st.nsys = (int)ns.size();
    std::vector<int4> items;
    std::vector<long long> soff;
    int nlarge = 0;
    std::vector<Route> routes;
    const bool use_routes = s->o.kernel_routes && s->mode != 2;
    int rc = build_items(st.nsys, off.data(), ns.data(), s->o.threads_per_cta,
                         st.order, items, soff, nlarge, use_routes ? &routes : nullptr);
    if (rc) return rc;
    // both buffers alternate; a buffer is reused two steps later, after the
    // step that used it completed (at most two steps in flight)
    st.buf = (int)(st.id & 1);
    Server::Buf &b = s->buf[st.buf];
    rc = ensure_buf(s, b, items.size(), st.nsys, nlarge);
    if (rc) return rc;
    std::copy(items.begin(), items.end(), b.h_items);
    std::copy(soff.begin(), soff.end(), b.h_off);
    const size_t ctl_words = 16 + nlarge + st.nsys;
    std::fill(b.h_ctl, b.h_ctl + ctl_words, 0u);
    b.h_ctl[1] = (unsigned)(16 + nlarge);
    cudaStream_t cs = s->comp;
    st.start = s->start_ev[st.id & 3];
    st.t_launch = Clock::now();
    TPRGB_CUDA(cudaEventRecord(st.start, cs));
    TPRGB_CUDA(cudaEventRecord(s->prep_ev[st.buf], s->prep));
    TPRGB_CUDA(cudaStreamWaitEvent(cs, s->prep_ev[st.buf], 0));
    TPRGB_CUDA(cudaMemcpyAsync(b.items, b.h_items, sizeof(int4) * items.size(),
                               cudaMemcpyHostToDevice, cs));
    TPRGB_CUDA(cudaMemcpyAsync(b.off, b.h_off, sizeof(long long) * st.nsys,
                               cudaMemcpyHostToDevice, cs));
    TPRGB_CUDA(cudaMemcpyAsync(b.ctl, b.h_ctl, sizeof(unsigned) * ctl_words,
                               cudaMemcpyHostToDevice, cs));
    // size groups on the staged / cluster kernels (largest first, dealt
    // round-robin onto the side streams), the rest on the queue kernel
    // after the side streams join
    const int nsides = std::min<int>(Server::kSides, (int)routes.size());
    const bool fork = nsides > 1;
    if (fork) {
        TPRGB_CUDA(cudaEventRecord(s->fork_ev, cs));
        for (int i = 0; i < nsides; i++)
            TPRGB_CUDA(cudaStreamWaitEvent(s->side[i], s->fork_ev, 0));
    }
    int ri = 0;
    for (const Route &r : routes) {
        BatchArgs A{s->A, s->B, s->Cc, s->D, s->X, r.count, r.n, s->o.refine_steps,
                    s->o.residual, 1};
        A.sys_off = b.off + r.first;
        A.sys_status = b.ctl + 16 + nlarge + r.first;
        A.status = b.ctl + 4;
        A.total_eq = s->cap_eq;
        cudaStream_t rs = fork ? s->side[ri++ % nsides] : cs;
        rc = r.kind == 2 ? launch_batch_cl(A, r.cfg, rs) : launch_batch_sw(A, r.cfg, rs);
        if (rc) break;
    }
    // join even after a failed launch, so the step stream still orders
    // after whatever was launched on the side streams
    if (fork) {
        for (int i = 0; i < nsides; i++) {
            TPRGB_CUDA(cudaEventRecord(s->join_ev[i], s->side[i]));
            TPRGB_CUDA(cudaStreamWaitEvent(cs, s->join_ev[i], 0));
        }
    }
    if (rc) return rc;
    int grid = std::max(1, std::min(s->grid, (int)items.size()));
    rc = launch_persistent(s->o.threads_per_cta, s->mode, grid, s->A, s->B,
                           s->Cc, s->D, s->X, b.items, (int)items.size(), b.off,
                           b.ctl, b.scratch, s->o.refine_steps, 1, cs);
    if (rc) return rc;
    // per-system status back to the pinned copy (read after completion)
    TPRGB_CUDA(cudaMemcpyAsync(b.h_ctl, b.ctl, sizeof(unsigned) * ctl_words,
                               cudaMemcpyDeviceToHost, cs));
    // host-array requests: solved systems back to the caller
    for (auto &pt : st.parts) {
        Request &r = *pt.req;
        if (!r.hx) continue;
        const long long a0 = r.rel[pt.first];
        const long long a1 = pt.first + pt.count < r.nsys ? r.rel[pt.first + pt.count]
                                                          : r.neq;
        TPRGB_CUDA(cudaMemcpyAsync(r.hx + a0, s->X + r.at + a0,
                                   sizeof(double) * (size_t)(a1 - a0),
                                   cudaMemcpyDeviceToHost, cs));
    }
    st.done = s->step_ev[st.id & 3];
    TPRGB_CUDA(cudaEventRecord(st.done, cs));
    s->inflight.push_back(std::move(st));
    return TPRGB_OK;
}

static void finish_step(Server *s, Step &st) {
    Server::Buf &b = s->buf[st.buf];
    const unsigned code = b.h_ctl[4];
    const unsigned nlarge = b.h_ctl[1] - 16;
    auto now = Clock::now();
    float step_ms = 0.f;
    if (cudaEventElapsedTime(&step_ms, st.start, st.done) != cudaSuccess) step_ms = 0.f;
    for (int k = 0; k < st.nsys; k++)
        if (b.h_ctl[16 + nlarge + k]) st.parts[st.owner[st.order[k]]].req->nonfinite++;
    for (auto &pt : st.parts) {
        Request &r = *pt.req;
        if (code == TPRGB_ETIMEOUT) r.timed_out = 1;
        r.unfinished -= pt.count;
        s->systems_done += pt.count;
        if (r.unfinished == 0 && r.next_sys == r.nsys) {
            r.t_done = now;
            r.queue_us =
                std::chrono::duration<double, std::micro>(st.t_launch - r.t_submit).count();
            r.step_us = step_ms * 1e3f;
            r.state = 3;
            r.step = st.id;
            if (r.timed_out)
                r.status = TPRGB_ETIMEOUT;
            else if (r.nonfinite)
                r.status = TPRGB_ENONFINITE;
            s->requests_done++;
            s->eq_done += r.neq;
        }
    }
    s->steps++;
}

static void scheduler(Server *s) {
    std::unique_lock<std::mutex> lk(s->mu);
    while (!s->stop.load()) {
        // 1. completed steps
        while (!s->inflight.empty() &&
               cudaEventQuery(s->inflight.front().done) == cudaSuccess) {
            finish_step(s, s->inflight.front());
            s->inflight.pop_front();
            s->cv_done.notify_all();
        }
        // 2. admission (FIFO; stop at the first request that does not fit)
        std::vector<std::shared_ptr<Request>> adm;
        while (!s->pending.empty()) {
            auto r = s->pending.front();
            long long at = s->alloc->alloc(r->neq);
            if (at < 0) break;
            r->at = at;
            s->pending.pop_front();
            adm.push_back(r);
        }
        if (!adm.empty()) {
            std::vector<Request *> seeded;
            int rc = TPRGB_OK;
            for (auto &r : adm) {
                if (r->ha)
                    rc = rc ? rc : prepare_host(s, *r);
                else
                    seeded.push_back(r.get());
            }
            if (!rc) rc = prepare_seeded(s, seeded);
            for (auto &r : adm) {
                if (rc) {
                    r->state = 4;
                    r->status = rc;
                    r->t_done = Clock::now();
                    s->alloc->release(r->at, r->neq);
                    r->at = -1;
                } else {
                    r->state = 1;
                    s->ready.push_back(r);
                }
            }
            if (rc) s->cv_done.notify_all();
        }
        // 3. next step: keep at most max_inflight (1 or 2) in flight
        if (!s->ready.empty() && (int)s->inflight.size() < s->o.max_inflight) {
            int rc = launch_step(s);
            if (rc) {
                s->fatal = rc;
                for (auto &st : s->inflight)
                    for (auto &pt : st.parts) pt.req->state = 4, pt.req->status = rc;
                s->cv_done.notify_all();
                break;
            }
            continue;
        }
        if (s->inflight.empty() && s->pending.empty() && s->ready.empty()) {
            s->cv_work.wait_for(lk, std::chrono::milliseconds(2));
        } else {
            lk.unlock();
            std::this_thread::yield();
            lk.lock();
        }
    }
}

static void server_free(Server *s) {
    if (s->thr.joinable()) {
        s->stop = true;
        s->cv_work.notify_all();
        s->thr.join();
    }
    if (s->comp) cudaStreamSynchronize(s->comp);
    if (s->prep) cudaStreamSynchronize(s->prep);
    for (int i = 0; i < Server::kSides; i++) {
        if (s->side[i]) {
            cudaStreamSynchronize(s->side[i]);
            cudaStreamDestroy(s->side[i]);
        }
        if (s->join_ev[i]) cudaEventDestroy(s->join_ev[i]);
    }
    if (s->fork_ev) cudaEventDestroy(s->fork_ev);
    for (auto &b : s->buf) {
        cudaFree(b.items);
        cudaFree(b.off);
        cudaFree(b.ctl);
        cudaFree(b.scratch);
        cudaFreeHost(b.h_items);
        cudaFreeHost(b.h_off);
        cudaFreeHost(b.h_ctl);
    }
    for (auto &g : s->gen) {
        cudaFree(g.off);
        cudaFree(g.n);
        cudaFree(g.seed);
        cudaFreeHost(g.h_off);
        cudaFreeHost(g.h_n);
        cudaFreeHost(g.h_seed);
        if (g.ev) cudaEventDestroy(g.ev);
    }
    for (auto &e : s->step_ev)
        if (e) cudaEventDestroy(e);
    for (auto &e : s->start_ev)
        if (e) cudaEventDestroy(e);
    cudaFree(s->A);
    for (int i = 0; i < 2; i++)
        if (s->prep_ev[i]) cudaEventDestroy(s->prep_ev[i]);
    if (s->prep) cudaStreamDestroy(s->prep);
    if (s->comp) cudaStreamDestroy(s->comp);
    delete s->alloc;
    delete s;
}

static int submit(Server *s, std::shared_ptr<Request> r, uint64_t *ticket) {
    if (r->neq > s->cap_eq)
        return fail(TPRGB_EBUSY, "request of %lld equations exceeds the budget (%lld)",
                    r->neq, s->cap_eq);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->fatal) return fail(s->fatal, "server stopped after an error");
    if ((long long)s->pending.size() >= s->o.max_pending)
        return fail(TPRGB_EBUSY, "pending queue full (%d)", s->o.max_pending);
    r->ticket = s->next_ticket++;
    r->t_submit = Clock::now();
    s->pending.push_back(r);
    s->all[r->ticket] = r;
    *ticket = r->ticket;
    s->cv_work.notify_all();
    return TPRGB_OK;
}

static int make_request(int nsys, const int *ns, std::shared_ptr<Request> &r) {
    if (nsys <= 0 || !ns) return fail(TPRGB_EINVAL, "nsys must be > 0");
    r = std::make_shared<Request>();
    r->nsys = nsys;
    r->ns.assign(ns, ns + nsys);
    r->rel.resize(nsys);
    long long o = 0;
    for (int k = 0; k < nsys; k++) {
        if (!is_pow2(ns[k]) || ns[k] < 16)
            return fail(TPRGB_EINVAL, "system %d: n=%d must be a power of two >= 16",
                        k, ns[k]);
        r->rel[k] = o;
        o += ns[k];
    }
    r->neq = o;
    return TPRGB_OK;
}

}  // namespace tprgb

using namespace tprgb;

struct tprgb_server {
    Server *s;
};

extern "C" {

TPRGB_API int tprgb_server_opts_default(tprgb_server_opts *o) {
    if (!o) return fail(TPRGB_EINVAL, "opts is NULL");
    o->budget_bytes = 8ULL << 30;
    o->max_pending = 1 << 20;
    o->refine_steps = 1;
    o->residual = TPRGB_RESID_DF;
    o->threads_per_cta = 256;
    o->max_step_eq = 0;
    o->max_inflight = 2;
    o->kernel_routes = 1;
    return TPRGB_OK;
}

TPRGB_API int tprgb_server_create(const tprgb_server_opts *opts,
                                  tprgb_server **out) {
    if (!out) return fail(TPRGB_EINVAL, "out is NULL");
    *out = nullptr;
    Server *s = new Server();
    if (opts)
        s->o = *opts;
    else
        tprgb_server_opts_default(&s->o);
    if (s->o.threads_per_cta != 256 && s->o.threads_per_cta != 512) {
        delete s;
        return fail(TPRGB_EINVAL, "threads_per_cta must be 256 or 512");
    }
    if (s->o.max_inflight != 1 && s->o.max_inflight != 2) {
        delete s;
        return fail(TPRGB_EINVAL, "max_inflight must be 1 or 2");
    }
    s->mode = s->o.refine_steps <= 0 ? 0 : (s->o.residual == TPRGB_RESID_F64 ? 2 : 1);
    s->cap_eq = (long long)(s->o.budget_bytes / 24) & ~31LL;
    if (s->cap_eq < 1024) {
        delete s;
        return fail(TPRGB_EINVAL, "budget too small");
    }
    int rc = persistent_capacity(s->o.threads_per_cta, s->mode, &s->grid);
    if (!rc && s->grid < 33) rc = fail(TPRGB_EUNSUPPORTED, "too few resident CTAs");
    cudaError_t e = cudaSuccess;
    if (!rc) e = cudaMalloc(&s->A, (size_t)s->cap_eq * 24);
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "server arena");
    if (rc) {
        server_free(s);
        return rc;
    }
    s->B = s->A + s->cap_eq;
    s->Cc = s->B + s->cap_eq;
    s->D = s->Cc + s->cap_eq;
    s->X = reinterpret_cast<double *>(s->D + s->cap_eq);
    s->alloc = new RangeAlloc(s->cap_eq);
    if (cudaStreamCreateWithFlags(&s->prep, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->comp, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->prep_ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->prep_ev[1], cudaEventDisableTiming) != cudaSuccess) {
        server_free(s);
        return fail(TPRGB_ECUDA, "server streams");
    }
    for (auto &e : s->step_ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDefault) != cudaSuccess) rc = TPRGB_ECUDA;
    for (int i = 0; i < Server::kSides; i++) {
        if (cudaStreamCreateWithFlags(&s->side[i], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->join_ev[i], cudaEventDisableTiming) != cudaSuccess)
            rc = TPRGB_ECUDA;
    }
    if (cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming) != cudaSuccess)
        rc = TPRGB_ECUDA;
    for (auto &e : s->start_ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDefault) != cudaSuccess) rc = TPRGB_ECUDA;
    for (auto &g : s->gen) {
        if (cudaEventCreateWithFlags(&g.ev, cudaEventDisableTiming) != cudaSuccess) rc = TPRGB_ECUDA;
        if (!rc) rc = gen_reserve(g, 1 << 16);
    }
    for (auto &b : s->buf)
        if (!rc) rc = ensure_buf(s, b, 1 << 16, 1 << 16, 1 << 12);
    if (rc) {
        server_free(s);
        return rc;
    }
    s->thr = std::thread(scheduler, s);
    *out = new tprgb_server{s};
    return TPRGB_OK;
}

TPRGB_API int tprgb_server_destroy(tprgb_server *srv) {
    if (!srv) return fail(TPRGB_EINVAL, "server is NULL");
    server_free(srv->s);
    delete srv;
    return TPRGB_OK;
}

TPRGB_API int tprgb_server_submit_seeded(tprgb_server *srv, int nsys,
                                         const int *ns, const uint64_t *seeds,
                                         int kind, uint64_t *ticket) {
    if (!srv || !ticket || !seeds) return fail(TPRGB_EINVAL, "null argument");
    if (kind < 0 || kind > 2) return fail(TPRGB_EINVAL, "kind %d not in 0..2", kind);
    std::shared_ptr<Request> r;
    int rc = make_request(nsys, ns, r);
    if (rc) return rc;
    r->seeds.assign(seeds, seeds + nsys);
    r->kind = kind;
    return submit(srv->s, r, ticket);
}

TPRGB_API int tprgb_server_submit_host(tprgb_server *srv, int nsys,
                                       const int *ns, const float *a,
                                       const float *b, const float *c,
                                       const float *d, double *x,
                                       uint64_t *ticket) {
    if (!srv || !ticket || !a || !b || !c || !d)
        return fail(TPRGB_EINVAL, "null argument");
    std::shared_ptr<Request> r;
    int rc = make_request(nsys, ns, r);
    if (rc) return rc;
    r->ha = a;
    r->hb = b;
    r->hc = c;
    r->hd = d;
    r->hx = x;
    return submit(srv->s, r, ticket);
}

TPRGB_API int tprgb_server_wait(tprgb_server *srv, uint64_t ticket,
                                int timeout_ms, tprgb_request_info *info) {
    if (!srv) return fail(TPRGB_EINVAL, "server is NULL");
    Server *s = srv->s;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return fail(TPRGB_ENOTFOUND, "unknown ticket %llu",
                                        (unsigned long long)ticket);
    auto r = it->second;
    auto pred = [&] { return r->state >= 3; };
    if (timeout_ms < 0)
        s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred))
        return fail(TPRGB_ETIMEOUT, "request %llu not done after %d ms",
                    (unsigned long long)ticket, timeout_ms);
    if (info) {
        info->status = r->status;
        info->nonfinite_systems = (int)r->nonfinite;
        info->step = r->step;
        info->latency_us =
            std::chrono::duration<double, std::micro>(r->t_done - r->t_submit).count();
        info->x_offset = r->at;
        info->neq = r->neq;
        info->queue_us = r->queue_us;
        info->step_us = r->step_us;
    }
    return r->status;
}

TPRGB_API int tprgb_server_fetch(tprgb_server *srv, uint64_t ticket,
                                 double *x_host) {
    if (!srv || !x_host) return fail(TPRGB_EINVAL, "null argument");
    Server *s = srv->s;
    std::shared_ptr<Request> r;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(ticket);
        if (it == s->all.end()) return fail(TPRGB_ENOTFOUND, "unknown ticket");
        r = it->second;
        if (r->state != 3) return fail(TPRGB_EBUSY, "request not done");
    }
    TPRGB_CUDA(cudaMemcpy(x_host, s->X + r->at, sizeof(double) * (size_t)r->neq,
                          cudaMemcpyDeviceToHost));
    return TPRGB_OK;
}

TPRGB_API int tprgb_server_fetch_system(tprgb_server *srv, uint64_t ticket,
                                        float *a, float *b, float *c,
                                        float *d) {
    if (!srv || !a || !b || !c || !d) return fail(TPRGB_EINVAL, "null argument");
    Server *s = srv->s;
    std::shared_ptr<Request> r;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(ticket);
        if (it == s->all.end()) return fail(TPRGB_ENOTFOUND, "unknown ticket");
        r = it->second;
        if (r->state != 3) return fail(TPRGB_EBUSY, "request not done");
    }
    size_t bytes = sizeof(float) * (size_t)r->neq;
    TPRGB_CUDA(cudaMemcpy(a, s->A + r->at, bytes, cudaMemcpyDeviceToHost));
    TPRGB_CUDA(cudaMemcpy(b, s->B + r->at, bytes, cudaMemcpyDeviceToHost));
    TPRGB_CUDA(cudaMemcpy(c, s->Cc + r->at, bytes, cudaMemcpyDeviceToHost));
    TPRGB_CUDA(cudaMemcpy(d, s->D + r->at, bytes, cudaMemcpyDeviceToHost));
    return TPRGB_OK;
}

TPRGB_API int tprgb_server_release(tprgb_server *srv, uint64_t ticket) {
    if (!srv) return fail(TPRGB_EINVAL, "server is NULL");
    Server *s = srv->s;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return fail(TPRGB_ENOTFOUND, "unknown ticket");
    auto r = it->second;
    if (r->state < 3) return fail(TPRGB_EBUSY, "request still in flight");
    if (r->at >= 0) s->alloc->release(r->at, r->neq);
    r->at = -1;
    s->all.erase(it);
    s->cv_work.notify_all();
    return TPRGB_OK;
}

TPRGB_API int tprgb_server_get_stats(tprgb_server *srv, tprgb_server_stats *st) {
    if (!srv || !st) return fail(TPRGB_EINVAL, "null argument");
    Server *s = srv->s;
    std::lock_guard<std::mutex> lk(s->mu);
    st->steps = s->steps;
    st->requests_done = s->requests_done;
    st->systems_done = s->systems_done;
    st->equations_done = s->eq_done;
    st->pending = (long long)s->pending.size();
    st->inflight_steps = (long long)s->inflight.size();
    st->arena_used_eq = s->alloc->used();
    st->arena_cap_eq = s->alloc->cap();
    return TPRGB_OK;
}

}  // extern "C"

// ---- load driver: Poisson arrivals of seeded requests ------------------------
#include <random>

extern "C" TPRGB_API int tprgb_server_run_load(
    tprgb_server *srv, int nreq, double rate_per_s, uint64_t seed, int min_sys,
    int max_sys, int kmin, int kmax, int kind, double *latencies_us,
    double *detail_us, double *elapsed_s, long long *systems_out) {
    using namespace tprgb;
    if (!srv || nreq <= 0 || min_sys < 1 || max_sys < min_sys || kmin < 4 ||
        kmax < kmin || kmax > 30)
        return fail(TPRGB_EINVAL, "bad load parameters");
    std::mt19937_64 rng(seed);
    std::uniform_int_distribution<int> nsys_d(min_sys, max_sys), k_d(kmin, kmax);
    std::exponential_distribution<double> gap(rate_per_s > 0 ? rate_per_s : 1.0);
    struct Plan1 {
        std::vector<int> ns;
        std::vector<uint64_t> seeds;
        double t;
    };
    std::vector<Plan1> reqs(nreq);
    double t = 0.0;
    long long total_sys = 0;
    for (int i = 0; i < nreq; i++) {
        int m = nsys_d(rng);
        reqs[i].ns.resize(m);
        reqs[i].seeds.resize(m);
        for (int k = 0; k < m; k++) {
            reqs[i].ns[k] = 1 << k_d(rng);
            reqs[i].seeds[k] = rng();
        }
        total_sys += m;
        if (rate_per_s > 0) t += gap(rng);
        reqs[i].t = t;
    }
    std::vector<uint64_t> tickets(nreq, 0);
    std::vector<int> sub_rc(nreq, TPRGB_OK);
    std::atomic<int> submitted{0};
    const auto t0 = Clock::now();
    std::thread producer([&]() {
        for (int i = 0; i < nreq; i++) {
            auto when = t0 + std::chrono::duration_cast<Clock::duration>(
                                 std::chrono::duration<double>(reqs[i].t));
            std::this_thread::sleep_until(when);
            sub_rc[i] = tprgb_server_submit_seeded(
                srv, (int)reqs[i].ns.size(), reqs[i].ns.data(),
                reqs[i].seeds.data(), kind, &tickets[i]);
            submitted.store(i + 1, std::memory_order_release);
        }
    });
    int first_err = TPRGB_OK;
    Clock::time_point last = t0;
    for (int i = 0; i < nreq; i++) {
        while (submitted.load(std::memory_order_acquire) <= i)
            std::this_thread::sleep_for(std::chrono::microseconds(20));
        if (sub_rc[i]) {
            if (!first_err) first_err = sub_rc[i];
            if (latencies_us) latencies_us[i] = -1.0;
            if (detail_us) detail_us[3 * i] = detail_us[3 * i + 1] = detail_us[3 * i + 2] = -1.0;
            continue;
        }
        tprgb_request_info info;
        int rc = tprgb_server_wait(srv, tickets[i], -1, &info);
        if (rc && !first_err) first_err = rc;
        if (latencies_us) latencies_us[i] = info.latency_us;
        if (detail_us) {
            detail_us[3 * i] = info.queue_us;
            detail_us[3 * i + 1] = info.step_us;
            detail_us[3 * i + 2] = (double)info.neq;
        }
        tprgb_server_release(srv, tickets[i]);
        last = Clock::now();
    }
    producer.join();
    if (elapsed_s) *elapsed_s = std::chrono::duration<double>(last - t0).count();
    if (systems_out) *systems_out = total_sys;
    return first_err;
}
