// tpr_gb.hpp -- header-only C++ drop-in for the reference's solver classes
// and GPU free functions, implemented over the C ABI in tpr_gb.h.
//
//   reference                                   here
//   class PTPR (src/ptpr.hpp:44-110)        ->  tprgb::PTPR   (also ::PTPR
//   class TPR  (src/tpr.hpp:44-112)              tprgb::TPR    with
//   class CR   (src/cr.hpp:24-81)                tprgb::CR     TPRGB_GLOBAL_
//   class PCR  (src/pcr.hpp:8-68)                tprgb::PCR    NAMES)
//   TPR_CU::tpr_cu / cr_cu (src/tpr.cuh:50-57)   TPR_CU::tpr_cu / cr_cu
//   PTPR_CU::ptpr_cu / pcr_cu (src/ptpr.cuh)     PTPR_CU::ptpr_cu / pcr_cu
//
// `real` is float unless _REAL_IS_DOUBLE_ is defined (src/lib.hpp:8-16).
// Same call sequence as the reference:
//     PTPR t(n, s);
//     t.set_tridiagonal_system(a, c, rhs);   // or (a, diag, c, rhs)
//     int flops = t.solve();
//     t.get_ans(x);
// Differences, all on the safe side: the solve runs on the GPU; the
// caller's arrays are copied at set_tridiagonal_system time and never
// modified (the reference keeps the pointers and overwrites a, c, rhs);
// errors throw tprgb::Error instead of exit()/abort().
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "tpr_gb.h"

#ifdef _REAL_IS_DOUBLE_
using tprgb_real = double;
#define TPRGB_REAL_PREC TPRGB_F64
#else
using tprgb_real = float;
#define TPRGB_REAL_PREC TPRGB_F32
#endif

namespace tprgb {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != TPRGB_OK) throw Error(rc, tprgb_last_error());
}

template <int KIND>
class Solver {
   public:
    using real = tprgb_real;

    Solver(int n, int s) : n_(n), s_(s) { init(); }
    // Copy constructor re-initialises its own buffers, as the reference's
    // does (src/ptpr.hpp:74-78) -- the basis of one-object-per-thread use.
    Solver(const Solver &o) : n_(o.n_), s_(o.s_) { init(); }
    Solver &operator=(const Solver &) = delete;
    ~Solver() {
        if (h_) tprgb_destroy(h_);
    }

    // 3-argument form: unit diagonal (src/ptpr.cpp:39-43)
    void set_tridiagonal_system(real *a, real *c, real *rhs) {
        check(tprgb_set_system(h_, a, nullptr, c, rhs));
    }
    // 4-argument form: normalised by diag (src/ptpr.hpp:80-90)
    void set_tridiagonal_system(real *a, real *diag, real *c, real *rhs) {
        check(tprgb_set_system(h_, a, diag, c, rhs));
    }
    int solve() {
        int f = 0;
        check(tprgb_solve(h_, &f));
        return f;
    }
    int get_ans(real *x) {
        check(tprgb_get_ans(h_, x));
        return 0;
    }

   protected:
    void init() { check(tprgb_create(KIND, n_, s_, TPRGB_REAL_PREC, &h_)); }
    int n_, s_;
    tprgb_solver *h_ = nullptr;
};

class PTPR : public Solver<TPRGB_PTPR> {
   public:
    PTPR(int n, int s) : Solver(n, s) {}
    PTPR(real *a, real *diag, real *c, real *rhs, int n, int s)
        : Solver(n, s) {
        set_tridiagonal_system(a, diag, c, rhs);  // src/ptpr.hpp:53-56
    }
};

class TPR : public Solver<TPRGB_TPR> {
   public:
    TPR(int n, int s) : Solver(n, s) {}
    // the reference's 6-argument TPR constructor ignores diag
    // (src/tpr.hpp:53-56)
    TPR(real *a, real *diag, real *c, real *rhs, int n, int s)
        : Solver(n, s) {
        (void)diag;
        set_tridiagonal_system(a, c, rhs);
    }
};

class CR : public Solver<TPRGB_CR> {
   public:
    explicit CR(int n) : Solver(n, n) {}
    // the reference's CR setter ignores diag (src/cr.cpp:17-21)
    CR(real *a, real *diag, real *c, real *rhs, int n) : Solver(n, n) {
        set_tridiagonal_system(a, diag, c, rhs);
    }
};

class PCR : public Solver<TPRGB_PCR> {
   public:
    explicit PCR(int n) : Solver(n, n) {}
    // the reference's 5-argument PCR constructor uses the 3-argument
    // setter (src/pcr.hpp:14-17)
    PCR(real *a, real *diag, real *c, real *rhs, int n) : Solver(n, n) {
        (void)diag;
        set_tridiagonal_system(a, c, rhs);
    }
};

// ---- batched solving (no counterpart in the reference, whose benchmark
// loops over single systems, src/pm.cpp:224-238): RAII wrappers over the C
// ABI's batch, host-pipeline, plan and server entry points.  Every call
// throws tprgb::Error on a non-OK status. -----------------------------------

// tprgb_batch_opts with the library defaults (FP32 + 1 refinement step,
// compensated residual, FP64 x, tuned tile).
struct BatchOptions : tprgb_batch_opts {
    BatchOptions() { check(tprgb_batch_opts_default(this)); }
    BatchOptions &refine(int steps) {
        refine_steps = steps;
        return *this;
    }
    BatchOptions &fp32_output() {
        x_f64 = 0;
        return *this;
    }
};

// nsys systems of n equations back to back in device arrays; asynchronous
// on `stream` (a cudaStream_t, or nullptr for the default stream).
inline void batch_solve(int nsys, int n, const float *d_a, const float *d_b,
                        const float *d_c, const float *d_d, void *d_x,
                        const BatchOptions &o = BatchOptions(),
                        void *stream = nullptr) {
    check(tprgb_batch_solve(nsys, n, d_a, d_b, d_c, d_d, d_x, &o, stream));
}

// Host arrays in and out (pinned for full link speed); device buffers for
// chunks of up to chunk_eq equations are allocated once, here.
class HostPipeline {
   public:
    explicit HostPipeline(int64_t chunk_eq = int64_t(1) << 22) {
        check(tprgb_host_ctx_create(chunk_eq, &h_));
    }
    HostPipeline(const HostPipeline &) = delete;
    HostPipeline &operator=(const HostPipeline &) = delete;
    ~HostPipeline() {
        if (h_) tprgb_host_ctx_destroy(h_);
    }
    // x: double[nsys * n] (float[] with o.fp32_output()); synchronous
    void solve(int nsys, int n, const float *a, const float *b, const float *c,
               const float *d, void *x, const BatchOptions &o = BatchOptions()) {
        check(tprgb_batch_solve_host(h_, nsys, n, a, b, c, d, x, &o));
    }

   private:
    tprgb_host_ctx *h_ = nullptr;
};

// Uneven batch: sizes and offsets fixed at construction, executed many
// times (optionally replayed from a CUDA graph).
class Plan {
   public:
    Plan(int nsys, const int64_t *offsets, const int *ns,
         const BatchOptions &o = BatchOptions(), bool graph = true)
        : nsys_(nsys) {
        check(tprgb_plan_create(nsys, offsets, ns, &o, &p_));
        check(tprgb_plan_use_graph(p_, graph ? 1 : 0));
    }
    Plan(const Plan &) = delete;
    Plan &operator=(const Plan &) = delete;
    ~Plan() {
        if (p_) tprgb_plan_destroy(p_);
    }
    void execute(const float *d_a, const float *d_b, const float *d_c,
                 const float *d_d, void *d_x, void *stream = nullptr) {
        check(tprgb_plan_execute(p_, d_a, d_b, d_c, d_d, d_x, stream));
    }
    // Waits for `stream`; per-system flags (1: non-finite solution) in the
    // caller's order.  Returns the status instead of throwing on
    // TPRGB_ENONFINITE, the expected outcome for singular systems.
    int status(std::vector<unsigned> &per_system, void *stream = nullptr) {
        per_system.assign((size_t)nsys_, 0u);
        unsigned code = 0;
        const int rc = tprgb_plan_status(p_, per_system.data(), &code, stream);
        if (rc != TPRGB_OK && rc != TPRGB_ENONFINITE) check(rc);
        return rc;
    }

   private:
    int nsys_;
    tprgb_plan *p_ = nullptr;
};

// Continuous-batching server over a device arena.
class Server {
   public:
    explicit Server(size_t budget_bytes = size_t(8) << 30) {
        tprgb_server_opts o;
        check(tprgb_server_opts_default(&o));
        o.budget_bytes = budget_bytes;
        check(tprgb_server_create(&o, &s_));
    }
    explicit Server(const tprgb_server_opts &o) { check(tprgb_server_create(&o, &s_)); }
    Server(const Server &) = delete;
    Server &operator=(const Server &) = delete;
    ~Server() {
        if (s_) tprgb_server_destroy(s_);
    }
    // Host request: a..d stay valid until the request is done; x (may be
    // null) receives the FP64 solution.
    uint64_t submit(int nsys, const int *ns, const float *a, const float *b,
                    const float *c, const float *d, double *x) {
        uint64_t t = 0;
        check(tprgb_server_submit_host(s_, nsys, ns, a, b, c, d, x, &t));
        return t;
    }
    uint64_t submit_seeded(int nsys, const int *ns, const uint64_t *seeds,
                           int kind = 1 /* uneven */) {
        uint64_t t = 0;
        check(tprgb_server_submit_seeded(s_, nsys, ns, seeds, kind, &t));
        return t;
    }
    // Waits for the request; returns its status (TPRGB_ENONFINITE for a
    // request with a non-finite system) and fills info.
    int wait(uint64_t ticket, tprgb_request_info *info = nullptr, int timeout_ms = -1) {
        tprgb_request_info local;
        const int rc = tprgb_server_wait(s_, ticket, timeout_ms, info ? info : &local);
        if (rc != TPRGB_OK && rc != TPRGB_ENONFINITE) check(rc);
        return rc;
    }
    void fetch(uint64_t ticket, double *x_host) { check(tprgb_server_fetch(s_, ticket, x_host)); }
    void release(uint64_t ticket) { check(tprgb_server_release(s_, ticket)); }

   private:
    tprgb_server *s_ = nullptr;
};

}  // namespace tprgb

// Reference GPU free functions: host arrays, unit diagonal, synchronous.
// The reference returns silently on unsupported (n, s) (src/tpr.cu:575-579);
// these throw tprgb::Error.
namespace TPR_CU {
inline void tpr_cu(float *a, float *c, float *rhs, float *x, int n, int s) {
    tprgb::check(tprgb_tpr_cu_f32(a, c, rhs, x, n, s));
}
inline void cr_cu(float *a, float *c, float *rhs, float *x, int n) {
    tprgb::check(tprgb_cr_cu_f32(a, c, rhs, x, n));
}
inline void tpr_cu(double *a, double *c, double *rhs, double *x, int n,
                   int s) {
    tprgb::check(tprgb_tpr_cu_f64(a, c, rhs, x, n, s));
}
inline void cr_cu(double *a, double *c, double *rhs, double *x, int n) {
    tprgb::check(tprgb_cr_cu_f64(a, c, rhs, x, n));
}
}  // namespace TPR_CU

namespace PTPR_CU {
inline void ptpr_cu(float *a, float *c, float *rhs, float *x, int n, int s) {
    tprgb::check(tprgb_ptpr_cu_f32(a, c, rhs, x, n, s));
}
inline void pcr_cu(float *a, float *c, float *rhs, float *x, int n) {
    tprgb::check(tprgb_pcr_cu_f32(a, c, rhs, x, n));
}
inline void ptpr_cu(double *a, double *c, double *rhs, double *x, int n,
                    int s) {
    tprgb::check(tprgb_ptpr_cu_f64(a, c, rhs, x, n, s));
}
inline void pcr_cu(double *a, double *c, double *rhs, double *x, int n) {
    tprgb::check(tprgb_pcr_cu_f64(a, c, rhs, x, n));
}
}  // namespace PTPR_CU

#ifdef TPRGB_GLOBAL_NAMES
using tprgb::CR;
using tprgb::PCR;
using tprgb::PTPR;
using tprgb::TPR;
#endif
