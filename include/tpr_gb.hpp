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

#include <stdexcept>
#include <string>

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
