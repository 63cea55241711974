// C entry points over the reference's PTPR class (src/ptpr.hpp:50-117),
// compiled together with the reference's own src/ptpr.cpp and src/pcr.cpp
// (PCR_SINGLE_THREAD, as src/CMakeLists.txt:69-75 builds them).
// TEST INFRASTRUCTURE ONLY: the result of this file is oracle/_ref/, the
// reference itself, used to pin the oracle restatement and as the
// reference-kind CPU baseline wherever the reference tree is present.
#include <omp.h>

#include <cstring>
#include <vector>

#include "ptpr.hpp"

extern "C" int ref_ptpr(int n, int s, real *a, real *c, real *rhs, real *x) {
    PTPR t(n, s);
    t.set_tridiagonal_system(a, c, rhs);
    int f = t.solve();
    t.get_ans(x);
    return f;
}

extern "C" int ref_ptpr_diag(int n, int s, real *a, real *diag, real *c,
                             real *rhs, real *x) {
    PTPR t(a, diag, c, rhs, n, s);
    int f = t.solve();
    t.get_ans(x);
    return f;
}

// OpenMP over independent systems with one private solver per thread (the
// firstprivate pattern of test/examples.cpp:130-154); the 4-argument setter
// normalises a private copy inside the timed region.
extern "C" void ref_batch_ptpr(int nsys, int n, int s, const real *a,
                               const real *b, const real *c, const real *d,
                               real *x, int nthreads) {
    omp_set_max_active_levels(1);
    PTPR proto(n, s);
#pragma omp parallel num_threads(nthreads) firstprivate(proto)
    {
        std::vector<real> wa(n), wb(n), wc(n), wr(n);
#pragma omp for schedule(static)
        for (int k = 0; k < nsys; k++) {
            size_t o = (size_t)k * (size_t)n;
            std::memcpy(wa.data(), a + o, sizeof(real) * n);
            std::memcpy(wb.data(), b + o, sizeof(real) * n);
            std::memcpy(wc.data(), c + o, sizeof(real) * n);
            std::memcpy(wr.data(), d + o, sizeof(real) * n);
            proto.set_tridiagonal_system(wa.data(), wb.data(), wc.data(),
                                         wr.data());
            proto.solve();
            proto.get_ans(x + o);
        }
    }
}

// The timed plain-solve loop of tpr_pm (src/pm.cpp:160-194): one solver,
// per iteration a fresh copy of the diag-normalised system (untimed: the
// solve overwrites it), the 3-argument setter, then solve() + get_ans()
// timed, with the solver's own OpenMP on nthreads threads.  Returns the
// seconds spent in solve + get_ans; x receives the last solution.
extern "C" double ref_time_plain_ptpr(int n, int s, const real *a, const real *c,
                                    const real *rhs, int iters, int nthreads,
                                    real *x) {
    omp_set_num_threads(nthreads > 0 ? nthreads : 1);
    PTPR t(n, s);
    std::vector<real> wa(n), wc(n), wr(n);
    double total = 0.0;
    for (int it = 0; it < iters; it++) {
        std::memcpy(wa.data(), a, sizeof(real) * n);
        std::memcpy(wc.data(), c, sizeof(real) * n);
        std::memcpy(wr.data(), rhs, sizeof(real) * n);
        t.set_tridiagonal_system(wa.data(), wc.data(), wr.data());
        double t0 = omp_get_wtime();
        t.solve();
        t.get_ans(x);
        total += omp_get_wtime() - t0;
    }
    return total;
}
