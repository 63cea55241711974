// C entry points over the reference's TPR class (src/tpr.hpp:44-112),
// compiled with the reference's src/tpr.cpp and src/cr.cpp (CR_SINGLE_THREAD,
// as src/CMakeLists.txt:60-66 builds them).
// TEST INFRASTRUCTURE ONLY (see shim_ptpr.cpp).
#include <omp.h>

#include <cstring>
#include <vector>

#include "tpr.hpp"

extern "C" int ref_tpr(int n, int s, real *a, real *c, real *rhs, real *x) {
    TPR t(n, s);
    t.set_tridiagonal_system(a, c, rhs);
    int f = t.solve();
    t.get_ans(x);
    return f;
}

extern "C" void ref_batch_tpr(int nsys, int n, int s, const real *a,
                              const real *b, const real *c, const real *d,
                              real *x, int nthreads) {
    omp_set_max_active_levels(1);
    TPR proto(n, s);
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
extern "C" double ref_time_plain_tpr(int n, int s, const real *a, const real *c,
                                    const real *rhs, int iters, int nthreads,
                                    real *x) {
    omp_set_num_threads(nthreads > 0 ? nthreads : 1);
    TPR t(n, s);
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
