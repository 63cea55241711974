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
