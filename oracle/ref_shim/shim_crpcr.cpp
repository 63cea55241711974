// C entry points over the reference's standalone CR and PCR classes
// (src/cr.hpp:24-81, src/pcr.hpp:8-68), built from src/cr.cpp and
// src/pcr.cpp without the *_SINGLE_THREAD defines (libcr / libpcr,
// src/CMakeLists.txt:46-50).
// TEST INFRASTRUCTURE ONLY (see shim_ptpr.cpp).
#include "cr.hpp"
#include "pcr.hpp"

extern "C" int ref_cr(int n, real *a, real *c, real *rhs, real *x) {
    CR t(n);
    t.set_tridiagonal_system(a, nullptr, c, rhs);
    int f = t.solve();
    t.get_ans(x);
    return f;
}

extern "C" int ref_pcr(int n, real *a, real *c, real *rhs, real *x) {
    PCR t(n);
    t.set_tridiagonal_system(a, c, rhs);
    int f = t.solve();
    t.get_ans(x);
    return f;
}

extern "C" int ref_real_size(void) { return (int)sizeof(real); }
