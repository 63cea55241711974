// C++ drop-in check: the reference's own test cases (test/examples.cpp,
// test/cuexamples.cpp) written against include/tpr_gb.hpp.
// usage: test_classes <ans1024.txt>   (1024 values, one per line)
// Prints one line per case and exits non-zero on the first failure.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#define TPRGB_GLOBAL_NAMES
#include "tpr_gb.hpp"

using real = tprgb_real;
static const int n = 1024;
static std::vector<real> ans(n);
static int failures = 0;

struct Fixed {  // src/system.cpp:118-130
    std::vector<real> a, diag, c, rhs;
    Fixed() : a(n), diag(n), c(n), rhs(n) { assign(); }
    void assign() {
        for (int i = 0; i < n; i++) {
            a[i] = -1.0 / 6.0;
            c[i] = -1.0 / 6.0;
            diag[i] = 1.0;
            rhs[i] = 1.0 * (i + 1);
        }
        a[0] = 0.0;
        c[n - 1] = 0.0;
    }
};

// tolerances of test/examples.cpp:36-56
static void expect_ans(const char *name, const std::vector<real> &x) {
    double maxsq = 0.0;
    bool ok = true;
    for (int i = 0; i < n; i++) {
        double d = std::fabs((double)ans[i] - (double)x[i]);
        if (!(d <= 1e-2)) ok = false;
        if (d * d > maxsq) maxsq = d * d;
    }
    if (!(maxsq <= 1e-3)) ok = false;
    printf("%-28s %s (max sq diff %.3e)\n", name, ok ? "ok" : "FAIL", maxsq);
    if (!ok) failures++;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    FILE *f = fopen(argv[1], "r");
    if (!f) return 2;
    for (int i = 0; i < n; i++) {
        double v;
        if (fscanf(f, "%lf", &v) != 1) return 2;
        ans[i] = (real)v;
    }
    fclose(f);

    try {
        {  // CRTest
            Fixed in;
            CR cr(in.a.data(), in.diag.data(), in.c.data(), in.rhs.data(), n);
            cr.solve();
            std::vector<real> x(n);
            cr.get_ans(x.data());
            expect_ans("CR", x);
        }
        {  // PCRTest
            Fixed in;
            PCR p(in.a.data(), in.diag.data(), in.c.data(), in.rhs.data(), n);
            p.solve();
            std::vector<real> x(n);
            p.get_ans(x.data());
            expect_ans("PCR", x);
        }
        for (int s = 4; s <= n; s *= 2) {  // TPRTest / PTPRTest
            Fixed in;
            std::vector<real> x(n);
            TPR t(in.a.data(), in.diag.data(), in.c.data(), in.rhs.data(), n, s);
            t.solve();
            t.get_ans(x.data());
            char name[64];
            snprintf(name, sizeof name, "TPR s=%d", s);
            expect_ans(name, x);
            PTPR p(in.a.data(), in.diag.data(), in.c.data(), in.rhs.data(), n, s);
            int flops = p.solve();
            p.get_ans(x.data());
            snprintf(name, sizeof name, "PTPR s=%d (flops %d)", s, flops);
            expect_ans(name, x);
        }
        for (int s = 64; s <= n; s *= 2) {  // CuExamples, test/cuexamples.cpp
            Fixed in;
            std::vector<real> x(n);
            TPR_CU::tpr_cu(in.a.data(), in.c.data(), in.rhs.data(), x.data(), n, s);
            char name[64];
            snprintf(name, sizeof name, "TPR_CU::tpr_cu s=%d", s);
            expect_ans(name, x);
            PTPR_CU::ptpr_cu(in.a.data(), in.c.data(), in.rhs.data(), x.data(), n, s);
            snprintf(name, sizeof name, "PTPR_CU::ptpr_cu s=%d", s);
            expect_ans(name, x);
        }
        {
            Fixed in;
            std::vector<real> x(n);
            TPR_CU::cr_cu(in.a.data(), in.c.data(), in.rhs.data(), x.data(), n);
            expect_ans("TPR_CU::cr_cu", x);
            PTPR_CU::pcr_cu(in.a.data(), in.c.data(), in.rhs.data(), x.data(), n);
            expect_ans("PTPR_CU::pcr_cu", x);
        }
        // *MultiThreadTest (test/examples.cpp:104-154): copies of one
        // solver on two threads agree
        for (int s = 4; s <= n; s *= 2) {
            PTPR proto(n, s);
            std::vector<Fixed> ins(2);
            std::vector<std::vector<real>> xs(2, std::vector<real>(n));
            std::vector<std::thread> th;
            for (int i = 0; i < 2; i++)
                th.emplace_back([&, i]() {
                    PTPR t(proto);
                    t.set_tridiagonal_system(ins[i].a.data(), ins[i].c.data(),
                                             ins[i].rhs.data());
                    t.solve();
                    t.get_ans(xs[i].data());
                });
            for (auto &t : th) t.join();
            bool same = xs[0] == xs[1];
            printf("PTPR multithread s=%-4d      %s\n", s, same ? "ok" : "FAIL");
            if (!same) failures++;
        }
        // unsupported sizes raise instead of exiting
        try {
            PTPR bad(1000, 8);
            printf("invalid n accepted FAIL\n");
            failures++;
        } catch (const tprgb::Error &e) {
            printf("invalid n -> error %d ok\n", e.code);
        }
    } catch (const tprgb::Error &e) {
        printf("unexpected error %d: %s\n", e.code, e.what());
        return 1;
    }
    printf("%s\n", failures ? "FAILED" : "ALL OK");
    return failures ? 1 : 0;
}
