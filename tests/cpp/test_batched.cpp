// C++ batched surface check (include/tpr_gb.hpp): HostPipeline, Plan and
// Server against an FP64 Thomas solve of the same FP32-stored systems,
// relative L2 error per system <= 1e-9 (the refined solver's bound).
// Prints one line per case and exits non-zero on the first failure.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <thread>
#include <vector>

#include "tpr_gb.hpp"

static int failures = 0;

struct Batch {
    std::vector<int> ns;
    std::vector<int64_t> off;
    std::vector<float> a, b, c, d;
    int64_t neq = 0;
};

// Diagonally dominant systems from a fixed linear congruential sequence:
// a, c ~ U(-1, 1) (a[0] = c[n-1] = 0), b = |a| + |c| + U(1, 2), d = A x_t.
static Batch make_batch(const std::vector<int> &ns, uint64_t seed) {
    Batch bt;
    bt.ns = ns;
    for (int n : ns) {
        bt.off.push_back(bt.neq);
        bt.neq += n;
    }
    bt.a.resize(bt.neq);
    bt.b.resize(bt.neq);
    bt.c.resize(bt.neq);
    bt.d.resize(bt.neq);
    uint64_t s = seed;
    auto u01 = [&]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return (double)(s >> 11) * (1.0 / 9007199254740992.0);
    };
    for (size_t k = 0; k < ns.size(); k++) {
        const int n = ns[k];
        const int64_t o = bt.off[k];
        std::vector<double> xt(n);
        for (int i = 0; i < n; i++) {
            float a = (float)(2 * u01() - 1), c = (float)(2 * u01() - 1);
            if (i == 0) a = 0.f;
            if (i == n - 1) c = 0.f;
            bt.a[o + i] = a;
            bt.c[o + i] = c;
            bt.b[o + i] = std::fabs(a) + std::fabs(c) + (float)(1 + u01());
            xt[i] = 2 * u01() - 1;
        }
        for (int i = 0; i < n; i++) {
            double v = (double)bt.b[o + i] * xt[i];
            if (i > 0) v += (double)bt.a[o + i] * xt[i - 1];
            if (i < n - 1) v += (double)bt.c[o + i] * xt[i + 1];
            bt.d[o + i] = (float)v;
        }
    }
    return bt;
}

// FP64 Thomas on the stored FP32 system; worst relative L2 error of x.
static double worst_error(const Batch &bt, const double *x) {
    double worst = 0.0;
    for (size_t k = 0; k < bt.ns.size(); k++) {
        const int n = bt.ns[k];
        const int64_t o = bt.off[k];
        std::vector<double> cp(n), dp(n), t(n);
        for (int i = 0; i < n; i++) {
            const double a = bt.a[o + i], b = bt.b[o + i], c = bt.c[o + i], d = bt.d[o + i];
            const double m = i ? b - a * cp[i - 1] : b;
            cp[i] = c / m;
            dp[i] = (i ? d - a * dp[i - 1] : d) / m;
        }
        t[n - 1] = dp[n - 1];
        for (int i = n - 2; i >= 0; i--) t[i] = dp[i] - cp[i] * t[i + 1];
        double num = 0.0, den = 0.0;
        for (int i = 0; i < n; i++) {
            num += (x[o + i] - t[i]) * (x[o + i] - t[i]);
            den += t[i] * t[i];
        }
        const double e = std::sqrt(num / den);
        if (!(e <= worst)) worst = e;  // NaN propagates
    }
    return worst;
}

static void expect(const char *name, double worst) {
    const bool ok = worst <= 1e-9;
    std::printf("%-40s worst rel-L2 %.3e %s\n", name, worst, ok ? "ok" : "FAIL");
    if (!ok) failures++;
}

// Uploads a batch, solves it on `stream` through the C++ wrapper, returns
// the worst error (1.0 when a call fails).  Device buffers are this call's.
static double device_solve(const Batch &bt, int n, const tprgb::BatchOptions &o,
                           cudaStream_t stream) {
    float *dv[4] = {};
    double *dx = nullptr;
    const size_t fb = sizeof(float) * (size_t)bt.neq;
    const std::vector<float> *hv[4] = {&bt.a, &bt.b, &bt.c, &bt.d};
    double worst = 1.0;
    bool ok = cudaMalloc(&dx, sizeof(double) * bt.neq) == cudaSuccess;
    for (int i = 0; i < 4 && ok; i++)
        ok = cudaMalloc(&dv[i], fb) == cudaSuccess &&
             cudaMemcpyAsync(dv[i], hv[i]->data(), fb, cudaMemcpyHostToDevice, stream) ==
                 cudaSuccess;
    if (ok) {
        try {
            tprgb::batch_solve((int)bt.ns.size(), n, dv[0], dv[1], dv[2], dv[3], dx, o, stream);
            std::vector<double> x(bt.neq);
            if (cudaMemcpyAsync(x.data(), dx, sizeof(double) * bt.neq, cudaMemcpyDeviceToHost,
                                stream) == cudaSuccess &&
                cudaStreamSynchronize(stream) == cudaSuccess)
                worst = worst_error(bt, x.data());
        } catch (const tprgb::Error &) {
        }
    }
    for (int i = 0; i < 4; i++) cudaFree(dv[i]);
    cudaFree(dx);
    return worst;
}

int main() {
    try {
        // first launches of four kernels at once from four host threads (the
        // launchers' one-time attribute and occupancy setup runs concurrently)
        {
            const int sizes[4] = {1024, 8192, 16384, 2048};
            const int nsys[4] = {64, 8, 4, 32};
            std::vector<Batch> bts;
            for (int i = 0; i < 4; i++)
                bts.push_back(make_batch(std::vector<int>(nsys[i], sizes[i]), 31 + i));
            double worst[4] = {1, 1, 1, 1};
            std::vector<std::thread> th;
            for (int i = 0; i < 4; i++)
                th.emplace_back([&, i]() {
                    cudaStream_t s = nullptr;
                    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
                        return;
                    worst[i] = device_solve(bts[i], sizes[i], tprgb::BatchOptions(), s);
                    cudaStreamDestroy(s);
                });
            for (auto &t : th) t.join();
            const char *names[4] = {"4 threads: first launch n=1024", "4 threads: first launch n=8192",
                                    "4 threads: first launch n=16384",
                                    "4 threads: first launch n=2048"};
            for (int i = 0; i < 4; i++) expect(names[i], worst[i]);
        }
        // uniform batch through the host pipeline (two calls, one context)
        {
            Batch bt = make_batch(std::vector<int>(300, 1024), 7);
            std::vector<double> x(bt.neq);
            tprgb::HostPipeline hp(int64_t(64) * 1024);
            for (int rep = 0; rep < 2; rep++) {
                hp.solve((int)bt.ns.size(), 1024, bt.a.data(), bt.b.data(), bt.c.data(),
                         bt.d.data(), x.data());
                expect("HostPipeline 300 x 1024", worst_error(bt, x.data()));
            }
        }
        // uneven plan on device buffers, graph replay
        {
            Batch bt = make_batch({64, 512, 4096, 16384, 128, 1024, 8192, 256}, 11);
            float *dv[4];
            double *dx;
            const size_t fb = sizeof(float) * (size_t)bt.neq;
            const std::vector<float> *hv[4] = {&bt.a, &bt.b, &bt.c, &bt.d};
            for (int i = 0; i < 4; i++) {
                if (cudaMalloc(&dv[i], fb) != cudaSuccess) throw tprgb::Error(-1, "cudaMalloc");
                cudaMemcpy(dv[i], hv[i]->data(), fb, cudaMemcpyHostToDevice);
            }
            if (cudaMalloc(&dx, sizeof(double) * bt.neq) != cudaSuccess)
                throw tprgb::Error(-1, "cudaMalloc");
            tprgb::Plan plan((int)bt.ns.size(), bt.off.data(), bt.ns.data());
            std::vector<double> x(bt.neq);
            for (int rep = 0; rep < 3; rep++) plan.execute(dv[0], dv[1], dv[2], dv[3], dx);
            std::vector<unsigned> st;
            const int rc = plan.status(st);
            cudaMemcpy(x.data(), dx, sizeof(double) * bt.neq, cudaMemcpyDeviceToHost);
            expect("Plan 8 sizes 64..16384", rc == TPRGB_OK ? worst_error(bt, x.data()) : 1.0);
            for (int i = 0; i < 4; i++) cudaFree(dv[i]);
            cudaFree(dx);
        }
        // serving loop: two host requests of mixed sizes
        {
            tprgb::Server srv(size_t(1) << 28);
            Batch b1 = make_batch({256, 1024, 8192}, 21), b2 = make_batch({2048, 512}, 22);
            std::vector<double> x1(b1.neq), x2(b2.neq);
            const uint64_t t1 = srv.submit((int)b1.ns.size(), b1.ns.data(), b1.a.data(),
                                           b1.b.data(), b1.c.data(), b1.d.data(), x1.data());
            const uint64_t t2 = srv.submit((int)b2.ns.size(), b2.ns.data(), b2.a.data(),
                                           b2.b.data(), b2.c.data(), b2.d.data(), x2.data());
            tprgb_request_info i1, i2;
            const int r1 = srv.wait(t1, &i1), r2 = srv.wait(t2, &i2);
            expect("Server request 1", r1 == TPRGB_OK ? worst_error(b1, x1.data()) : 1.0);
            expect("Server request 2", r2 == TPRGB_OK ? worst_error(b2, x2.data()) : 1.0);
            srv.release(t1);
            srv.release(t2);
        }
        // an invalid call throws tprgb::Error with the status code
        {
            bool threw = false;
            try {
                tprgb::batch_solve(1, 1000, nullptr, nullptr, nullptr, nullptr, nullptr);
            } catch (const tprgb::Error &e) {
                threw = e.code == TPRGB_EINVAL;
            }
            std::printf("%-40s %s\n", "batch_solve(n=1000) throws EINVAL", threw ? "ok" : "FAIL");
            if (!threw) failures++;
        }
    } catch (const tprgb::Error &e) {
        std::printf("error %d: %s\n", e.code, e.what());
        return 2;
    }
    if (failures) {
        std::printf("%d FAILED\n", failures);
        return 1;
    }
    std::printf("ALL OK\n");
    return 0;
}
