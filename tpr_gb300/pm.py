"""`tpr_pm`-compatible benchmark front end (src/pm.cpp:66-137, 140-268).

    python -m tpr_gb300.pm N S ITER SOLVER [OUTPUT]

SOLVER: tpr | ptpr | pcr | cr (reference-semantics GPU solvers through the
class surface, timed per solve with the host round trip included, as the
reference's CPU timers include get_ans), cutpr | cuptpr (the *_cu free
functions, host arrays in and out), cusparse (cuSPARSE gtsv2_nopivot,
device time of the solve as the reference's device timer measures it,
src/reference_cusparse.cu:166-205), batch (ITER systems in one launch of
the batched solver, FP32 + one refinement step).

Input per iteration: a = c = -1/6, diag = 1, rhs ~ U(-1, 1) (the
reference's ExampleRandomRHSInput, src/system.cpp:146-158), seeded.
Output: one line per iteration "n,s,solver,milliseconds" (the reference's
GPU format, src/pm.cpp:262-266); OUTPUT receives the last solution as
comma-separated values (src/lib.hpp:98-127).
"""
from __future__ import annotations

import sys
import time

import numpy as np

import tpr_gb300 as T

SOLVERS = ("tpr", "ptpr", "pcr", "cr", "cutpr", "cuptpr", "cusparse", "batch")


def _input(n, rng):
    a = np.full(n, -1.0 / 6.0, np.float32)
    c = np.full(n, -1.0 / 6.0, np.float32)
    a[0] = 0.0
    c[n - 1] = 0.0
    diag = np.ones(n, np.float32)
    rhs = rng.uniform(-1.0, 1.0, n).astype(np.float32)
    return a, diag, c, rhs


def run(n: int, s: int, iters: int, solver: str, out=None, seed: int = 0):
    solver = solver.lower()
    if solver not in SOLVERS:
        raise SystemExit(f"Solver Not Found: {solver}")
    rng = np.random.default_rng(seed)
    times, x = [], None
    if solver == "cusparse":
        import ctypes
        L = T.load()
        for _ in range(iters):
            a, diag, c, rhs = _input(n, rng)
            x = np.empty(n, np.float32)
            ms = ctypes.c_float()
            ptr = lambda v: v.ctypes.data_as(ctypes.c_void_p)
            T.check(L.tprgb_cusparse_gtsv(T.F32, n, ptr(a), ptr(diag), ptr(c),
                                          ptr(rhs), ptr(x), ctypes.byref(ms)))
            times.append(ms.value)
    elif solver == "batch":
        from . import batch as B
        from . import generate as G
        bt = G.batch(np.full(iters, n), seed, "dominant")
        t0 = time.perf_counter()
        xx = B.solve_host(bt, refine_steps=1)
        times = [(time.perf_counter() - t0) * 1e3 / iters] * iters
        x = xx[-n:]
    else:
        cls = {"tpr": T.TPR, "ptpr": T.PTPR, "pcr": T.PCR, "cr": T.CR}
        obj = None
        if solver in cls:
            obj = cls[solver](n, s) if solver in ("tpr", "ptpr") else \
                cls[solver](n)
        for _ in range(iters):
            a, diag, c, rhs = _input(n, rng)
            t0 = time.perf_counter()
            if obj is not None:
                obj.set_tridiagonal_system(a, c, rhs)
                obj.solve()
                x = obj.get_ans()
            elif solver == "cutpr":
                x = T.tpr_cu(a, c, rhs, n, s)
            else:
                x = T.ptpr_cu(a, c, rhs, n, s)
            times.append((time.perf_counter() - t0) * 1e3)
    for t in times:
        print(f"{n},{s},{solver},{t}")
    if out:
        with open(out, "w") as f:
            f.write(",".join(f"{v:f}" for v in np.asarray(x, np.float64)) + "\n")
    return times, x


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) < 4:
        sys.stderr.write("Usage: python -m tpr_gb300.pm n s iter solver "
                         "[destination for the result]\n")
        return 1
    run(int(argv[0]), int(argv[1]), int(argv[2]), argv[3],
        argv[4] if len(argv) > 4 else None)
    return 0


if __name__ == "__main__":
    sys.exit(main())
