"""Measurements of the configurations other than bench.py's headline batch.

    python -m tpr_gb300.workloads [plain|one_launch|uneven|precision|all]

plain       one system, N=2048, S=512, FP32 (seed 42): PTPR and TPR through
            the class surface (host arrays in and out, like the reference's
            timed loop, src/pm.cpp:178-194) and the device-only kernel time;
            1000 solves (bench.py's line carries the same numbers beside the
            reference's CPU PTPR / TPR timed on the host cores).
one_launch  the plain one-launch-per-system FP32 path (reference-semantics
            PTPR kernel launched once per system) on 16384 x N=1024, S=128,
            against the batched refined solver on the same systems.
uneven      4096 systems, N = 2^k, k ~ U{6..16}, b = |a|+|c|+U(0.1,1),
            FP32 + 1 refinement, one persistent launch per step replayed from
            a CUDA graph.
precision   1024 systems, N = 32768, b = |a|+|c|+10^U(-4,-1), FP32 + 1
            refinement step (the row's 1-2 steps: one already meets 1e-9),
            beside two steps, the native FP64 residual and a plain FP64 GPU
            solve (reference-semantics PTPR in double); errors against FP64
            Thomas.

Each prints one JSON line: systems/s, algorithmic GB/s (24 B per equation
for refined solves, 20 B for plain FP32), fraction of the measured HBM peak,
and the worst per-system relative L2 error.
"""
from __future__ import annotations

import ctypes
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"])
    return 6800.0


def _oracle():
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    return O.port()


def _events(torch):
    return (torch.cuda.Event(enable_timing=True),
            torch.cuda.Event(enable_timing=True))


def plain(iters=1000):
    import tpr_gb300 as T
    from . import generate as G
    a, b, c, d, xt = G.one_system(2048, 42, "dominant")
    out = {"workload": "plain single system N=2048 S=512 FP32", "iters": iters}
    for cls, name in ((T.PTPR, "ptpr"), (T.TPR, "tpr")):
        t = cls(2048, 512)
        for _ in range(10):
            t.set_tridiagonal_system(a, b, c, d)
            t.solve()
            x = t.get_ans()
        t0 = time.perf_counter()
        for _ in range(iters):
            t.set_tridiagonal_system(a, b, c, d)
            t.solve()
            x = t.get_ans()
        dt = (time.perf_counter() - t0) / iters
        err = float(np.linalg.norm(x.astype(np.float64) - xt) /
                    np.linalg.norm(xt))
        # the same round trip timed in C++ (no Python per call), with the
        # 3-argument setter on the diag-normalised system (as tpr_pm
        # sets it) and with the 4-argument setter on the raw one
        L = T.load()
        h = t._h
        us3, us4 = ctypes.c_double(), ctypes.c_double()
        an3, cn3, rn3 = (np.ascontiguousarray((v / b).astype(np.float32)) for v in (a, c, d))
        xo = np.empty(2048, np.float32)
        ptr = lambda v: v.ctypes.data_as(ctypes.c_void_p)
        T.check(L.tprgb_time_roundtrip(h, ptr(an3), None, ptr(cn3), ptr(rn3), ptr(xo),
                                       iters, ctypes.byref(us3)))
        a4, b4, c4, d4 = (np.ascontiguousarray(v, np.float32) for v in (a, b, c, d))
        T.check(L.tprgb_time_roundtrip(h, ptr(a4), ptr(b4), ptr(c4), ptr(d4), ptr(xo),
                                       iters, ctypes.byref(us4)))
        out[name] = {"us_per_solve_host_round_trip": dt * 1e6,
                     "us_per_solve_round_trip_cxx_3arg": us3.value,
                     "us_per_solve_round_trip_cxx_4arg": us4.value,
                     "rel_l2_vs_xt": err}
    # device-only time of the fused kernel
    import torch
    L = T.load()
    an, cn, rn = (torch.from_numpy((v / b).astype(np.float32)).cuda()
                  for v in (a, c, d))
    x = torch.empty_like(an)
    s0, s1 = _events(torch)
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(10):
        L.tprgb_ref_solve_device(0, 1, 2048, 512, 0, an.data_ptr(),
                                 cn.data_ptr(), rn.data_ptr(), x.data_ptr(),
                                 None, 0, st)
    s0.record()
    for _ in range(iters):
        L.tprgb_ref_solve_device(0, 1, 2048, 512, 0, an.data_ptr(),
                                 cn.data_ptr(), rn.data_ptr(), x.data_ptr(),
                                 None, 0, st)
    s1.record()
    torch.cuda.synchronize()
    out["ptpr"]["us_per_solve_device"] = s0.elapsed_time(s1) * 1e3 / iters
    return out


def one_launch(nsys=16384, n=1024, s=128):
    import torch

    import tpr_gb300 as T
    from . import batch as B
    from . import generate as G
    L = T.load()
    bt = G.uniform_batch(nsys, n, 77, "dominant")
    dev = [torch.from_numpy(v).cuda() for v in (bt.a, bt.b, bt.c, bt.d)]
    norm = [torch.from_numpy((v / bt.b).astype(np.float32)).cuda()
            for v in (bt.a, bt.c, bt.d)]
    x32 = torch.empty(nsys * n, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    esz = 4

    def per_system():
        for k in range(nsys):
            o = k * n * esz
            L.tprgb_ref_solve_device(0, 1, n, s, 0, norm[0].data_ptr() + o,
                                     norm[1].data_ptr() + o,
                                     norm[2].data_ptr() + o,
                                     x32.data_ptr() + o, None, 0, st)

    per_system()
    torch.cuda.synchronize()
    s0, s1 = _events(torch)
    s0.record()
    per_system()
    s1.record()
    torch.cuda.synchronize()
    t_one = s0.elapsed_time(s1) * 1e-3
    x = torch.empty(nsys * n, dtype=torch.float64, device="cuda")
    o = B.opts(refine_steps=1)
    for _ in range(3):
        B.solve_into(x, *dev, n, o)
    s0.record()
    for _ in range(20):
        B.solve_into(x, *dev, n, o)
    s1.record()
    torch.cuda.synchronize()
    t_b = s0.elapsed_time(s1) * 1e-3 / 20
    port = _oracle()
    truth = port.batch_thomas(bt)
    e1, _ = port.batch_rel_l2(bt, x32.cpu().numpy(), truth)
    e2, _ = port.batch_rel_l2(bt, x.cpu().numpy(), truth)
    return {"workload": f"{nsys} x N={n} S={s}",
            "one_launch_per_system_fp32": {"systems_per_s": nsys / t_one,
                                           "rel_l2_max": e1},
            "batched_refined": {"systems_per_s": nsys / t_b, "rel_l2_max": e2},
            "speedup": t_one / t_b}


def uneven(nsys=4096, seed=2024):
    import torch

    from . import batch as B
    from . import generate as G
    ns = G.uneven_sizes(nsys, 6, 16, seed)
    bt = G.batch(ns, seed, "uneven")
    p = B.Plan(bt.ns, bt.offsets, refine_steps=1, graph=True)
    dev = [torch.from_numpy(v).cuda() for v in (bt.a, bt.b, bt.c, bt.d)]
    x = torch.empty(bt.neq, dtype=torch.float64, device="cuda")
    for _ in range(3):
        p.execute(x, *dev)
    torch.cuda.synchronize()
    s0, s1 = _events(torch)
    reps = 20
    s0.record()
    for _ in range(reps):
        p.execute(x, *dev)
    s1.record()
    torch.cuda.synchronize()
    t = s0.elapsed_time(s1) * 1e-3 / reps
    rc, st, code = p.status()
    port = _oracle()
    worst, _ = port.batch_rel_l2(bt, x.cpu().numpy(), port.batch_thomas(bt))
    gbs = 24 * bt.neq / t / 1e9
    return {"workload": f"uneven {nsys} systems N=2^U{{6..16}} "
                        f"({bt.neq} eq), FP32 + 1 refinement, CUDA graph",
            "systems_per_s": nsys / t, "ms_per_step": t * 1e3,
            "gb_per_s": gbs, "frac_of_peak": gbs / _peak(),
            "rel_l2_max": worst, "status": rc, "plan": p.info()}


def precision(nsys=1024, n=32768, steps=1):
    """The precision-stress row: FP32 solve + `steps` compensated refinement
    steps through a plan (CUDA graph) and through the uniform batch API
    (one thread-block cluster per system); beside it the same kernel with
    the other step count (2 when steps is 1), with the native FP64 residual,
    and the plain FP64 GPU solve.  Every result's worst relative L2 error
    against FP64 Thomas of the FP32-stored systems."""
    import torch

    import tpr_gb300 as T
    from . import batch as B
    from . import generate as G
    bt = G.uniform_batch(nsys, n, 5150, "weak")
    dev = [torch.from_numpy(v).cuda() for v in (bt.a, bt.b, bt.c, bt.d)]
    x = torch.empty(bt.neq, dtype=torch.float64, device="cuda")
    port = _oracle()
    truth = port.batch_thomas(bt)
    reps = 5
    s0, s1 = _events(torch)

    def timed(launch):
        for _ in range(2):
            launch()
        torch.cuda.synchronize()
        s0.record()
        for _ in range(reps):
            launch()
        s1.record()
        torch.cuda.synchronize()
        t = s0.elapsed_time(s1) * 1e-3 / reps
        worst, _ = port.batch_rel_l2(bt, x.cpu().numpy(), truth)
        gbs = 24 * bt.neq / t / 1e9
        return {"systems_per_s": nsys / t, "gb_per_s": gbs,
                "frac_of_peak": gbs / _peak(), "rel_l2_max_vs_thomas": worst}

    p = B.Plan(bt.ns, bt.offsets, refine_steps=steps, graph=True)
    main_row = timed(lambda: p.execute(x, *dev))
    p.close()
    uni = timed(lambda: B.solve_into(x, *dev, n, B.opts(refine_steps=steps)))
    uni["tile"] = list(B.tile_for(n))
    other = 2 if steps == 1 else 1
    alt = timed(lambda: B.solve_into(x, *dev, n, B.opts(refine_steps=other)))
    f64 = timed(lambda: B.solve_into(x, *dev, n, B.opts(refine_steps=steps,
                                                       residual=B.RESID_F64)))
    # plain FP64 GPU solve of the same systems (reference-semantics PTPR)
    L = T.load()
    b64 = bt.b.astype(np.float64)
    norm = [torch.from_numpy(v.astype(np.float64) / b64).cuda()
            for v in (bt.a, bt.c, bt.d)]
    sz = ctypes.c_size_t()
    T.check(L.tprgb_ref_workspace_bytes(0, nsys, n, 256, 1, ctypes.byref(sz)))
    work = torch.empty(max(sz.value, 1), dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    s0.record()
    T.check(L.tprgb_ref_solve_device(0, nsys, n, 256, 1, norm[0].data_ptr(),
                                     norm[1].data_ptr(), norm[2].data_ptr(),
                                     x.data_ptr(), work.data_ptr(),
                                     sz.value, st))
    s1.record()
    torch.cuda.synchronize()
    t64 = s0.elapsed_time(s1) * 1e-3
    w64, _ = port.batch_rel_l2(bt, x.cpu().numpy(), truth)
    out = {"workload": f"precision stress {nsys} x N={n}, weakly dominant, "
                       f"FP32 + {steps} refinement step(s), plan + CUDA graph"}
    out.update(main_row)
    out.update({"uniform_batch_api": uni,
                f"uniform_batch_api_{other}_steps": alt,
                "native_fp64_residual": f64,
                "plain_fp64_gpu": {"systems_per_s": nsys / t64,
                                   "rel_l2_max_vs_thomas": w64}})
    return out


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    which = argv[0] if argv else "all"
    from . import autotune
    autotune.apply()
    todo = ["plain", "one_launch", "uneven", "precision"] if which == "all" \
        else [which]
    for name in todo:
        print(json.dumps({name: globals()[name]()}), flush=True)


if __name__ == "__main__":
    main()
