"""Batched hierarchical solver against the FP64 Thomas oracle (FP32-stored
systems).  Tolerances: plain FP32 solve <= 1e-5 relative L2 per system;
with refinement <= 1e-9 (the accuracy target of the refined solver)."""
import ctypes

import numpy as np
import pytest

import tpr_gb300 as T
from tpr_gb300 import batch as B
from tpr_gb300 import generate as G

pytestmark = pytest.mark.gpu


def _err(port, bt, x):
    truth = port.batch_thomas(bt)
    worst, per = port.batch_rel_l2(bt, x, truth)
    return worst, per


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512, 1024, 2048, 4096,
                               8192])
@pytest.mark.parametrize("L", [4, 8])
def test_plain_fp32_all_sizes(cuda, port, n, L):
    if n < 2 * L or n // L > 1024:
        pytest.skip("tile does not cover this size")
    nt = max(128, min(1024, n // L))
    bt = G.uniform_batch(37, n, 1000 + n, "uneven")
    x = B.solve_host(bt, refine_steps=0, x_f64=False, eq_per_thread=L,
                     threads_per_cta=nt)
    assert x.dtype == np.float32
    worst, _ = _err(port, bt, x)
    assert worst <= 1e-5, worst


@pytest.mark.parametrize("n", [64, 1024, 8192])
@pytest.mark.parametrize("resid", [B.RESID_DF, B.RESID_F64])
def test_refined_reaches_1e9(cuda, port, n, resid):
    bt = G.uniform_batch(29, n, 2000 + n, "uneven")
    x = B.solve_host(bt, refine_steps=1, residual=resid)
    assert x.dtype == np.float64
    worst, _ = _err(port, bt, x)
    assert worst <= 1e-9, worst


@pytest.mark.parametrize("steps", [1, 2, 3])
def test_weakly_dominant_refinement_steps(cuda, port, steps):
    """Precision-stress generator (cond up to ~1e4): each step contracts
    the error; two steps reach 1e-9."""
    bt = G.uniform_batch(16, 4096, 77, "weak")
    errs = []
    for k in range(steps + 1):
        x = B.solve_host(bt, refine_steps=k)
        errs.append(_err(port, bt, x)[0])
    assert all(errs[i + 1] < errs[i] or errs[i + 1] < 1e-12
               for i in range(steps))
    if steps >= 2:
        assert errs[2] <= 1e-9, errs


def test_uniform_configs_shape_sample(cuda, port):
    """The ADI-style uniform batch shape (N=1024) on a sample of systems,
    every tile shape giving the same accuracy."""
    bt = G.uniform_batch(300, 1024, 5, "dominant")
    for L, nt in ((4, 256), (4, 512), (8, 128), (8, 256), (8, 1024)):
        x = B.solve_host(bt, refine_steps=1, eq_per_thread=L,
                         threads_per_cta=nt)
        worst, _ = _err(port, bt, x)
        assert worst <= 1e-9, (L, nt, worst)


def test_result_independent_of_batch_position(cuda):
    """A system's solution does not depend on which CTA / slot solved it."""
    bt = G.uniform_batch(10, 256, 9, "uneven")
    x_all = B.solve_host(bt, refine_steps=1)
    for k in (0, 3, 9):
        one = G.Batch([256], *[v[k * 256:(k + 1) * 256] for v in
                               (bt.a, bt.b, bt.c, bt.d, bt.xt)])
        x1 = B.solve_host(one, refine_steps=1)
        np.testing.assert_array_equal(x1, x_all[k * 256:(k + 1) * 256])


def test_rejects_bad_arguments(cuda):
    import tpr_gb300 as T
    torch = cuda
    a = torch.zeros(1000, device="cuda")
    with pytest.raises(T.TprError):
        B.solve(a, a, a, a, 1000)  # not a power of two
    a = torch.zeros(1 << 15, device="cuda")
    with pytest.raises(T.TprError):
        B.solve(a, a, a, a, 1 << 15, eq_per_thread=8, threads_per_cta=256)


@pytest.mark.parametrize("n", [16, 64, 256, 1024, 4096])
@pytest.mark.parametrize("L,nt", [(4, 256), (4, 512), (8, 256), (8, 512)])
def test_staged_kernel_matches_register_kernel(cuda, port, n, L, nt):
    """The TMA-staged variant computes the same bits as the register
    variant (same arithmetic, different data path) and meets 1e-9; the
    batch ends in a partial tile."""
    if n < 2 * L or n // L > nt:
        pytest.skip("tile does not cover this size")
    nsys = 3 * (nt * L // n) + 1
    bt = G.uniform_batch(nsys, n, 31 + n, "uneven")
    xs = B.solve_host(bt, refine_steps=1, eq_per_thread=L, threads_per_cta=nt,
                      variant=B.STAGED)
    xr = B.solve_host(bt, refine_steps=1, eq_per_thread=L, threads_per_cta=nt,
                      variant=B.REGISTERS)
    np.testing.assert_array_equal(xs, xr)
    worst, _ = _err(port, bt, xs)
    assert worst <= 1e-9, worst
    xp = B.solve_host(bt, refine_steps=0, x_f64=False, eq_per_thread=L,
                      threads_per_cta=nt, variant=B.STAGED)
    worst, _ = _err(port, bt, xp)
    assert worst <= 1e-5, worst
    import ctypes
    code = ctypes.c_uint()
    assert B.load().tprgb_batch_status(ctypes.byref(code), 1) == 0
    assert code.value == 0


@pytest.mark.parametrize("n", [32, 64, 256, 1024, 4096])
@pytest.mark.parametrize("L,nt", [(8, 64), (8, 128), (8, 256), (16, 64),
                                  (16, 128), (16, 256)])
def test_swizzled_kernel(cuda, port, n, L, nt):
    """Tensor-map staging with the 128-byte swizzle: with 8 equations per
    thread the same bits as the register variant; with 16 the refined
    solution meets 1e-9 and the plain one 1e-5; one and two stages agree
    bit for bit; the batch ends in a partial tile."""
    if n < 2 * L or n // L > nt:
        pytest.skip("tile does not cover this size")
    nsys = 3 * (nt * L // n) + 1
    bt = G.uniform_batch(nsys, n, 57 + n, "uneven")
    xs = B.solve_host(bt, refine_steps=1, eq_per_thread=L, threads_per_cta=nt,
                      variant=B.SWIZZLED)
    x1 = B.solve_host(bt, refine_steps=1, eq_per_thread=L, threads_per_cta=nt,
                      variant=B.SWIZZLED_ONE)
    np.testing.assert_array_equal(xs, x1)
    if L == 8 and nt >= 128:
        xr = B.solve_host(bt, refine_steps=1, eq_per_thread=L,
                          threads_per_cta=nt, variant=B.REGISTERS)
        np.testing.assert_array_equal(xs, xr)
    worst, _ = _err(port, bt, xs)
    assert worst <= 1e-9, worst
    xp = B.solve_host(bt, refine_steps=0, x_f64=False, eq_per_thread=L,
                      threads_per_cta=nt, variant=B.SWIZZLED)
    worst, _ = _err(port, bt, xp)
    assert worst <= 1e-5, worst
    import ctypes
    code = ctypes.c_uint()
    assert B.load().tprgb_batch_status(ctypes.byref(code), 1) == 0
    assert code.value == 0


def test_swizzled_rejects_bad_tiles(cuda):
    bt = G.uniform_batch(4, 16, 3, "dominant")
    with pytest.raises(T.TprError):   # n < 32
        B.solve_host(bt, eq_per_thread=8, threads_per_cta=64,
                     variant=B.SWIZZLED)
    bt = G.uniform_batch(4, 64, 3, "dominant")
    with pytest.raises(T.TprError):   # 512 threads
        B.solve_host(bt, eq_per_thread=8, threads_per_cta=512,
                     variant=B.SWIZZLED)
    with pytest.raises(T.TprError):   # FP64 residual
        B.solve_host(bt, eq_per_thread=8, threads_per_cta=64,
                     variant=B.SWIZZLED, residual=B.RESID_F64)


@pytest.mark.parametrize("n,nt,nsys", [(2048, 64, 5), (4096, 128, 3),
                                       (8192, 64, 9), (16384, 256, 4),
                                       (16384, 64, 100), (32768, 256, 3),
                                       (65536, 256, 40), (16384, 512, 7),
                                       (65536, 512, 10)])
def test_cluster_kernel(cuda, port, n, nt, nsys):
    """One system per thread-block cluster (P = n / (16 nt) CTAs, boundary
    rows exchanged in distributed shared memory): refined solutions meet
    1e-9 and plain FP32 1e-5 against FP64 Thomas; batches with more systems
    than resident clusters walk the grid-stride loop."""
    bt = G.uniform_batch(nsys, n, 91 + n + nt, "uneven")
    xs = B.solve_host(bt, refine_steps=1, eq_per_thread=16, threads_per_cta=nt,
                      variant=B.CLUSTER)
    worst, _ = _err(port, bt, xs)
    assert worst <= 1e-9, worst
    x2 = B.solve_host(bt, refine_steps=2, eq_per_thread=16, threads_per_cta=nt,
                      variant=B.CLUSTER)
    worst2, _ = _err(port, bt, x2)
    assert worst2 <= 1e-9, worst2
    xp = B.solve_host(bt, refine_steps=0, x_f64=False, eq_per_thread=16,
                      threads_per_cta=nt, variant=B.CLUSTER)
    worst, _ = _err(port, bt, xp)
    assert worst <= 1e-5, worst
    # native FP64 residual (x accumulated in FP64)
    xd = B.solve_host(bt, refine_steps=1, residual=B.RESID_F64, eq_per_thread=16,
                      threads_per_cta=nt, variant=B.CLUSTER)
    worst, _ = _err(port, bt, xd)
    assert worst <= 1e-9, worst
    import ctypes
    code = ctypes.c_uint()
    assert B.load().tprgb_batch_status(ctypes.byref(code), 1) == 0
    assert code.value == 0


def test_cluster_default_and_rejects(cuda, port):
    """Above 8192 equations the default tile is the cluster variant (with
    either residual); sizes that need more than 16 or fewer than 2 CTAs are
    refused."""
    bt = G.uniform_batch(2, 32768, 5, "dominant")
    x = B.solve_host(bt, refine_steps=1)
    worst, _ = _err(port, bt, x)
    assert worst <= 1e-9, worst
    x = B.solve_host(bt, refine_steps=1, residual=B.RESID_F64)
    worst, _ = _err(port, bt, x)
    assert worst <= 1e-9, worst
    with pytest.raises(T.TprError):   # 32 CTAs of 2048
        B.solve_host(G.uniform_batch(1, 65536, 5, "dominant"),
                     eq_per_thread=16, threads_per_cta=128, variant=B.CLUSTER)
    with pytest.raises(T.TprError):   # one CTA
        B.solve_host(G.uniform_batch(2, 1024, 5, "dominant"),
                     eq_per_thread=16, threads_per_cta=64, variant=B.CLUSTER)


@pytest.mark.parametrize("steps,resid", [(1, B.RESID_DF), (2, B.RESID_DF),
                                         (2, B.RESID_F64)])
def test_cluster_precision_stress_shape(cuda, port, steps, resid):
    """The precision-stress generator (weakly dominant, condition numbers up
    to about 1e4) at N = 32768 on the cluster kernel: one or two refinement
    steps reach 1e-9 with either residual."""
    bt = G.uniform_batch(6, 32768, 5150, "weak")
    x = B.solve_host(bt, refine_steps=steps, residual=resid)
    worst, _ = _err(port, bt, x)
    assert worst <= 1e-9, worst


@pytest.mark.parametrize("n,nsys,L,nt,v", [
    (32, 1, 8, 64, B.SWIZZLED),        # smallest swizzled size, one system
    (1024, 1, 16, 64, B.SWIZZLED_ONE),  # one system, one CTA
    (512, 3, 16, 256, B.SWIZZLED),      # fewer systems than one tile holds
    (4096, 1, 16, 128, B.CLUSTER),      # one system, one cluster of 2
    (65536, 1, 16, 256, B.CLUSTER),     # one system, one cluster of 16
])
def test_small_batches_edge_tiles(cuda, port, n, nsys, L, nt, v):
    bt = G.uniform_batch(nsys, n, 300 + n + nsys, "uneven")
    x = B.solve_host(bt, refine_steps=1, eq_per_thread=L, threads_per_cta=nt,
                     variant=v)
    worst, _ = _err(port, bt, x)
    assert worst <= 1e-9, worst


@pytest.mark.parametrize("v,n,L,nt", [(B.SWIZZLED, 1024, 16, 64),
                                     (B.CLUSTER, 4096, 16, 128), (0, 4096, 0, 0)])
def test_empty_batch_is_a_no_op(cuda, v, n, L, nt):
    o = B.opts(refine_steps=1, eq_per_thread=L, threads_per_cta=nt, variant=v)
    rc = B.load().tprgb_batch_solve(0, n, None, None, None, None, None,
                                    ctypes.byref(o), None)
    assert rc == 0


@pytest.mark.parametrize("nsys,chunk_systems", [(300, 32), (40, 32), (7, 64)])
def test_host_pipeline_matches_device_solve(cuda, nsys, chunk_systems):
    """tprgb_batch_solve_host (host arrays, chunks ramped 1/8, 1/4, 1/2 of a
    full chunk at both ends over three streams; small batches in equal
    chunks) gives the same bits as the device-resident solve, with the four
    arrays separate, in one block at equal spacing (one 2D upload per
    chunk, pinned or pageable) and in one block at unequal spacing."""
    import torch
    n = 1024
    bt = G.uniform_batch(nsys, n, 4242 + nsys, "uneven")
    want = B.solve_host(bt, refine_steps=1)
    pin = [torch.from_numpy(v).pin_memory() for v in (bt.a, bt.b, bt.c, bt.d)]
    x = torch.zeros(nsys * n, dtype=torch.float64).pin_memory()
    ctx = B.HostContext(chunk_eq=chunk_systems * n)
    for _ in range(2):   # repeated calls reuse the context
        x.zero_()
        ctx.solve(nsys, n, *pin, x, B.opts(refine_steps=1))
        np.testing.assert_array_equal(x.numpy(), want)
    # a, b, c, d one after the other in one block (pinned, then pageable):
    # each chunk uploads with one 2D copy; same bits
    neq = nsys * n
    blk = torch.empty(4 * neq, dtype=torch.float32).pin_memory()
    for i, v in enumerate((bt.a, bt.b, bt.c, bt.d)):
        blk[i * neq:(i + 1) * neq].copy_(torch.from_numpy(v))
    for block in (blk, blk.numpy().copy()):
        views = [block[i * neq:(i + 1) * neq] for i in range(4)]
        x.zero_()
        ctx.solve(nsys, n, *views, x, B.opts(refine_steps=1))
        np.testing.assert_array_equal(x.numpy(), want)
    # one block at unequal spacing: four copies per chunk, same bits
    gaps = (0, neq + 16, 2 * neq + 48, 3 * neq + 64)
    blk2 = np.zeros(4 * neq + 64, dtype=np.float32)
    views = [blk2[g:g + neq] for g in gaps]
    for v, src in zip(views, (bt.a, bt.b, bt.c, bt.d)):
        v[:] = src
    x.zero_()
    ctx.solve(nsys, n, *views, x, B.opts(refine_steps=1))
    np.testing.assert_array_equal(x.numpy(), want)


def test_host_pipeline_async_calls_pipeline_correctly(cuda):
    """Asynchronous host calls queued back to back (different inputs,
    different outputs, the ring shared across calls) give each batch the
    device solve's bits once the context is waited on."""
    bts = [G.uniform_batch(300, 1024, 70 + i, "dominant") for i in range(3)]
    ctx = B.HostContext(chunk_eq=32 * 1024)
    try:
        o = B.opts(refine_steps=1)
        outs = [np.empty(300 * 1024, np.float64) for _ in bts]
        for bt, x in zip(bts, outs):
            ctx.solve_async(300, 1024, bt.a, bt.b, bt.c, bt.d, x, o)
        ctx.wait()
        for bt, x in zip(bts, outs):
            ref = B.solve_host(bt, refine_steps=1)
            np.testing.assert_array_equal(x, ref)
    finally:
        ctx.close()
