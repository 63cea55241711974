"""Reference-semantics GPU path against the oracle: the reference's own
outputs (tests/golden) bit for bit, the reference's known answer with its
tolerances, and the C restatement on fresh inputs.  Calls go through the C
ABI (tpr_gb300 is a ctypes layer over it)."""
import ctypes

import numpy as np
import pytest

import tpr_gb300 as T
from tpr_gb300 import generate as G

pytestmark = pytest.mark.gpu
SWEEP = [4, 8, 16, 32, 64, 128, 256, 512, 1024]


def _kat(ans, x):
    x = np.asarray(x, np.float64)
    assert np.all(np.abs(x - ans) <= 1e-2)
    assert np.max((x - ans) ** 2) <= 1e-3


def _bits_equal(x, y):
    """Bit-identical, except that any NaN equals any NaN (CUDA produces the
    canonical 0x7fffffff NaN, x86 the negative quiet NaN)."""
    x = np.asarray(x)
    y = np.asarray(y)
    assert x.dtype == y.dtype and x.shape == y.shape
    nx, ny = np.isnan(x), np.isnan(y)
    np.testing.assert_array_equal(nx, ny)
    u = np.uint32 if x.dtype == np.float32 else np.uint64
    np.testing.assert_array_equal(x[~nx].view(u), y[~ny].view(u))


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_fixed_system_classes(cuda, golden, ans1024, prec):
    """test/examples.cpp:59-102 and test/cuexamples.cpp:49-83 cases."""
    dt = np.float32 if prec == "f32" else np.float64
    a, diag, c, rhs = [v.astype(dt) for v in G.fixed_system(1024)]
    for cls, key in ((T.CR, "cr"), (T.PCR, "pcr")):
        t = cls(1024, dtype=dt)
        t.set_tridiagonal_system(a, diag, c, rhs)
        assert t.solve() > 0
        x = np.zeros(1024, dt)
        assert t.get_ans(x) == 0
        _bits_equal(x, golden[f"fixed_{key}_{prec}"])
        _kat(ans1024, x)
    for s in SWEEP:
        for cls, key in ((T.PTPR, "ptpr"), (T.TPR, "tpr")):
            t = cls(1024, s, dtype=dt)
            t.set_tridiagonal_system(a, diag, c, rhs)
            t.solve()
            x = t.get_ans()
            _bits_equal(x, golden[f"fixed_{key}_s{s}_{prec}"])
            _kat(ans1024, x)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_large_cr_pcr_objects(cuda, port, prec):
    """CR / PCR objects and cr_cu / pcr_cu above one CTA's shared memory
    (n = 32768, no size cap, as the reference's CPU classes): the handle
    allocates the workspace; same bits as the C restatement."""
    dt = np.float32 if prec == "f32" else np.float64
    n = 1 << 15
    a, b, c, d, _ = G.one_system(n, 5, "uneven")
    an, cn, rn = port.normalize(a, b, c, d, dt)
    _bits_equal(T.cr_cu(an, cn, rn, n, dt), port.cr(an, cn, rn, dt)[0])
    _bits_equal(T.pcr_cu(an, cn, rn, n, dt), port.pcr(an, cn, rn, dt)[0])
    t = T.PCR(n, dtype=dt)
    t.set_tridiagonal_system(an, np.ones(n, dt), cn, rn)
    assert t.solve() == 14 * n * 15  # src/pcr.cpp:88
    _bits_equal(t.get_ans(), port.pcr(an, cn, rn, dt)[0])


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_fixed_system_free_functions(cuda, golden, ans1024, prec):
    dt = np.float32 if prec == "f32" else np.float64
    a, _, c, rhs = [v.astype(dt) for v in G.fixed_system(1024)]
    _bits_equal(T.cr_cu(a, c, rhs, 1024, dt), golden[f"fixed_cr_{prec}"])
    _bits_equal(T.pcr_cu(a, c, rhs, 1024, dt), golden[f"fixed_pcr_{prec}"])
    for s in (64, 128, 256, 512, 1024):  # test/cuexamples.cpp:73-83
        x = T.ptpr_cu(a, c, rhs, 1024, s, dt)
        _bits_equal(x, golden[f"fixed_ptpr_s{s}_{prec}"])
        _kat(ans1024, x)
        x = T.tpr_cu(a, c, rhs, 1024, s, dt)
        _bits_equal(x, golden[f"fixed_tpr_s{s}_{prec}"])
        _kat(ans1024, x)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("s", [64, 128, 256, 512, 1024, 2048])
def test_plain_system_bitwise(cuda, golden, prec, s):
    """The plain single-system workload (N=2048, seed 42), 4-arg setter on
    the device, against the reference CPU PTPR / TPR."""
    dt = np.float32 if prec == "f32" else np.float64
    a, b, c, d, xt = G.one_system(2048, 42, "dominant")
    a, b, c, d = [v.astype(dt) for v in (a, b, c, d)]
    for cls, key in ((T.PTPR, "ptpr"), (T.TPR, "tpr")):
        t = cls(2048, s, dtype=dt)
        t.set_tridiagonal_system(a, b, c, d)
        t.solve()
        x = t.get_ans()
        ref = golden[f"plain_{key}_s{s}_{prec}"]
        _bits_equal(x, ref)
        err = np.linalg.norm(x.astype(np.float64) - ref) / np.linalg.norm(ref)
        assert err <= (1e-5 if prec == "f32" else 1e-12)


@pytest.mark.parametrize("k", range(1, 21))
def test_nstab_fixtures(cuda, golden, nstab, k):
    a, diag, c, rhs = [v.astype(np.float32) for v in nstab[f"eq{k}"]]
    for s in (16, 64, 512):
        for cls, key in ((T.PTPR, "ptpr"), (T.TPR, "tpr")):
            t = cls(512, s)
            t.set_tridiagonal_system(a, diag, c, rhs)
            t.solve()
            _bits_equal(t.get_ans(), golden[f"nstab_eq{k}_{key}_s{s}_f32"])


def _device_batch(torch, nsys, n, dt, seed):
    bt = G.uniform_batch(nsys, n, seed, "uneven")
    tdt = torch.float32 if dt == np.float32 else torch.float64
    norm = [bt.a / bt.b, bt.c / bt.b, bt.d / bt.b]
    if dt == np.float32:
        norm = [(v.astype(np.float32)) for v in
                (bt.a / bt.b, bt.c / bt.b, bt.d / bt.b)]
    dev = [torch.from_numpy(np.ascontiguousarray(v, dt)).to("cuda", tdt)
           for v in norm]
    return bt, norm, dev


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("kind,n,s", [(0, 1024, 128), (1, 1024, 128),
                                      (0, 32768, 256), (1, 32768, 256),
                                      (0, 65536, 1024), (1, 16384, 64),
                                      (2, 2048, 0), (3, 2048, 0),
                                      (2, 8192, 0), (3, 8192, 0),
                                      (2, 65536, 0), (3, 65536, 0)])
def test_device_batched_vs_port(cuda, port, prec, kind, n, s):
    """Several systems per launch, fused and sliced shapes, against the C
    restatement (bit for bit).  Standalone CR / PCR run in one CTA's
    shared memory up to n = 8192 (FP32) / 4096 (FP64) and level by level
    over a global workspace above: 8192 covers both sides of the FP64
    switch, 65536 the multi-launch CR levels (two before and after the
    one-CTA tail)."""
    torch = cuda
    dt = np.float32 if prec == "f32" else np.float64
    nsys = 3
    bt, norm, (da, dc, dr) = _device_batch(torch, nsys, n, dt, 100 + n)
    dx = torch.empty_like(da)
    L = T.load()
    sz = ctypes.c_size_t()
    T.check(L.tprgb_ref_workspace_bytes(kind, nsys, n, s or n,
                                        T.F32 if prec == "f32" else T.F64,
                                        ctypes.byref(sz)))
    work = torch.empty(max(1, sz.value), dtype=torch.uint8, device="cuda")
    T.check(L.tprgb_ref_solve_device(
        kind, nsys, n, s or n, T.F32 if prec == "f32" else T.F64,
        da.data_ptr(), dc.data_ptr(), dr.data_ptr(), dx.data_ptr(),
        work.data_ptr() if sz.value else None, sz.value,
        torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    x = dx.cpu().numpy()
    for k in range(nsys):
        sl = slice(k * n, (k + 1) * n)
        a, c, r = norm[0][sl], norm[1][sl], norm[2][sl]
        if kind == 0:
            xr, _ = port.ptpr(a, c, r, s, dt)
        elif kind == 1:
            xr, _ = port.tpr(a, c, r, s, dt)
        elif kind == 2:
            xr, _ = port.cr(a, c, r, dt)
        else:
            xr, _ = port.pcr(a, c, r, dt)
        _bits_equal(x[sl], xr)


EDGE_SHAPES = [(2, 2), (4, 2), (8, 2), (8, 8), (16, 2), (32, 2), (64, 2),
               (64, 4), (1024, 2), (4096, 2), (32768, 4), (65536, 8)]


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("kind", [0, 1])
def test_edge_shapes_vs_port(cuda, port, prec, kind):
    """The smallest slices and systems (s = 2, n = s, n = 2), one-launch
    cluster shapes (2 <= n / s <= 16), one-CTA shapes with a long reduced
    system (m = 512 at s = 2), and the sliced path at its largest reduced
    system (m = 8192, which FP64 rejects as more than one CTA's shared
    memory): same bits as the C restatement, through the batched device
    entry point and through the *_cu host functions."""
    torch = cuda
    dt = np.float32 if prec == "f32" else np.float64
    L = T.load()
    pr = T.F32 if prec == "f32" else T.F64
    cu = T.ptpr_cu if kind == 0 else T.tpr_cu
    for n, s in EDGE_SHAPES:
        nsys = 2
        bt, norm, (da, dc, dr) = _device_batch(torch, nsys, n, dt, 300 + n + s)
        sz = ctypes.c_size_t()
        rc = L.tprgb_ref_workspace_bytes(kind, nsys, n, s, pr, ctypes.byref(sz))
        if rc == T.EUNSUPPORTED:
            assert prec == "f64" and n // s == 8192, (n, s)
            continue
        T.check(rc)
        work = torch.empty(max(1, sz.value), dtype=torch.uint8, device="cuda")
        dx = torch.empty_like(da)
        T.check(L.tprgb_ref_solve_device(
            kind, nsys, n, s, pr, da.data_ptr(), dc.data_ptr(), dr.data_ptr(),
            dx.data_ptr(), work.data_ptr() if sz.value else None, sz.value,
            torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        x = dx.cpu().numpy()
        for k in range(nsys):
            sl = slice(k * n, (k + 1) * n)
            a, c, r = norm[0][sl], norm[1][sl], norm[2][sl]
            xr = (port.ptpr if kind == 0 else port.tpr)(a, c, r, s, dt)[0]
            _bits_equal(x[sl], xr)
            if k == 0:
                _bits_equal(cu(a, c, r, n, s, dt), xr)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("cls,kind", [("PTPR", 0), ("TPR", 1)])
def test_handle_repeated_solves(cuda, port, prec, cls, kind):
    """One handle, many solves: the one-launch path is captured into a CUDA
    graph at the second solve (one graph per setter form) and replayed,
    and completion is read from the mapped word the kernel counts up.
    New systems every time, the 3- and 4-argument setters alternating, a
    solve whose x is never read before the next set: every x the same bits
    as the C restatement."""
    dt = np.float32 if prec == "f32" else np.float64
    n, s = 2048, 512
    t = getattr(T, cls)(n, s, dtype=dt)
    ref = port.ptpr if kind == 0 else port.tpr
    for it in range(7):
        a, b, c, d, _ = G.one_system(n, 900 + it, "uneven")
        a, b, c, d = (v.astype(dt) for v in (a, b, c, d))
        if it % 2:
            t.set_tridiagonal_system(a, b, c, d)
        else:
            t.set_tridiagonal_system(a / b, c / b, d / b)
        t.solve()
        if it == 3:
            continue  # the next set waits for this solve
        an, cn, rn = port.normalize(a, b, c, d, dt)
        if it % 2 == 0:
            an, cn, rn = a / b, c / b, d / b
        _bits_equal(t.get_ans(), ref(an, cn, rn, s, dt)[0])


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_tiny_cr_pcr_vs_port(cuda, port, prec):
    """Standalone CR / PCR on n = 1, 2, 4, 8 (n = 1: x = rhs, no reduction;
    n = 2: the two-row solve alone): same bits as the C restatement."""
    dt = np.float32 if prec == "f32" else np.float64
    for n in (1, 2, 4, 8):
        a, b, c, d, _ = G.one_system(max(n, 2), 17 + n, "uneven")
        an, cn, rn = port.normalize(a[:n], b[:n], c[:n], d[:n], dt)
        _bits_equal(T.cr_cu(an, cn, rn, n, dt), port.cr(an, cn, rn, dt)[0])
        _bits_equal(T.pcr_cu(an, cn, rn, n, dt), port.pcr(an, cn, rn, dt)[0])


def test_invalid_arguments_return_codes(cuda):
    with pytest.raises(T.TprError) as e:
        T.PTPR(1000, 8)
    assert e.value.code == T.EINVAL
    with pytest.raises(T.TprError) as e:
        T.TPR(1024, 2048)
    assert e.value.code == T.EINVAL
    t = T.PTPR(64, 8)
    with pytest.raises(T.TprError):
        t.solve()  # no system set


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_timed_round_trip_same_bits(cuda, golden, prec):
    """tprgb_time_roundtrip runs the handle's set / solve / get sequence in
    C++ (4-argument setter): a positive time per round trip and the
    reference's bits in x."""
    import ctypes
    dt = np.float32 if prec == "f32" else np.float64
    L = T.load()
    a, b, c, d = [np.ascontiguousarray(v, dt)
                  for v in G.one_system(2048, 42, "dominant")[:4]]
    p = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    for kind, key in ((T.PTPR_KIND, "ptpr"), (T.TPR_KIND, "tpr")):
        h = ctypes.c_void_p()
        T.check(L.tprgb_create(kind, 2048, 512, T.F32 if prec == "f32" else T.F64,
                               ctypes.byref(h)))
        try:
            us = ctypes.c_double()
            x = np.zeros(2048, dt)
            T.check(L.tprgb_time_roundtrip(h, p(a), p(b), p(c), p(d), p(x), 5,
                                           ctypes.byref(us)))
            assert us.value > 0
            _bits_equal(x, golden[f"plain_{key}_s512_{prec}"])
        finally:
            L.tprgb_destroy(h)
