"""The allocation-free reference-semantics entry point
(tprgb_ref_solve_device_static), for callers that cannot call cudaMalloc --
code inside CUDA stream capture, latency-critical loops, hosts whose device
memory belongs to another allocator.  Its workspace is the library's own
16 MiB device array.  Checked through the C ABI against the existing entry
point (caller-provided workspace) on two calls in a row, bit for bit (the
tolerance of the reference-semantics tests).  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

import tpr_gb300 as T
from tpr_gb300 import generate as G

pytestmark = pytest.mark.gpu


def _inputs(torch, nsys, n, seed, dt):
    bt = G.uniform_batch(nsys, n, seed, "uneven")
    tdt = torch.float32 if dt == np.float32 else torch.float64
    arrs = [(bt.a / bt.b).astype(dt), (bt.c / bt.b).astype(dt),
            (bt.d / bt.b).astype(dt)]
    return [torch.from_numpy(v).to("cuda", tdt) for v in arrs]


def _existing(torch, L, kind, nsys, n, s, prec, a, c, r):
    sz = ctypes.c_size_t()
    T.check(L.tprgb_ref_workspace_bytes(kind, nsys, n, s, prec,
                                        ctypes.byref(sz)))
    work = torch.empty(max(sz.value, 1), dtype=torch.uint8, device="cuda")
    x = torch.empty_like(a)
    T.check(L.tprgb_ref_solve_device(
        kind, nsys, n, s, prec, a.data_ptr(), c.data_ptr(), r.data_ptr(),
        x.data_ptr(), work.data_ptr(), sz.value,
        torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return x.cpu().numpy()


def _static(torch, L, kind, nsys, n, s, prec, a, c, r):
    x = torch.full_like(a, float("nan"))
    T.check(L.tprgb_ref_solve_device_static(
        kind, nsys, n, s, prec, a.data_ptr(), c.data_ptr(), r.data_ptr(),
        x.data_ptr(), torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return x.cpu().numpy()


@pytest.mark.parametrize("kind", [T.PTPR_KIND, T.TPR_KIND])
@pytest.mark.parametrize("prec", [T.F32, T.F64])
def test_static_workspace_matches_caller_workspace(cuda, kind, prec):
    torch = cuda
    L = T.load()
    dt = np.float32 if prec == T.F32 else np.float64
    n, s, nsys = 1 << 15, 256, 3            # sliced shape: uses a workspace
    for call, seed in enumerate((11, 12)):  # two calls in a row
        a, c, r = _inputs(torch, nsys, n, seed + 10 * kind, dt)
        want = _existing(torch, L, kind, nsys, n, s, prec, a, c, r)
        got = _static(torch, L, kind, nsys, n, s, prec, a, c, r)
        assert np.isfinite(got).all(), call
        np.testing.assert_array_equal(got, want)


def test_static_workspace_limit(cuda):
    torch = cuda
    L = T.load()
    n, s = 1 << 20, 1024                    # 3n+3m floats = 12.6 MB per system
    a = torch.zeros(2 * n, device="cuda")
    rc = L.tprgb_ref_solve_device_static(
        T.PTPR_KIND, 2, n, s, T.F32, a.data_ptr(), a.data_ptr(),
        a.data_ptr(), a.data_ptr(), None)
    assert rc == T.EUNSUPPORTED
    assert b"16777216" in L.tprgb_last_error()
