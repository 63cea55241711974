"""The allocation-free reference-semantics entry point
(tprgb_ref_solve_device_static), for callers that cannot call cudaMalloc:
plugins whose device memory belongs to a host framework's allocator, and
latency-critical loops where an allocation would synchronise the device.
Its workspace is the library's own 16 MiB device array.

Each case calls it through the C ABI twice in a row (new inputs each time,
so the second call runs over the first call's leftovers in the shared
array) and compares it with the existing entry point (caller-provided
workspace) bit for bit -- the tolerance of the reference-semantics tests.
Shapes: the sliced path (which uses the array), including the largest batch
whose workspace fits in 16 MiB; standalone CR / PCR above one CTA's shared
memory (which use it too); the one-CTA fused path and small standalone
CR / PCR (which need no workspace); and one system past the limit.

The file name sorts last so that a run stopping at its first failure has
run every other test before this one.  Nothing here depends on the other
tests: every case also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

import tpr_gb300 as T
from tpr_gb300 import generate as G

pytestmark = pytest.mark.gpu

LIMIT = 16 << 20  # bytes of the built-in workspace


def _inputs(torch, nsys, n, seed, dt):
    bt = G.uniform_batch(nsys, n, seed, "uneven")
    tdt = torch.float32 if dt == np.float32 else torch.float64
    arrs = [(bt.a / bt.b).astype(dt), (bt.c / bt.b).astype(dt),
            (bt.d / bt.b).astype(dt)]
    return [torch.from_numpy(v).to("cuda", tdt) for v in arrs]


def _need(L, kind, nsys, n, s, prec):
    sz = ctypes.c_size_t()
    T.check(L.tprgb_ref_workspace_bytes(kind, nsys, n, s, prec,
                                        ctypes.byref(sz)))
    return sz.value


def _existing(torch, L, kind, nsys, n, s, prec, a, c, r):
    need = _need(L, kind, nsys, n, s, prec)
    work = torch.empty(max(need, 1), dtype=torch.uint8, device="cuda")
    x = torch.empty_like(a)
    T.check(L.tprgb_ref_solve_device(
        kind, nsys, n, s, prec, a.data_ptr(), c.data_ptr(), r.data_ptr(),
        x.data_ptr(), work.data_ptr() if need else None, need,
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


def _two_calls(torch, kind, nsys, n, s, prec, seed):
    L = T.load()
    dt = np.float32 if prec == T.F32 else np.float64
    for call in range(2):
        a, c, r = _inputs(torch, nsys, n, seed + 10 * kind + call, dt)
        want = _existing(torch, L, kind, nsys, n, s, prec, a, c, r)
        got = _static(torch, L, kind, nsys, n, s, prec, a, c, r)
        assert np.isfinite(got).all(), call
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("kind", [T.PTPR_KIND, T.TPR_KIND])
@pytest.mark.parametrize("prec", [T.F32, T.F64])
def test_sliced_path_matches_caller_workspace(cuda, kind, prec):
    n, s, nsys = 1 << 15, 256, 3
    assert _need(T.load(), kind, nsys, n, s, prec) > 0  # uses the array
    _two_calls(cuda, kind, nsys, n, s, prec, 11)


@pytest.mark.parametrize("kind,n,s", [(T.PTPR_KIND, 2048, 512),
                                      (T.TPR_KIND, 2048, 512),
                                      (T.CR_KIND, 1024, 1024),
                                      (T.PCR_KIND, 1024, 1024)])
def test_paths_without_workspace_match(cuda, kind, n, s):
    assert _need(T.load(), kind, 4, n, s, T.F32) == 0
    _two_calls(cuda, kind, 4, n, s, T.F32, 21)


@pytest.mark.parametrize("kind", [T.CR_KIND, T.PCR_KIND])
def test_stepped_cr_pcr_uses_the_array(cuda, kind):
    """Standalone CR / PCR above one CTA's shared memory keep their rows in
    the workspace: 3 x 16384 FP64 systems (PCR: 2.4 MB of the array)."""
    n, nsys = 1 << 14, 3
    assert _need(T.load(), kind, nsys, n, n, T.F64) > 0
    _two_calls(cuda, kind, nsys, n, n, T.F64, 41)


def test_largest_batch_that_fits(cuda):
    L = T.load()
    n, s = 1 << 15, 256
    per = _need(L, T.PTPR_KIND, 1, n, s, T.F32)
    nsys = LIMIT // per                      # 42 systems: 16.58 of 16.78 MB
    assert 0 < LIMIT - nsys * per < per
    _two_calls(cuda, T.PTPR_KIND, nsys, n, s, T.F32, 31)
    # one more system no longer fits: rejected, nothing launched
    a = cuda.zeros((nsys + 1) * n, device="cuda")
    rc = L.tprgb_ref_solve_device_static(
        T.PTPR_KIND, nsys + 1, n, s, T.F32, a.data_ptr(), a.data_ptr(),
        a.data_ptr(), a.data_ptr(), None)
    assert rc == T.EUNSUPPORTED
    assert b"16777216" in L.tprgb_last_error()


def test_far_over_limit_rejected(cuda):
    L = T.load()
    n, s = 1 << 20, 1024                    # 3n+3m floats = 12.6 MB per system
    a = cuda.zeros(2 * n, device="cuda")
    rc = L.tprgb_ref_solve_device_static(
        T.PTPR_KIND, 2, n, s, T.F32, a.data_ptr(), a.data_ptr(),
        a.data_ptr(), a.data_ptr(), None)
    assert rc == T.EUNSUPPORTED
    assert b"16777216" in L.tprgb_last_error()
