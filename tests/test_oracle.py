"""The CPU oracle, pinned against the reference's golden vectors and against
outputs of the reference's own solvers (tests/golden, made by
tests/golden/make_golden.py)."""
import hashlib

import numpy as np
import pytest

from tpr_gb300 import generate as G

SWEEP = [4, 8, 16, 32, 64, 128, 256, 512, 1024]


def _fixed(dtype):
    a, diag, c, rhs = G.fixed_system(1024)
    return a.astype(dtype), c.astype(dtype), rhs.astype(dtype)


def _assert_kat(ans, x):
    """Known-answer check with the reference's tolerances
    (test/examples.cpp:36-56): |x_i - ans_i| <= 1e-2 and max squared
    difference <= 1e-3."""
    x = np.asarray(x, np.float64)
    assert np.all(np.abs(x - ans) <= 1e-2)
    assert np.max((x - ans) ** 2) <= 1e-3


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_fixed_cr_pcr_bitwise(port, golden, ans1024, prec):
    dt = np.float32 if prec == "f32" else np.float64
    a, c, r = _fixed(dt)
    x, f = port.cr(a, c, r, dt)
    assert f == 17 * 1024
    np.testing.assert_array_equal(x, golden[f"fixed_cr_{prec}"])
    _assert_kat(ans1024, x)
    x, f = port.pcr(a, c, r, dt)
    assert f == 14 * 1024 * 10
    np.testing.assert_array_equal(x, golden[f"fixed_pcr_{prec}"])
    _assert_kat(ans1024, x)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("s", SWEEP)
def test_fixed_tpr_ptpr_bitwise(port, golden, ans1024, prec, s):
    dt = np.float32 if prec == "f32" else np.float64
    a, c, r = _fixed(dt)
    x, _ = port.ptpr(a, c, r, s, dt)
    np.testing.assert_array_equal(x, golden[f"fixed_ptpr_s{s}_{prec}"])
    _assert_kat(ans1024, x)
    x, _ = port.tpr(a, c, r, s, dt)
    np.testing.assert_array_equal(x, golden[f"fixed_tpr_s{s}_{prec}"])
    _assert_kat(ans1024, x)


def test_plain_inputs_unchanged(golden):
    """The generator still produces the inputs the fixtures were made on."""
    a, b, c, d, _ = G.one_system(2048, 42, "dominant")
    h = hashlib.sha256()
    for x in (a, b, c, d):
        h.update(np.ascontiguousarray(x).tobytes())
    assert h.hexdigest().encode() == golden["plain_input_sha256"].tobytes()


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("s", [64, 128, 256, 512, 1024, 2048])
def test_plain_ptpr_tpr_bitwise(port, golden, prec, s):
    dt = np.float32 if prec == "f32" else np.float64
    a, b, c, d, xt = G.one_system(2048, 42, "dominant")
    an, cn, rn = port.normalize(a, b, c, d, dt)
    for name in ("ptpr", "tpr"):
        x, _ = getattr(port, name)(an, cn, rn, s, dt)
        np.testing.assert_array_equal(x, golden[f"plain_{name}_s{s}_{prec}"])
        # FP32 inputs limit accuracy against x_t to ~cond * 6e-8
        assert port.rel_l2(x, xt) < (1e-6 if prec == "f32" else 1e-7)


@pytest.mark.parametrize("k", range(1, 21))
def test_nstab_fixtures_bitwise(port, golden, nstab, k):
    """Stability fixtures: same bits as the reference, including the
    non-finite results on the non-dominant / singular fixtures."""
    a, diag, c, rhs = nstab[f"eq{k}"]
    an, cn, rn = port.normalize(a, diag, c, rhs, np.float32)
    with np.errstate(all="ignore"):
        for s in (16, 64, 512):
            for name in ("ptpr", "tpr"):
                x, _ = getattr(port, name)(an, cn, rn, s, np.float32)
                np.testing.assert_array_equal(
                    x, golden[f"nstab_eq{k}_{name}_s{s}_f32"])


def test_thomas_matches_dense_solve(port):
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 17, 64):
        a, b, c, d, _ = G.one_system(n, int(rng.integers(1 << 30)), "weak")
        A = np.diag(b.astype(np.float64))
        if n > 1:
            A += np.diag(a[1:].astype(np.float64), -1)
            A += np.diag(c[:-1].astype(np.float64), 1)
        x = port.thomas(a, b, c, d)
        np.testing.assert_allclose(x, np.linalg.solve(A, d.astype(np.float64)),
                                   rtol=1e-9, atol=1e-12)


def test_batch_thomas_and_rel_l2(port):
    bt = G.batch([64, 256, 1024, 128], 11, "uneven")
    x = port.batch_thomas(bt, threads=2)
    for k in range(bt.nsys):
        a, b, c, d = bt.system(k)
        o, n = bt.offsets[k], bt.ns[k]
        np.testing.assert_array_equal(x[o:o + n], port.thomas(a, b, c, d))
    worst, per = port.batch_rel_l2(bt, x, bt.xt, threads=2)
    assert worst == per.max() and worst < 1e-6
    assert port.rel_l2(bt.xt, bt.xt) == 0.0


def test_batch_cpu_baseline_matches_single(port):
    bt = G.uniform_batch(6, 256, 5)
    for kind, name in ((0, "ptpr"), (1, "tpr")):
        xb = port.batch_tpr(kind, 6, 256, 32, bt.a, bt.b, bt.c, bt.d, threads=3)
        for k in range(6):
            a, b, c, d = bt.system(k)
            an, cn, rn = port.normalize(a, b, c, d)
            x, _ = getattr(port, name)(an, cn, rn, 32)
            np.testing.assert_array_equal(xb[k * 256:(k + 1) * 256], x)


def test_reference_build_agrees_when_present(port):
    """Where the reference was compiled here, the port equals it on a fresh
    random case (the fixtures pin the same thing elsewhere)."""
    from oracle import oracle as O
    r = O.ref("f32")
    if r is None:
        pytest.skip("reference solvers not built on this machine")
    a, b, c, d, _ = G.one_system(4096, 7, "uneven")
    an, cn, rn = port.normalize(a, b, c, d)
    for s in (8, 256):
        np.testing.assert_array_equal(port.ptpr(an, cn, rn, s)[0],
                                      r.ptpr(an, cn, rn, s)[0])
        np.testing.assert_array_equal(port.tpr(an, cn, rn, s)[0],
                                      r.tpr(an, cn, rn, s)[0])


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_reference_cr_pcr_agree_at_large_n(port, prec):
    """Standalone CR / PCR above one CTA's shared memory (n = 16384): the
    port equals the compiled reference, which has no size cap."""
    from oracle import oracle as O
    r = O.ref(prec)
    if r is None:
        pytest.skip("reference solvers not built on this machine")
    dt = np.float32 if prec == "f32" else np.float64
    a, b, c, d, _ = G.one_system(16384, 9, "uneven")
    an, cn, rn = port.normalize(a, b, c, d, dt)
    np.testing.assert_array_equal(port.cr(an, cn, rn, dt)[0], r.cr(an, cn, rn)[0])
    np.testing.assert_array_equal(port.pcr(an, cn, rn, dt)[0], r.pcr(an, cn, rn)[0])


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_timed_plain_loop_threads_same_bits(port, golden, prec):
    """The timed single-system loop with solver-internal OpenMP (stages 1
    and 3 parallel over slices) gives the fixtures' bits at any thread
    count, so the timed CPU baseline computes what the reference computes."""
    dt = np.float32 if prec == "f32" else np.float64
    a, b, c, d, _ = G.one_system(2048, 42, "dominant")
    an, cn, rn = port.normalize(a, b, c, d, dt)
    for kind, name in ((0, "ptpr"), (1, "tpr")):
        for threads in (1, 3, 4):
            t, x = port.time_plain(kind, an, cn, rn, 512, 3, threads, dt)
            assert t > 0.0
            np.testing.assert_array_equal(x, golden[f"plain_{name}_s512_{prec}"])


def test_reference_timed_loop_agrees_when_present(port):
    """Where the reference was compiled here, its own timed loop (the
    tpr_pm pattern) returns the port's bits."""
    from oracle import oracle as O
    r = O.ref("f32")
    if r is None:
        pytest.skip("reference solvers not built on this machine")
    a, b, c, d, _ = G.one_system(2048, 42, "dominant")
    an, cn, rn = port.normalize(a, b, c, d)
    for kind in (0, 1):
        _, xr = r.time_plain(kind, an, cn, rn, 512, 3, 4)
        _, xp = port.time_plain(kind, an, cn, rn, 512, 3, 4)
        np.testing.assert_array_equal(xp, xr)
