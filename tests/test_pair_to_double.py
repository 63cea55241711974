"""The FP32-pair -> FP64 bit assembly used for the solver's FP64 output
(hier::pair_to_double), emulated step for step on the CPU and checked
against the exact sum, including values at and around powers of two; the
GPU test runs the device function itself through a diagnostics entry
point."""
import ctypes

import numpy as np
import pytest


def f32_to_f64_normal(f):
    """Bits of the double equal to a normal float, built as on the device
    (hier::f32_to_f64_normal)."""
    u = int(np.array(f, np.float32).view(np.uint32))
    hi = (((u & 0x7FFFFFFF) >> 3) + 0x38000000) | (u & 0x80000000)
    lo = (u << 29) & 0xFFFFFFFF
    return float(np.array((hi << 32) | lo, np.uint64).view(np.float64))


def fast_ok(h, l):
    m = int(np.array(h, np.float32).view(np.uint32)) & 0x7FFFFFFF
    el = int(np.array(l, np.float32).view(np.uint32)) & 0x7F800000
    return (m - 0x1E000000) % (1 << 32) < 0x7F800000 - 0x1E000000 and \
        el != 0x7F800000


def emulate(hi, lo):
    """hier::pair_to_double step for step: a DADD (numpy float64 addition,
    round to nearest even) of the two bit-built doubles, or of the exact
    conversions on the slow route."""
    h, l = np.float32(hi), np.float32(lo)
    if fast_ok(h, l):
        return f32_to_f64_normal(h) + f32_to_f64_normal(l)
    return float(h) + float(l)


def cases(seed=0, n=20000):
    rng = np.random.default_rng(seed)
    hi = (rng.uniform(-1, 1, n) * 10.0 ** rng.integers(-12, 12, n)
          ).astype(np.float32)
    lo = (hi * rng.uniform(-2.0 ** -22, 2.0 ** -22, n)).astype(np.float32)
    extra = []
    for e in range(-30, 30):
        p = np.float32(2.0 ** e)
        for f in (1, -1):
            for r in (-2.0 ** -25, -2.0 ** -26, 2.0 ** -25, -0.75 * 2.0 ** -24,
                      0.0):
                extra.append((np.float32(f * p), np.float32(f * p * r)))
    extra += [(0.0, 1e-30), (1e-40, 0.0), (3.0, 0.0), (1e-30, 1e-38)]
    # smallest magnitudes on the integer route: subnormal low parts
    for e in (-74, -73, -72):
        for m in (1.0, 1.5, -1.0):
            for t in (1e-45, -1e-45, 3e-39, -5.9e-39, 1.1e-38):
                extra.append((np.float32(m * 2.0 ** e), np.float32(t)))
    # the screen's edge: |hi| around 2^-67 with zero / subnormal lo
    for e in (-68, -67, -66):
        for t in (0.0, -0.0, 1e-45, -3e-39, 1.17e-38):
            extra.append((np.float32(1.25 * 2.0 ** e), np.float32(t)))
    # non-finite operands (slow route)
    extra += [(np.inf, 1.0), (-np.inf, 0.0), (1.0, np.inf), (2.0, -np.inf)]
    # largest magnitudes
    for m in (3.4e38, -3.4e38, 2.0 ** 127, 1.7e38):
        for r in (2.0 ** -25, -2.0 ** -26, 0.3 * 2.0 ** -24):
            extra.append((np.float32(m), np.float32(m * r)))
    # exact halfway cases between doubles (ties to even)
    for h in (1.0, 1.0 + 2.0 ** -23, -1.0, 1.5, 2.0 ** 20):
        u = 2.0 ** (np.floor(np.log2(abs(h))) - 53)
        for m in (1, 3, 5, -1, -3):
            extra.append((np.float32(h), np.float32(m * u)))
    eh = np.array([x for x, _ in extra], np.float32)
    el = np.array([y for _, y in extra], np.float32)
    return np.concatenate([hi, eh]), np.concatenate([lo, el])


def test_emulated_assembly_is_exact():
    hi, lo = cases()
    for h, l in zip(hi, lo):
        assert emulate(h, l) == float(h) + float(l), (h, l)


def test_bit_built_double_is_exact_for_normal_floats():
    rng = np.random.default_rng(3)
    bits = rng.integers(0x00800000, 0x7F800000, 5000, dtype=np.int64)
    bits = np.concatenate([bits, bits | 0x80000000]).astype(np.uint32)
    for f in bits.view(np.float32):
        assert f32_to_f64_normal(f) == float(f), f


@pytest.mark.gpu
def test_device_assembly_matches(cuda, lib):
    torch = cuda
    hi, lo = cases(1)
    dh = torch.from_numpy(hi).cuda()
    dl = torch.from_numpy(lo).cuda()
    out = torch.empty(len(hi), dtype=torch.float64, device="cuda")
    rc = lib.tprgb_diag_pair_to_double(len(hi), ctypes.c_void_p(dh.data_ptr()),
                                       ctypes.c_void_p(dl.data_ptr()),
                                       ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    want = hi.astype(np.float64) + lo.astype(np.float64)
    np.testing.assert_array_equal(out.cpu().numpy(), want)
