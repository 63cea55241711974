"""The refinement residual (hier::residual_df) emulated step for step in
FP32 on the CPU and checked against the exact residual (rational
arithmetic): the error must be small relative to the residual itself plus
an eps^2-sized term of the row's magnitude, since the correction solve only
needs r to a few digits of its own size."""
from fractions import Fraction

import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def two_prod(a, b):
    p = f32(a * b)
    e = f32(Fraction(float(a)) * Fraction(float(b)) - Fraction(float(p)))
    return p, e   # the FMA's error term is exact (representable)


def residual(a, b, c, d, xmh, xml, xh, xlo, xph, xpl, lo_terms):
    p1, e1 = two_prod(a, xmh)
    p2, e2 = two_prod(c, xph)
    q, eq = two_sum(p1, p2)
    pb, eb = two_prod(b, xh)
    s1, es = two_sum(d, -pb)
    lo = f32(f32(es - eb) - f32(eq + f32(e1 + e2)))
    if lo_terms:
        for u, v in ((a, xml), (b, xlo), (c, xpl)):
            lo = f32(Fraction(float(-u)) * Fraction(float(v)) + Fraction(float(lo)))
    return f32(f32(s1 - q) + lo)


def exact(a, b, c, d, xmh, xml, xh, xlo, xph, xpl):
    F = lambda v: Fraction(float(v))
    return (F(d) - F(a) * (F(xmh) + F(xml)) - F(b) * (F(xh) + F(xlo))
            - F(c) * (F(xph) + F(xpl)))


def test_residual_relative_accuracy():
    rng = np.random.default_rng(5)
    rel = []
    for k in range(3000):
        a, c = (f32(v) for v in rng.uniform(-1, 1, 2))
        b = f32(abs(a) + abs(c) + rng.uniform(1e-4, 2))
        xm, x, xp = rng.uniform(-1, 1, 3) * 10.0 ** rng.integers(-3, 4)
        d64 = float(a) * xm + float(b) * x + float(c) * xp
        d = f32(d64)
        # x as an FP32 solution with a small error, split into hi + lo
        xs = []
        for v in (xm, x, xp):
            v = v * (1 + rng.uniform(-1e-6, 1e-6))
            h = f32(v)
            xs += [h, f32(v - float(h))]
        xmh, xml, xh, xlo, xph, xpl = xs
        lo_terms = k % 2 == 1
        if not lo_terms:
            xml = xlo = xpl = f32(0)
        r = residual(a, b, c, d, xmh, xml, xh, xlo, xph, xpl, lo_terms)
        t = exact(a, b, c, d, xmh, xml, xh, xlo, xph, xpl)
        scale = abs(float(b) * float(xh)) + abs(float(a) * float(xmh)) + \
            abs(float(c) * float(xph)) + abs(float(d))
        err = abs(float(Fraction(float(r)) - t))
        bound = 4 * 2.0 ** -24 * abs(float(t)) + 8 * 2.0 ** -48 * scale
        assert err <= bound, (k, err, float(t), scale)
        rel.append(err / max(abs(float(t)), 1e-300))
    # typically a few FP32 ulps of r itself
    assert np.median(rel) < 1e-6
