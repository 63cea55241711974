"""Seeded synthetic tridiagonal systems for the TPR / PTPR workloads.

Each system is ``a[i] x[i-1] + b[i] x[i] + c[i] x[i+1] = d[i]`` stored in
FP32 with ``a[0] = c[n-1] = 0``.  The generator follows the workload
definitions the solver is measured on:

* ``"dominant"``   (plain single system and the uniform ADI-style batch):
  a, c ~ U(-1, 1); b = |a| + |c| + U(1, 2) (strictly diagonally dominant)
* ``"uneven"``     (the uneven autotuned batch and the serving stream):
  b = |a| + |c| + U(0.1, 1)
* ``"weak"``       (the precision-stress batch): b = |a| + |c| + 10^U(-4,-1)
  (condition numbers up to about 1e4)

The true solution x_t ~ U(-1, 1) is kept in FP64 and d = A x_t is computed
in FP64 from the FP32-stored a, b, c, then rounded to FP32.  System ``k`` of
a batch uses its own stream seeded ``seed + k``.

The reference's own generators (src/system.cpp:118-158) are a fixed
a = c = -1/6, b = 1, rhs = i + 1 system (``fixed_system`` here) and uniform
random inputs; the batch workloads above are the measured configurations.
"""
from __future__ import annotations

import numpy as np

KINDS = ("dominant", "uneven", "weak")


def _margin(rng: np.random.Generator, n: int, kind: str) -> np.ndarray:
    if kind == "dominant":
        return rng.uniform(1.0, 2.0, n)
    if kind == "uneven":
        return rng.uniform(0.1, 1.0, n)
    if kind == "weak":
        return 10.0 ** rng.uniform(-4.0, -1.0, n)
    raise ValueError(f"unknown system kind {kind!r}")


def one_system(n: int, seed: int, kind: str = "dominant"):
    """Return (a, b, c, d, x_t) for one system; a..d float32, x_t float64."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a64 = rng.uniform(-1.0, 1.0, n)
    c64 = rng.uniform(-1.0, 1.0, n)
    a64[0] = 0.0
    c64[n - 1] = 0.0
    a = a64.astype(np.float32)
    c = c64.astype(np.float32)
    b = (np.abs(a.astype(np.float64)) + np.abs(c.astype(np.float64))
         + _margin(rng, n, kind)).astype(np.float32)
    xt = rng.uniform(-1.0, 1.0, n)
    d = apply(a, b, c, xt).astype(np.float32)
    return a, b, c, d, xt


def apply(a, b, c, x) -> np.ndarray:
    """y = A x in FP64 for one system (a[0], c[n-1] ignored)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    c = np.asarray(c, np.float64)
    x = np.asarray(x, np.float64)
    y = b * x
    y[1:] += a[1:] * x[:-1]
    y[:-1] += c[:-1] * x[1:]
    return y


class Batch:
    """A batch of systems laid out back to back in four FP32 arrays.

    ``offsets[k]`` is the first equation of system ``k`` and ``ns[k]`` its
    size; every offset is a multiple of 4 equations (16 bytes)."""

    def __init__(self, ns, a, b, c, d, xt, offsets=None):
        self.ns = np.asarray(ns, dtype=np.int32)
        if offsets is None:
            offsets = np.zeros(len(self.ns), dtype=np.int64)
            if len(self.ns) > 1:
                offsets[1:] = np.cumsum(self.ns[:-1], dtype=np.int64)
        self.offsets = np.asarray(offsets, dtype=np.int64)
        self.a, self.b, self.c, self.d = a, b, c, d
        self.xt = xt

    @property
    def nsys(self) -> int:
        return int(len(self.ns))

    @property
    def neq(self) -> int:
        return int(self.a.shape[0])

    def system(self, k: int):
        o, n = int(self.offsets[k]), int(self.ns[k])
        return (self.a[o:o + n], self.b[o:o + n], self.c[o:o + n],
                self.d[o:o + n])


def batch(ns, seed: int, kind: str = "dominant") -> Batch:
    """Batch whose system k has size ns[k] and seed seed + k."""
    ns = np.asarray(ns, dtype=np.int64)
    total = int(ns.sum())
    a = np.empty(total, np.float32)
    b = np.empty(total, np.float32)
    c = np.empty(total, np.float32)
    d = np.empty(total, np.float32)
    xt = np.empty(total, np.float64)
    o = 0
    for k, n in enumerate(ns):
        n = int(n)
        a[o:o + n], b[o:o + n], c[o:o + n], d[o:o + n], xt[o:o + n] = \
            one_system(n, seed + k, kind)
        o += n
    return Batch(ns, a, b, c, d, xt)


def uniform_batch(nsys: int, n: int, seed: int, kind: str = "dominant"):
    return batch(np.full(nsys, n), seed, kind)


def uneven_sizes(nsys: int, kmin: int, kmax: int, seed: int) -> np.ndarray:
    """N = 2^k with k uniform in [kmin, kmax] (inclusive)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return (1 << rng.integers(kmin, kmax + 1, nsys)).astype(np.int64)


def fixed_system(n: int):
    """a = c = -1/6, diag = 1, rhs = i + 1 (src/system.cpp:118-130)."""
    a = np.full(n, -1.0 / 6.0, np.float64)
    c = np.full(n, -1.0 / 6.0, np.float64)
    diag = np.ones(n, np.float64)
    rhs = np.arange(1, n + 1, dtype=np.float64)
    a[0] = 0.0
    c[n - 1] = 0.0
    return a, diag, c, rhs
