"""Host mirror of the device-side seeded generator (gen_kernels.cu):
bit-identical a, b, c, d for the same (n, seed, kind), used to check the
device generator and to materialise a served request on the host."""
from __future__ import annotations

import numpy as np

KIND = {"dominant": 0, "uneven": 1, "weak": 2}
_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(z):
    z = (z + np.uint64(0x9E3779B97F4A7C15)) & _M
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M
    return z ^ (z >> np.uint64(31))


def _u01(seed, i, which):
    i = np.asarray(i, np.int64).astype(np.uint64)
    k = _mix64(np.uint64(seed) ^ _mix64((i << np.uint64(2)) | np.uint64(which)))
    return (k >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)


def _coef(seed, i, which):
    return (np.float32(2.0) * _u01(seed, i, which)).astype(np.float32) - \
        np.float32(1.0)


def system(n: int, seed: int, kind: str = "uneven"):
    """(a, b, c, d) float32 exactly as the device generator writes them
    (the weak kind's 10^x margin uses the device exp10f, so only the
    dominant and uneven kinds are mirrored bit for bit)."""
    with np.errstate(over="ignore"):
        i = np.arange(n, dtype=np.int64)
        a = _coef(seed, i, 0)
        c = _coef(seed, i, 1)
        a[0] = 0.0
        c[n - 1] = 0.0
        u = _u01(seed, i, 2)
        k = KIND[kind]
        if k == 0:
            m = np.float32(1.0) + u
        elif k == 1:
            m = np.float32(0.1) + (np.float32(0.9) * u).astype(np.float32)
        else:
            m = (10.0 ** ((np.float32(3.0) * u).astype(np.float32)
                          - np.float32(4.0)).astype(np.float64)
                 ).astype(np.float32)
        b = ((np.abs(a) + np.abs(c)).astype(np.float32) + m).astype(np.float32)
        xt = _coef(seed, i, 3)
        xm = np.concatenate([[np.float32(0)], xt[:-1]]).astype(np.float32)
        xp = np.concatenate([xt[1:], [np.float32(0)]]).astype(np.float32)
        d = ((a * xm).astype(np.float32) + (b * xt).astype(np.float32)
             ).astype(np.float32)
        d = (d + (c * xp).astype(np.float32)).astype(np.float32)
    return a, b, c, d
