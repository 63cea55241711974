"""ctypes front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests, ``__graft_entry__.smoke`` and
bench.py's CPU-baseline leg; the solver package never imports it.

``port()``  -> the C restatement (oracle/oracle.c, built as liboracle.so)
``ref(p)``  -> the reference's own CPU solvers compiled from its sources
               (oracle/_ref/libtprref_{f32,f64}.so), or None where they were
               not built (the reference tree exists only in the build
               container).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_PORT = os.path.join(HERE, "liboracle.so")
_REF = {"f32": os.path.join(HERE, "_ref", "libtprref_f32.so"),
        "f64": os.path.join(HERE, "_ref", "libtprref_f64.so")}
# The reference tree (read only; used to build oracle/_ref and to make the
# golden fixtures): $TPR_REFERENCE_ROOT, else a `reference` directory beside
# this repository's root.
REFERENCE_ROOT = os.environ.get(
    "TPR_REFERENCE_ROOT",
    os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

_fp = C.c_void_p
_i = C.c_int
_i64p = C.c_void_p


def build(reference: bool | None = None) -> None:
    """Compile liboracle.so, and the reference solvers when the reference
    tree is present."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if reference is None:
        reference = os.path.isdir(os.path.join(REFERENCE_ROOT, "src"))
    if reference:
        subprocess.run(["make", "-s", "-C", HERE, "ref",
                        f"REF={REFERENCE_ROOT}"], check=True)


def _ptr(x: np.ndarray):
    return x.ctypes.data_as(C.c_void_p)


class Port:
    """The C restatement."""

    def __init__(self, path: str = _PORT):
        if not os.path.exists(path):
            build(reference=False)
        self.lib = C.CDLL(path)
        L = self.lib
        for sfx in ("f32", "f64"):
            getattr(L, f"orc_ptpr_{sfx}").argtypes = [_i, _i, _fp, _fp, _fp, _fp]
            getattr(L, f"orc_tpr_{sfx}").argtypes = [_i, _i, _fp, _fp, _fp, _fp]
            getattr(L, f"orc_cr_{sfx}").argtypes = [_i, _fp, _fp, _fp, _fp]
            getattr(L, f"orc_pcr_{sfx}").argtypes = [_i, _fp, _fp, _fp]
            getattr(L, f"orc_normalize_{sfx}").argtypes = [_i, _fp, _fp, _fp, _fp]
            for f in ("ptpr", "tpr", "cr", "pcr"):
                getattr(L, f"orc_{f}_{sfx}").restype = _i
        L.orc_thomas_f64.argtypes = [_i, _fp, _fp, _fp, _fp, _fp]
        L.orc_batch_thomas_f32in.argtypes = [_i, _i64p, _fp, _fp, _fp, _fp,
                                             _fp, _fp, _i]
        L.orc_batch_thomas_f64.argtypes = [_i, _i64p, _fp, _fp, _fp, _fp,
                                           _fp, _fp, _i]
        L.orc_rel_l2_f64.argtypes = [C.c_int64, _fp, _fp]
        L.orc_rel_l2_f64.restype = C.c_double
        L.orc_batch_rel_l2.argtypes = [_i, _i64p, _fp, _fp, _fp, _fp, _i]
        L.orc_batch_rel_l2.restype = C.c_double
        L.orc_batch_tpr_f32.argtypes = [_i, _i, _i, _i, _fp, _fp, _fp, _fp,
                                        _fp, _i]
        L.orc_max_threads.restype = _i
        for sfx in ("f32", "f64"):
            fn = getattr(L, f"orc_time_plain_{sfx}")
            fn.argtypes = [_i, _i, _i, _fp, _fp, _fp, _i, _i, _fp]
            fn.restype = C.c_double

    # -- reference solver restatements (inputs copied, never mutated) -----
    @staticmethod
    def _prep(dtype, *arrs):
        return [np.array(x, dtype=dtype, copy=True) for x in arrs]

    def normalize(self, a, diag, c, rhs, dtype=np.float32):
        a, diag, c, rhs = self._prep(dtype, a, diag, c, rhs)
        sfx = "f32" if dtype == np.float32 else "f64"
        getattr(self.lib, f"orc_normalize_{sfx}")(len(a), _ptr(a), _ptr(diag),
                                                  _ptr(c), _ptr(rhs))
        return a, c, rhs

    def _tprlike(self, name, a, c, rhs, s, dtype):
        a, c, rhs = self._prep(dtype, a, c, rhs)
        x = np.zeros(len(a), dtype)
        sfx = "f32" if dtype == np.float32 else "f64"
        flops = getattr(self.lib, f"orc_{name}_{sfx}")(len(a), s, _ptr(a),
                                                       _ptr(c), _ptr(rhs),
                                                       _ptr(x))
        return x, flops

    def ptpr(self, a, c, rhs, s, dtype=np.float32):
        return self._tprlike("ptpr", a, c, rhs, s, dtype)

    def tpr(self, a, c, rhs, s, dtype=np.float32):
        return self._tprlike("tpr", a, c, rhs, s, dtype)

    def cr(self, a, c, rhs, dtype=np.float32):
        a, c, rhs = self._prep(dtype, a, c, rhs)
        x = np.zeros(len(a), dtype)
        sfx = "f32" if dtype == np.float32 else "f64"
        f = getattr(self.lib, f"orc_cr_{sfx}")(len(a), _ptr(a), _ptr(c),
                                               _ptr(rhs), _ptr(x))
        return x, f

    def pcr(self, a, c, rhs, dtype=np.float32):
        a, c, rhs = self._prep(dtype, a, c, rhs)
        sfx = "f32" if dtype == np.float32 else "f64"
        f = getattr(self.lib, f"orc_pcr_{sfx}")(len(a), _ptr(a), _ptr(c),
                                                _ptr(rhs))
        return rhs, f

    # -- FP64 truth ------------------------------------------------------
    def thomas(self, a, b, c, d):
        a, b, c, d = self._prep(np.float64, a, b, c, d)
        x = np.zeros(len(a), np.float64)
        self.lib.orc_thomas_f64(len(a), _ptr(a), _ptr(b), _ptr(c), _ptr(d),
                                _ptr(x))
        return x

    def batch_thomas(self, batch, threads: int = 0):
        """FP64 Thomas of every system of a FP32 generate.Batch."""
        x = np.empty(batch.neq, np.float64)
        self.lib.orc_batch_thomas_f32in(
            batch.nsys, _ptr(batch.offsets), _ptr(batch.ns), _ptr(batch.a),
            _ptr(batch.b), _ptr(batch.c), _ptr(batch.d), _ptr(x),
            threads or os.cpu_count())
        return x

    def batch_thomas_f64(self, nsys, offsets, ns, a, b, c, d, threads=0):
        x = np.empty(len(a), np.float64)
        offsets = np.ascontiguousarray(offsets, np.int64)
        ns = np.ascontiguousarray(ns, np.int32)
        self.lib.orc_batch_thomas_f64(nsys, _ptr(offsets), _ptr(ns), _ptr(a),
                                      _ptr(b), _ptr(c), _ptr(d), _ptr(x),
                                      threads or os.cpu_count())
        return x

    def rel_l2(self, x, xt) -> float:
        x = np.ascontiguousarray(x, np.float64)
        xt = np.ascontiguousarray(xt, np.float64)
        return float(self.lib.orc_rel_l2_f64(len(x), _ptr(x), _ptr(xt)))

    def batch_rel_l2(self, batch, x, xt, threads: int = 0):
        """Per-system relative L2 errors; returns (max, array)."""
        x = np.ascontiguousarray(x, np.float64)
        xt = np.ascontiguousarray(xt, np.float64)
        out = np.empty(batch.nsys, np.float64)
        worst = self.lib.orc_batch_rel_l2(batch.nsys, _ptr(batch.offsets),
                                          _ptr(batch.ns), _ptr(x), _ptr(xt),
                                          _ptr(out), threads or os.cpu_count())
        return float(worst), out

    def batch_tpr(self, kind, nsys, n, s, a, b, c, d, threads=0):
        """Uniform-batch PTPR (kind 0) / TPR (kind 1), FP32, OpenMP over
        systems; returns x (float32)."""
        x = np.empty(nsys * n, np.float32)
        self.lib.orc_batch_tpr_f32(kind, nsys, n, s, _ptr(a), _ptr(b),
                                   _ptr(c), _ptr(d), _ptr(x),
                                   threads or os.cpu_count())
        return x

    def max_threads(self) -> int:
        return int(self.lib.orc_max_threads())

    def time_plain(self, kind, a, c, rhs, s, iters, threads=0,
                   dtype=np.float32):
        """The reference's timed single-system loop (src/pm.cpp:160-194)
        on the diag-normalised a, c, rhs: PTPR (kind 0) or TPR (kind 1)
        with solver-internal OpenMP on `threads` threads.  Returns (seconds
        in solve + get_ans over all iterations, last x)."""
        a, c, rhs = self._prep(dtype, a, c, rhs)
        x = np.zeros(len(a), dtype)
        sfx = "f32" if dtype == np.float32 else "f64"
        t = getattr(self.lib, f"orc_time_plain_{sfx}")(
            kind, len(a), s, _ptr(a), _ptr(c), _ptr(rhs), iters,
            threads or os.cpu_count(), _ptr(x))
        return float(t), x


class Ref:
    """The reference's own CPU solvers (built from its sources)."""

    def __init__(self, prec: str = "f32"):
        self.dtype = np.float32 if prec == "f32" else np.float64
        self.lib = C.CDLL(_REF[prec])
        L = self.lib
        L.ref_ptpr.argtypes = [_i, _i, _fp, _fp, _fp, _fp]
        L.ref_ptpr_diag.argtypes = [_i, _i, _fp, _fp, _fp, _fp, _fp]
        L.ref_tpr.argtypes = [_i, _i, _fp, _fp, _fp, _fp]
        L.ref_cr.argtypes = [_i, _fp, _fp, _fp, _fp]
        L.ref_pcr.argtypes = [_i, _fp, _fp, _fp, _fp]
        L.ref_batch_ptpr.argtypes = [_i, _i, _i, _fp, _fp, _fp, _fp, _fp, _i]
        L.ref_batch_tpr.argtypes = [_i, _i, _i, _fp, _fp, _fp, _fp, _fp, _i]
        for f in ("ref_time_plain_ptpr", "ref_time_plain_tpr"):
            getattr(L, f).argtypes = [_i, _i, _fp, _fp, _fp, _i, _i, _fp]
            getattr(L, f).restype = C.c_double
        for f in ("ref_ptpr", "ref_ptpr_diag", "ref_tpr", "ref_cr", "ref_pcr"):
            getattr(L, f).restype = _i
        assert L.ref_real_size() == np.dtype(self.dtype).itemsize

    def _run(self, fn, a, c, rhs, *extra):
        a, c, rhs = [np.array(x, self.dtype, copy=True) for x in (a, c, rhs)]
        x = np.zeros(len(a), self.dtype)
        if extra:
            f = fn(len(a), extra[0], _ptr(a), _ptr(c), _ptr(rhs), _ptr(x))
        else:
            f = fn(len(a), _ptr(a), _ptr(c), _ptr(rhs), _ptr(x))
        return x, f

    def ptpr(self, a, c, rhs, s):
        return self._run(self.lib.ref_ptpr, a, c, rhs, s)

    def tpr(self, a, c, rhs, s):
        return self._run(self.lib.ref_tpr, a, c, rhs, s)

    def cr(self, a, c, rhs):
        return self._run(self.lib.ref_cr, a, c, rhs)

    def pcr(self, a, c, rhs):
        return self._run(self.lib.ref_pcr, a, c, rhs)

    def time_plain(self, kind, a, c, rhs, s, iters, threads=0):
        """tpr_pm's timed loop on the reference's own PTPR (kind 0) / TPR
        (kind 1); returns (seconds, last x) like Port.time_plain."""
        a, c, rhs = [np.array(v, self.dtype, copy=True) for v in (a, c, rhs)]
        x = np.zeros(len(a), self.dtype)
        fn = self.lib.ref_time_plain_ptpr if kind == 0 else \
            self.lib.ref_time_plain_tpr
        t = fn(len(a), s, _ptr(a), _ptr(c), _ptr(rhs), iters,
               threads or os.cpu_count(), _ptr(x))
        return float(t), x

    def batch(self, kind, nsys, n, s, a, b, c, d, threads=0):
        x = np.empty(nsys * n, self.dtype)
        fn = self.lib.ref_batch_ptpr if kind == 0 else self.lib.ref_batch_tpr
        fn(nsys, n, s, _ptr(a), _ptr(b), _ptr(c), _ptr(d), _ptr(x),
           threads or os.cpu_count())
        return x


def port() -> Port:
    return Port()


def ref(prec: str = "f32"):
    """The compiled reference, or None if it was not built here."""
    if not os.path.exists(_REF[prec]):
        return None
    return Ref(prec)
