"""tpr_gb300 -- GB300 (sm_103a) tridiagonal TPR / PTPR solver.

Python host layer over the C ABI of ``libtprgb.so`` (include/tpr_gb.h).
The compute path is the CUDA library only: if it cannot be loaded every
entry point raises; there is no CPU fallback.

Reference-interface mirror (src/ptpr.hpp:44-110, src/tpr.hpp:44-112,
src/cr.hpp:24-81, src/pcr.hpp:8-68)::

    t = PTPR(n, s)                      # or TPR(n, s), CR(n), PCR(n)
    t.set_tridiagonal_system(a, c, rhs)          # 3-arg: unit diagonal
    t.set_tridiagonal_system(a, diag, c, rhs)    # 4-arg: normalised by diag
    flops = t.solve()
    t.get_ans(x)                        # fills x, returns 0

Device-pointer entry points (batched, refined, serving) live in
``tpr_gb300.batch`` and ``tpr_gb300.server``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtprgb.so")

OK, EINVAL, ENOMEM, EUNSUPPORTED, ENONFINITE, ETIMEOUT, ECUDA, EBUSY, \
    ENOTFOUND = range(9)
PTPR_KIND, TPR_KIND, CR_KIND, PCR_KIND = range(4)
F32, F64 = 0, 1

_lib = None


class TprError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[tprgb error {code}] {msg}")
        self.code = code


def _declare(L):
    vp, i, sz = C.c_void_p, C.c_int, C.c_size_t
    sig = {
        "tprgb_last_error": (C.c_char_p, []),
        "tprgb_version": (C.c_char_p, []),
        "tprgb_flops": (i, [i, i, i, C.POINTER(i)]),
        "tprgb_ref_workspace_bytes": (i, [i, i, i, i, i, C.POINTER(sz)]),
        "tprgb_ref_solve_device": (i, [i, i, i, i, i, vp, vp, vp, vp, vp, sz,
                                       vp]),
        "tprgb_normalize_device": (i, [i, C.c_int64, vp, vp, vp, vp, vp]),
        "tprgb_ref_solve_device_static": (i, [i, i, i, i, i, vp, vp, vp, vp,
                                              vp]),
        "tprgb_create": (i, [i, i, i, i, C.POINTER(vp)]),
        "tprgb_destroy": (i, [vp]),
        "tprgb_set_system": (i, [vp, vp, vp, vp, vp]),
        "tprgb_solve": (i, [vp, C.POINTER(i)]),
        "tprgb_get_ans": (i, [vp, vp]),
        "tprgb_release_cached": (i, []),
        "tprgb_time_roundtrip": (i, [vp, vp, vp, vp, vp, vp, i,
                                     C.POINTER(C.c_double)]),
        "tprgb_cusparse_gtsv": (i, [i, i, vp, vp, vp, vp, vp,
                                    C.POINTER(C.c_float)]),
    }
    for prec in ("f32", "f64"):
        for f in ("tpr", "ptpr"):
            sig[f"tprgb_{f}_cu_{prec}"] = (i, [vp, vp, vp, vp, i, i])
        for f in ("cr", "pcr"):
            sig[f"tprgb_{f}_cu_{prec}"] = (i, [vp, vp, vp, vp, i])
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    try:
        from . import batch as _batch
        _batch._declare(L)
    except ImportError:
        pass


def load(build_if_missing: bool = True):
    """Load libtprgb.so (building it in-tree first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise TprError(ECUDA, f"{LIB_PATH} is not built")
        from . import build as _build
        _build.build()
    L = C.CDLL(LIB_PATH)
    _declare(L)
    _lib = L
    return L


def last_error() -> str:
    return load().tprgb_last_error().decode()


def check(rc: int) -> None:
    if rc != OK:
        raise TprError(rc, last_error())


def _host(x, dtype):
    arr = np.ascontiguousarray(x, dtype=dtype)
    return arr, arr.ctypes.data_as(C.c_void_p)


class _Solver:
    """State of one reference solver object, backed by a device handle."""
    kind = PTPR_KIND

    def __init__(self, n: int, s: int = 0, dtype=np.float32):
        self.n, self.s = int(n), int(s or n)
        self.dtype = np.dtype(dtype)
        self.prec = F32 if self.dtype == np.float32 else F64
        L = load()
        h = C.c_void_p()
        check(L.tprgb_create(self.kind, self.n, self.s, self.prec,
                             C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.tprgb_destroy(h)
            self._h = None

    def __copy__(self):  # the reference copy constructor re-initialises
        return type(self)(self.n, self.s, self.dtype)

    def set_tridiagonal_system(self, *arrays):
        if len(arrays) == 3:
            a, c, rhs = arrays
            diag = None
        elif len(arrays) == 4:
            a, diag, c, rhs = arrays
        else:
            raise TypeError("set_tridiagonal_system(a, c, rhs) or "
                            "(a, diag, c, rhs)")
        keep = []
        ptrs = []
        for x in (a, diag, c, rhs):
            if x is None:
                ptrs.append(None)
                continue
            arr, p = _host(x, self.dtype)
            if arr.shape != (self.n,):
                raise ValueError(f"expected {self.n} elements, got {arr.shape}")
            keep.append(arr)
            ptrs.append(p)
        check(load().tprgb_set_system(self._h, *ptrs))

    def solve(self) -> int:
        f = C.c_int()
        check(load().tprgb_solve(self._h, C.byref(f)))
        return f.value

    def get_ans(self, x=None):
        """Copy the solution into ``x`` (a writable array of n elements) and
        return 0 as the reference does; with no argument return it."""
        out = np.empty(self.n, self.dtype)
        check(load().tprgb_get_ans(self._h, out.ctypes.data_as(C.c_void_p)))
        if x is None:
            return out
        x[...] = out
        return 0


class PTPR(_Solver):
    kind = PTPR_KIND


class TPR(_Solver):
    kind = TPR_KIND


class CR(_Solver):
    kind = CR_KIND

    def __init__(self, n: int, dtype=np.float32):
        super().__init__(n, n, dtype)


class PCR(_Solver):
    kind = PCR_KIND

    def __init__(self, n: int, dtype=np.float32):
        super().__init__(n, n, dtype)


def _cu(name, a, c, rhs, n, s=None, dtype=np.float32):
    dtype = np.dtype(dtype)
    sfx = "f32" if dtype == np.float32 else "f64"
    arrs = [_host(v, dtype) for v in (a, c, rhs)]
    x = np.empty(n, dtype)
    fn = getattr(load(), f"tprgb_{name}_cu_{sfx}")
    args = [p for _, p in arrs] + [x.ctypes.data_as(C.c_void_p), n]
    if s is not None:
        args.append(s)
    check(fn(*args))
    return x


def tpr_cu(a, c, rhs, n, s, dtype=np.float32):
    """TPR_CU::tpr_cu (src/tpr.cuh:50-57): returns x."""
    return _cu("tpr", a, c, rhs, n, s, dtype)


def ptpr_cu(a, c, rhs, n, s, dtype=np.float32):
    """PTPR_CU::ptpr_cu (src/ptpr.cuh:50-57): returns x."""
    return _cu("ptpr", a, c, rhs, n, s, dtype)


def cr_cu(a, c, rhs, n, dtype=np.float32):
    return _cu("cr", a, c, rhs, n, None, dtype)


def pcr_cu(a, c, rhs, n, dtype=np.float32):
    return _cu("pcr", a, c, rhs, n, None, dtype)
