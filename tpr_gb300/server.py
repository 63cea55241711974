"""Serving loop (continuous batching) over the C ABI (tprgb_server_*).

    srv = Server(budget_bytes=8 << 30, refine_steps=1)
    t = srv.submit_seeded(ns, seeds, kind="uneven")    # systems made on device
    info = srv.wait(t)                                 # latency_us, status...
    x = srv.fetch(t)                                   # FP64 solution
    srv.release(t)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import check, load
from .devgen import KIND


class ServerOpts(C.Structure):
    _fields_ = [("budget_bytes", C.c_size_t), ("max_pending", C.c_int),
                ("refine_steps", C.c_int), ("residual", C.c_int),
                ("threads_per_cta", C.c_int), ("max_step_eq", C.c_longlong),
                ("max_inflight", C.c_int), ("kernel_routes", C.c_int)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("nonfinite_systems", C.c_int),
                ("step", C.c_longlong), ("latency_us", C.c_double),
                ("x_offset", C.c_longlong), ("neq", C.c_longlong),
                ("queue_us", C.c_double), ("step_us", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_longlong) for k in
                ("steps", "requests_done", "systems_done", "equations_done",
                 "pending", "inflight_steps", "arena_used_eq",
                 "arena_cap_eq")]


def _declare(L):
    vp, i, u64 = C.c_void_p, C.c_int, C.c_uint64
    sig = {
        "tprgb_server_opts_default": (i, [C.POINTER(ServerOpts)]),
        "tprgb_server_create": (i, [C.POINTER(ServerOpts), C.POINTER(vp)]),
        "tprgb_server_destroy": (i, [vp]),
        "tprgb_server_submit_seeded": (i, [vp, i, vp, vp, i,
                                           C.POINTER(u64)]),
        "tprgb_server_submit_host": (i, [vp, i, vp, vp, vp, vp, vp, vp,
                                         C.POINTER(u64)]),
        "tprgb_server_wait": (i, [vp, u64, i, C.POINTER(RequestInfo)]),
        "tprgb_server_fetch": (i, [vp, u64, vp]),
        "tprgb_server_fetch_system": (i, [vp, u64, vp, vp, vp, vp]),
        "tprgb_server_release": (i, [vp, u64]),
        "tprgb_server_get_stats": (i, [vp, C.POINTER(ServerStats)]),
        "tprgb_server_run_load": (i, [vp, i, C.c_double, u64, i, i, i, i, i,
                                      vp, vp, C.POINTER(C.c_double),
                                      C.POINTER(C.c_longlong)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


class Server:
    def __init__(self, budget_bytes: int = 8 << 30, refine_steps: int = 1,
                 residual: int = 0, threads_per_cta: int = 256,
                 max_pending: int = 1 << 20, max_step_eq: int = 0,
                 max_inflight: int = 2, kernel_routes: bool = True):
        L = load()
        _declare(L)
        o = ServerOpts()
        check(L.tprgb_server_opts_default(C.byref(o)))
        o.budget_bytes = int(budget_bytes)
        o.refine_steps = refine_steps
        o.residual = residual
        o.threads_per_cta = threads_per_cta
        o.max_pending = max_pending
        o.max_step_eq = max_step_eq
        o.max_inflight = max_inflight
        o.kernel_routes = int(bool(kernel_routes))
        self._h = C.c_void_p()
        self._keep = {}
        check(L.tprgb_server_create(C.byref(o), C.byref(self._h)))

    def submit_seeded(self, ns, seeds, kind: str = "uneven") -> int:
        ns = np.ascontiguousarray(ns, np.int32)
        seeds = np.ascontiguousarray(seeds, np.uint64)
        t = C.c_uint64()
        check(load().tprgb_server_submit_seeded(
            self._h, len(ns), ns.ctypes.data, seeds.ctypes.data, KIND[kind],
            C.byref(t)))
        return t.value

    def submit_host(self, ns, a, b, c, d, x=None) -> int:
        """a..d: float32 host arrays (kept alive until the request is done);
        x: optional float64 array receiving the solution."""
        ns = np.ascontiguousarray(ns, np.int32)
        arrs = [np.ascontiguousarray(v, np.float32) for v in (a, b, c, d)]
        t = C.c_uint64()
        xp = x.ctypes.data if x is not None else None
        check(load().tprgb_server_submit_host(
            self._h, len(ns), ns.ctypes.data, *[v.ctypes.data for v in arrs],
            xp, C.byref(t)))
        self._keep[t.value] = (ns, arrs, x)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1) -> dict:
        info = RequestInfo()
        rc = load().tprgb_server_wait(self._h, ticket, timeout_ms,
                                      C.byref(info))
        out = {f: getattr(info, f) for f, _ in RequestInfo._fields_}
        out["rc"] = rc
        return out

    def fetch(self, ticket: int, neq: int) -> np.ndarray:
        x = np.empty(neq, np.float64)
        check(load().tprgb_server_fetch(self._h, ticket, x.ctypes.data))
        return x

    def fetch_system(self, ticket: int, neq: int):
        arrs = [np.empty(neq, np.float32) for _ in range(4)]
        check(load().tprgb_server_fetch_system(self._h, ticket,
                                               *[v.ctypes.data for v in arrs]))
        return arrs

    def release(self, ticket: int) -> None:
        check(load().tprgb_server_release(self._h, ticket))
        self._keep.pop(ticket, None)

    def stats(self) -> dict:
        s = ServerStats()
        check(load().tprgb_server_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}

    def run_load(self, nreq: int, rate_per_s: float, seed: int = 1,
                 min_sys: int = 1, max_sys: int = 512, kmin: int = 8,
                 kmax: int = 14, kind: str = "uneven"):
        """Poisson load driven from a native thread; returns (latencies_us,
        elapsed_s, systems, rc).  Per request queue time, device time of
        its finishing step and equations are left in ``last_detail``
        (nreq x 3, microseconds / count)."""
        lat = np.zeros(nreq, np.float64)
        detail = np.zeros((nreq, 3), np.float64)
        el = C.c_double()
        nsys = C.c_longlong()
        rc = load().tprgb_server_run_load(
            self._h, nreq, float(rate_per_s), seed, min_sys, max_sys, kmin,
            kmax, KIND[kind], lat.ctypes.data, detail.ctypes.data,
            C.byref(el), C.byref(nsys))
        self.last_detail = detail
        return lat, el.value, nsys.value, rc

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().tprgb_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
