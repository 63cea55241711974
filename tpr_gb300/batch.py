"""Batched solver entry points (device memory through torch, calls through
the C ABI).

    x = solve(a, b, c, d, n, refine_steps=1)        # torch CUDA tensors
    x = solve_host(batch, refine_steps=1)           # generate.Batch -> numpy

Inputs are raw FP32 systems (a[i] x[i-1] + b[i] x[i] + c[i] x[i+1] = d[i])
laid out back to back; x is FP64 (default) or FP32.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import check, load  # noqa: F401  (load re-exported)

RESID_DF, RESID_F64 = 0, 1


class BatchOpts(C.Structure):
    _fields_ = [("refine_steps", C.c_int), ("residual", C.c_int),
                ("x_f64", C.c_int), ("eq_per_thread", C.c_int),
                ("threads_per_cta", C.c_int), ("variant", C.c_int)]


def _declare(L):
    vp, i = C.c_void_p, C.c_int
    sig = {
        "tprgb_batch_opts_default": (i, [C.POINTER(BatchOpts)]),
        "tprgb_batch_solve": (i, [i, i, vp, vp, vp, vp, vp,
                                  C.POINTER(BatchOpts), vp]),
        "tprgb_host_ctx_create": (i, [C.c_int64, C.POINTER(vp)]),
        "tprgb_host_ctx_destroy": (i, [vp]),
        "tprgb_batch_solve_host": (i, [vp, i, i, vp, vp, vp, vp, vp,
                                       C.POINTER(BatchOpts)]),
        "tprgb_batch_solve_host_async": (i, [vp, i, i, vp, vp, vp, vp, vp,
                                             C.POINTER(BatchOpts)]),
        "tprgb_host_ctx_wait": (i, [vp]),
        "tprgb_diag_pair_to_double": (i, [C.c_int64, vp, vp, vp, vp]),
        "tprgb_tune_set": (i, [i, i, i, i]),
        "tprgb_tune_get": (i, [i, C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
        "tprgb_batch_status": (i, [C.POINTER(C.c_uint), i]),
        "tprgb_selftest_wait_timeout": (i, [i, C.c_uint, C.POINTER(C.c_uint)]),
        "tprgb_tune_clear": (i, []),
        "tprgb_plan_create": (i, [i, vp, vp, C.POINTER(BatchOpts),
                                  C.POINTER(vp)]),
        "tprgb_plan_destroy": (i, [vp]),
        "tprgb_plan_use_graph": (i, [vp, i]),
        "tprgb_plan_execute": (i, [vp, vp, vp, vp, vp, vp, vp]),
        "tprgb_plan_info": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i),
                                C.POINTER(i)]),
        "tprgb_plan_routes": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i),
                                  C.POINTER(i)]),
        "tprgb_plan_status": (i, [vp, vp, C.POINTER(C.c_uint), vp]),
    }
    for name, (res, args) in sig.items():
        if hasattr(L, name):
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args


# kernel variants (tprgb_batch_opts.variant): inputs loaded to registers;
# staged by TMA bulk copies; staged by swizzled tensor-map copies with two
# stages; the same with one stage; one system per thread-block cluster
REGISTERS, STAGED, SWIZZLED, SWIZZLED_ONE, CLUSTER = 1, 2, 3, 4, 5


def opts(refine_steps: int = 1, residual: int = RESID_DF, x_f64: bool = True,
         eq_per_thread: int = 0, threads_per_cta: int = 0,
         variant: int = 0) -> BatchOpts:
    o = BatchOpts()
    check(load().tprgb_batch_opts_default(C.byref(o)))
    o.refine_steps = refine_steps
    o.residual = residual
    o.x_f64 = int(bool(x_f64))
    o.eq_per_thread = eq_per_thread
    o.threads_per_cta = threads_per_cta
    o.variant = variant
    return o


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("tpr_gb300.batch needs a CUDA device")
    return torch


def solve_into(x, a, b, c, d, n: int, o: BatchOpts | None = None,
               stream=None) -> None:
    """Uniform batch on the device: x, a, b, c, d are CUDA tensors; no
    synchronisation."""
    torch = _torch()
    nsys = a.numel() // n
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    check(load().tprgb_batch_solve(nsys, n, a.data_ptr(), b.data_ptr(),
                                   c.data_ptr(), d.data_ptr(), x.data_ptr(),
                                   C.byref(o or opts()), stream))


def solve(a, b, c, d, n: int, refine_steps: int = 1, residual: int = RESID_DF,
          x_f64: bool = True, **tile):
    torch = _torch()
    o = opts(refine_steps, residual, x_f64, **tile)
    x = torch.empty(a.numel(), dtype=torch.float64 if x_f64 else torch.float32,
                    device=a.device)
    solve_into(x, a, b, c, d, n, o)
    return x


def solve_host(batch, refine_steps: int = 1, residual: int = RESID_DF,
               x_f64: bool = True, **tile) -> np.ndarray:
    """Solve a generate.Batch whose systems all have the same size."""
    torch = _torch()
    n = int(batch.ns[0])
    if not np.all(batch.ns == n):
        raise ValueError("solve_host handles uniform batches only")
    dev = [torch.from_numpy(v).cuda() for v in (batch.a, batch.b, batch.c,
                                                  batch.d)]
    x = solve(*dev, n, refine_steps, residual, x_f64, **tile)
    torch.cuda.synchronize()
    return x.cpu().numpy()


class HostContext:
    """Device buffers for the host-array pipeline (tprgb_batch_solve_host)."""

    def __init__(self, chunk_eq: int = 1 << 22):
        self._h = C.c_void_p()
        check(load().tprgb_host_ctx_create(int(chunk_eq), C.byref(self._h)))

    def solve(self, nsys, n, a, b, c, d, x, o: BatchOpts | None = None):
        """a..d, x: host arrays (numpy, ideally pinned), system k at k*n."""
        ptr = lambda v: C.c_void_p(v.ctypes.data if isinstance(v, np.ndarray)
                                   else v.data_ptr())
        check(load().tprgb_batch_solve_host(self._h, nsys, n, ptr(a), ptr(b),
                                            ptr(c), ptr(d), ptr(x),
                                            C.byref(o or opts())))

    def solve_async(self, nsys, n, a, b, c, d, x, o: BatchOpts | None = None):
        """Queue the batch behind earlier ones without waiting; keep a..d
        and x untouched until wait()."""
        ptr = lambda v: C.c_void_p(v.ctypes.data if isinstance(v, np.ndarray)
                                   else v.data_ptr())
        check(load().tprgb_batch_solve_host_async(
            self._h, nsys, n, ptr(a), ptr(b), ptr(c), ptr(d), ptr(x),
            C.byref(o or opts())))

    def wait(self):
        check(load().tprgb_host_ctx_wait(self._h))

    def close(self):
        if self._h is not None and self._h.value:
            load().tprgb_host_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """Uneven batch: systems of any power-of-two sizes at given offsets
    (tprgb_plan_*), routed by size to the staged, cluster or persistent
    queue kernels; variant=REGISTERS keeps every system on the queue
    kernel."""

    def __init__(self, ns, offsets=None, refine_steps: int = 1,
                 residual: int = RESID_DF, x_f64: bool = True,
                 threads_per_cta: int = 0, graph: bool = True,
                 variant: int = 0):
        ns = np.ascontiguousarray(ns, np.int32)
        if offsets is None:
            offsets = np.zeros(len(ns), np.int64)
            if len(ns) > 1:
                offsets[1:] = np.cumsum(ns[:-1], dtype=np.int64)
        offsets = np.ascontiguousarray(offsets, np.int64)
        self.ns, self.offsets = ns, offsets
        self.neq = int((offsets + ns).max()) if len(ns) else 0
        self.x_f64 = x_f64
        o = opts(refine_steps, residual, x_f64, 0, threads_per_cta, variant)
        self._h = C.c_void_p()
        check(load().tprgb_plan_create(len(ns), offsets.ctypes.data,
                                       ns.ctypes.data, C.byref(o),
                                       C.byref(self._h)))
        check(load().tprgb_plan_use_graph(self._h, int(graph)))

    def execute(self, x, a, b, c, d, stream=None):
        torch = _torch()
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        check(load().tprgb_plan_execute(self._h, a.data_ptr(), b.data_ptr(),
                                        c.data_ptr(), d.data_ptr(),
                                        x.data_ptr(), stream))

    def info(self):
        v = [C.c_int() for _ in range(4)]
        check(load().tprgb_plan_info(self._h, *[C.byref(t) for t in v]))
        out = dict(zip(("items", "grid", "multi_cta_systems", "graph"),
                       [t.value for t in v]))
        r = [C.c_int() for _ in range(4)]
        check(load().tprgb_plan_routes(self._h, *[C.byref(t) for t in r]))
        out.update(zip(("staged_systems", "cluster_systems", "queue_systems",
                        "launches"), [t.value for t in r]))
        return out

    def status(self, stream=None):
        """(rc, per-system status array, device code) after an execute."""
        torch = _torch()
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        st = np.zeros(len(self.ns), np.uint32)
        code = C.c_uint()
        rc = load().tprgb_plan_status(self._h, st.ctypes.data, C.byref(code),
                                      stream)
        return rc, st, code.value

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load().tprgb_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_plan_host(batch, refine_steps: int = 1, residual: int = RESID_DF,
                    x_f64: bool = True, threads_per_cta: int = 0,
                    graph: bool = False, repeats: int = 1, variant: int = 0,
                    info: dict | None = None):
    """Solve a generate.Batch (any sizes) through a plan; returns (x, plan
    status tuple); `info` (a dict) receives the plan's info()."""
    torch = _torch()
    p = Plan(batch.ns, batch.offsets, refine_steps, residual, x_f64,
             threads_per_cta, graph, variant)
    if info is not None:
        info.update(p.info())
    dev = [torch.from_numpy(v).cuda() for v in (batch.a, batch.b, batch.c,
                                                  batch.d)]
    x = torch.empty(batch.neq, dtype=torch.float64 if x_f64 else
                    torch.float32, device="cuda")
    for _ in range(repeats):
        p.execute(x, *dev)
    torch.cuda.synchronize()
    st = p.status()
    out = x.cpu().numpy()
    p.close()
    return out, st


def tile_for(n: int):
    """(equations per thread, threads per CTA, variant) used for size n."""
    L, nt, v = C.c_int(), C.c_int(), C.c_int()
    check(load().tprgb_tune_get(n, C.byref(L), C.byref(nt), C.byref(v)))
    return L.value, nt.value, v.value
