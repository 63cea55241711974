"""Per-size tile autotuner for the batched solver.

For every power-of-two system size n it times each feasible tile of the
uniform kernel -- equations per thread L in {4, 8}, threads per CTA in
{128, 256, 512, 1024}, threads per system T = n / L <= threads per CTA --
on a synthetic batch of about `eq_per_trial` equations (larger than L2),
with CUDA events, and keeps the fastest.  The winner sets the tile of the
uniform kernel for that size and the equations per thread that the
persistent queue kernel (plans, serving) uses for it.

    python -m tpr_gb300.autotune            # writes tpr_gb300/tuned_tiles.json
    tpr_gb300.autotune.apply()              # loads the table into the library

The table is keyed by the device name, so a table tuned on one GPU model is
not applied on another.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

from . import check, load

PKG = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(PKG, "tuned_tiles.json")
SIZES = [16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192, 16384, 32768,
         65536]
# (equations per thread, threads per CTA, variant: 1 registers, 2 staged,
# 3 swizzled staged with two stages, 4 swizzled with one stage, 5 one
# system per thread-block cluster)
CANDIDATES = [(4, 128, 1), (4, 256, 1), (4, 512, 1), (4, 1024, 1),
              (8, 128, 1), (8, 256, 1), (8, 512, 1), (8, 1024, 1),
              (4, 128, 2), (4, 256, 2), (4, 512, 2),
              (8, 128, 2), (8, 256, 2), (8, 512, 2),
              (8, 64, 3), (8, 128, 3), (8, 256, 3),
              (16, 64, 3), (16, 128, 3), (16, 256, 3),
              (8, 128, 4), (16, 64, 4), (16, 128, 4), (16, 256, 4),
              (16, 64, 5), (16, 128, 5), (16, 256, 5)]
# Cluster CTAs of 512 threads (one per SM: 132 KB of staging) serve
# n = 16384 .. 65536 when asked for explicitly.  They time 10-14 % slower
# than 256 threads alone (n = 65536: 0.195 vs 0.176 ms per 16.8 M equations;
# 32768: 0.158 vs 0.138) and, routed for n = 65536 in the 4096-system uneven
# plan, 7.7 M against 9.25 M systems/s, so they are not candidates.
VARIANT_TAG = {1: "", 2: "s", 3: "w", 4: "w1", 5: "c"}


def fits(n, L, nt, v):
    """Whether tile (L, nt, variant v) serves systems of size n."""
    if v == 5:
        return n % (16 * nt) == 0 and 2 <= n // (16 * nt) <= 16
    return not (n < 2 * L or n // L > nt or (v >= 3 and n < 32))


def _device_name():
    import torch
    return torch.cuda.get_device_name(0)


def time_tile(n, L, nt, variant=1, refine_steps=1, eq_per_trial=1 << 24,
              reps=10, dev_arrays=None):
    """Mean milliseconds per launch of the uniform kernel for one tile."""
    import torch

    from . import batch as B
    nsys = max(1, eq_per_trial // n)
    if dev_arrays is None:
        g = torch.Generator(device="cuda").manual_seed(n)
        a = torch.rand(nsys * n, device="cuda", generator=g) * 2 - 1
        c = torch.rand(nsys * n, device="cuda", generator=g) * 2 - 1
        b = a.abs() + c.abs() + 1.0 + torch.rand(nsys * n, device="cuda",
                                                  generator=g)
        d = torch.rand(nsys * n, device="cuda", generator=g)
    else:
        a, b, c, d = dev_arrays
    x = torch.empty(nsys * n, dtype=torch.float64, device="cuda")
    o = B.opts(refine_steps=refine_steps, eq_per_thread=L, threads_per_cta=nt,
               variant=variant)
    for _ in range(3):
        B.solve_into(x, a, b, c, d, n, o)
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        B.solve_into(x, a, b, c, d, n, o)
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps, nsys


def tune(sizes=SIZES, refine_steps=1, verbose=True):
    import torch
    table = {}
    for n in sizes:
        nsys = max(1, (1 << 24) // n)
        g = torch.Generator(device="cuda").manual_seed(n)
        a = torch.rand(nsys * n, device="cuda", generator=g) * 2 - 1
        c = torch.rand(nsys * n, device="cuda", generator=g) * 2 - 1
        b = a.abs() + c.abs() + 1.0 + torch.rand(nsys * n, device="cuda",
                                                  generator=g)
        d = torch.rand(nsys * n, device="cuda", generator=g)
        best = None
        trials = {}
        for L, nt, v in CANDIDATES:
            if not fits(n, L, nt, v):
                continue
            ms, _ = time_tile(n, L, nt, v, refine_steps,
                              dev_arrays=(a, b, c, d))
            trials[f"{L}x{nt}{VARIANT_TAG[v]}"] = ms
            if best is None or ms < best[3]:
                best = (L, nt, v, ms)
        table[str(n)] = {"eq_per_thread": best[0], "threads_per_cta": best[1],
                         "variant": best[2], "ms": best[3], "systems": nsys,
                         "systems_per_s": nsys / (best[3] * 1e-3),
                         "trials_ms": trials}
        if verbose:
            print(f"n={n:6d}: best L={best[0]} nt={best[1]} v={best[2]} "
                  f"{best[3]:.4f} ms  {trials}", flush=True)
        del a, b, c, d
    return table


def save(table, path=TABLE):
    doc = {"device": _device_name(), "refine_steps": 1, "tiles": table}
    with open(path, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)


def apply(path=TABLE, device_name=None) -> int:
    """Load a tuned table into the library; returns the entries applied."""
    if not os.path.exists(path):
        return 0
    with open(path) as f:
        doc = json.load(f)
    if device_name is None:
        try:
            device_name = _device_name()
        except Exception:
            device_name = None
    if device_name is not None and doc.get("device") != device_name:
        return 0
    L = load()
    k = 0
    for n, ent in doc["tiles"].items():
        check(L.tprgb_tune_set(int(n), int(ent["eq_per_thread"]),
                               int(ent["threads_per_cta"]),
                               int(ent.get("variant", 1))))
        k += 1
    return k


if __name__ == "__main__":
    sizes = [int(v) for v in sys.argv[1:]] or SIZES
    t = tune(sizes)
    save(t)
    print(TABLE)
