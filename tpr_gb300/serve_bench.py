"""Serving benchmark: Poisson streams of seeded solve requests through the
continuous-batching server (tprgb_server_*).

Each request holds U{1..512} systems of size 2^k, k ~ U{8..14}, generated
on the device (uneven generator: b = |a|+|c|+U(0.1,1)), FP32 + one
compensated-residual refinement step, an 8 GiB device budget.  First the
saturated throughput (all requests submitted at once), then Poisson
arrivals at 25 %, 50 % and 90 % of it; p50 / p99 latency per load.

    python -m tpr_gb300.serve_bench [--requests N] [--budget-gib G]
        [--max-step-eq E] [--max-inflight 1|2]
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from .server import Server


def run(nreq: int, budget_gib: float = 8.0, loads=(0.25, 0.5, 0.9),
        seed: int = 11, max_sys: int = 512, max_step_eq: int = 0,
        max_inflight: int = 2, kernel_routes: bool = True):
    out = {"workload": f"{nreq} requests, U{{1..{max_sys}}} systems of "
                       f"N=2^U{{8..14}}, FP32 + 1 refinement, "
                       f"{budget_gib:g} GiB budget, step cap "
                       f"{max_step_eq or 'none'} eq, {max_inflight} step(s) "
                       f"in flight, "
                       f"{'size routes' if kernel_routes else 'queue kernel only'}",
           "loads": []}
    with Server(budget_bytes=int(budget_gib * (1 << 30)),
                max_step_eq=max_step_eq, max_inflight=max_inflight,
                kernel_routes=kernel_routes) as s:
        s.run_load(min(nreq, 64), 0.0, seed=seed + 99, max_sys=max_sys)  # warm
        lat, el, nsys, rc = s.run_load(nreq, 0.0, seed=seed, max_sys=max_sys)
        sat_req = nreq / el
        out["saturated"] = {"requests_per_s": sat_req, "systems_per_s":
                            nsys / el, "elapsed_s": el, "rc": rc,
                            "systems": nsys}
        for f in loads:
            lat, el, nsys, rc = s.run_load(nreq, f * sat_req, seed=seed + 1,
                                           max_sys=max_sys)
            p50, p99 = np.percentile(lat, [50, 99])
            det = s.last_detail
            # where the time goes: queueing vs the finishing step's device
            # time, for the median and the slowest 1 % of requests
            slow = lat >= p99
            out["loads"].append({
                "load": f, "rate_req_per_s": f * sat_req,
                "p50_ms": p50 / 1e3, "p99_ms": p99 / 1e3,
                "p99_over_p50": p99 / p50, "systems_per_s": nsys / el,
                "rc": rc,
                "median_queue_ms": float(np.median(det[:, 0])) / 1e3,
                "median_step_ms": float(np.median(det[:, 1])) / 1e3,
                "slowest1pct": {
                    "queue_ms": float(np.mean(det[slow, 0])) / 1e3,
                    "step_ms": float(np.mean(det[slow, 1])) / 1e3,
                    "meq": float(np.mean(det[slow, 2])) / 1e6},
                "median_meq": float(np.median(det[:, 2])) / 1e6})
        out["stats"] = s.stats()
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--requests", type=int, default=100000)
    p.add_argument("--budget-gib", type=float, default=8.0)
    p.add_argument("--max-step-eq", type=int, default=0)
    p.add_argument("--max-inflight", type=int, default=2, choices=(1, 2))
    p.add_argument("--queue-only", action="store_true",
                   help="every step on the persistent queue kernel")
    a = p.parse_args()
    from . import autotune
    autotune.apply()
    print(json.dumps(run(a.requests, a.budget_gib,
                         max_step_eq=a.max_step_eq,
                         max_inflight=a.max_inflight,
                         kernel_routes=not a.queue_only)), flush=True)


if __name__ == "__main__":
    main()
