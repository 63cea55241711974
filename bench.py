"""Benchmark: the uniform ADI-style batch -- 16384 independent tridiagonal
systems, N = 1024 each, FP32 storage and arithmetic, one FP64-residual-class
refinement step (compensated FP32) so every system meets relative L2 <= 1e-9
against the FP64 Thomas oracle -- solved in one launch per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  value = systems/s over all ranks (inputs resident
in HBM; the 268 MB of inputs exceed the 129 MB L2, so every step streams
from HBM); e2e = the same metric through the host-array C ABI call
(tprgb_batch_solve_host_async per step, then tprgb_host_ctx_wait: pinned
host in, host x out, every step's copies inside the timed region).
Multi-GPU: weak scaling, each rank solves its own 16384 systems, no
collective on the data path (the systems are independent).

--impl reference times the reference algorithm's CPU implementation (PTPR,
FP32, OpenMP over systems, all host threads) on a bounded sample of the same
workload per step (2048 systems, more when few steps are asked for, so that
the timed steps take about a second): the reference's own solvers compiled
from its sources where present (oracle/_ref), else the C restatement (oracle
port, same bits).  The in-arm cpu_baseline times the same 2048-system
samples for --cpu-seconds; plain_single_system adds the N=2048, S=512 single
solve on the GPU beside the reference's CPU PTPR / TPR on the host cores.
At N=1, after the timed region, `rows` adds the other configurations the
reference's benchmark names, measured on this GPU: the uneven batch (4096
systems of 2^U{6..16} through a plan), the precision stress (1024 x 32768,
weakly dominant) and serving (Poisson arrivals, 20000 requests per load);
--no-rows leaves them out.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NSYS, N, SLICE = 16384, 1024, 128
REFINE = 1
ALGO_BYTES_PER_EQ = 16 + 8  # a, b, c, d FP32 in + x FP64 out
METRIC = "systems/s"
# The workload both arms solve (identical in both lines); how each arm
# solves it goes under "solver".
CONFIG = {
    "workload": "uniform ADI batch: 16384 independent tridiagonal systems "
                "x N=1024, FP32 a, b, c, d (a,c~U(-1,1), b=|a|+|c|+U(1,2), "
                "d=A x_t), seeded",
    "nsys_per_gpu": NSYS, "n": N,
    "l2": "inputs 268 MB > 129 MB L2 (no flush needed)",
}
CPU_SAMPLE = 2048  # systems per CPU step (both CPU legs)


def env_rank():
    return (int(os.environ.get("RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons, sampled during a timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, period_ms: int = 20):
        self.index, self.period = index, period_ms
        self.rows, self.proc = [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", f"--loop-ms={self.period}"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def wait_ready(self, timeout_s: float = 3.0):
        """Block until the first sample arrived (nvidia-smi takes a moment
        to start), so that the timed region that follows is sampled."""
        end = time.time() + timeout_s
        while self.proc and not self.rows and time.time() < end:
            time.sleep(0.01)

    def mark(self) -> int:
        return len(self.rows)

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(self.period / 1000.0)
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self, lo: int = 0, hi: int = None):
        """Samples taken between mark() lo and mark() hi, plus the nearest
        one on each side (a short timed region may fall between two)."""
        hi = len(self.rows) if hi is None else hi
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for r in self.rows[max(0, lo - 1):hi + 1]:
            try:
                mhz.append(float(r[0]))
                mx = float(r[1])
                for k, v in zip(names, r[4:8]):
                    if v.lower() == "active":
                        reasons.add(k)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(mhz) if mhz else None,
                "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(mhz)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


PROFILE = os.path.join(ROOT, "profiles", "batch_sw_n1024_full.md")


def profiled_traffic():
    """DRAM bytes (read + write) per launch of the batched kernel, from the
    committed ncu summary of the same workload (profiles/), or None."""
    if not os.path.exists(PROFILE):
        return None
    got = {}
    unit = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9,
            "B": 1.0, "KB": 1e3, "MB": 1e6, "GB": 1e9}
    for line in open(PROFILE):
        for key in ("DRAM read", "DRAM write"):
            if line.startswith(f"| {key} |"):
                v, u = line.split("|")[2].split()
                if u not in unit:
                    return None
                got[key] = float(v) * unit[u]
    if len(got) != 2:
        return None
    return got["DRAM read"] + got["DRAM write"]


def cpu_reference_sample(port_or_ref, bt, nsys_sample, threads):
    """One bounded CPU step: PTPR FP32 (4-arg setter inside) over
    nsys_sample systems, OpenMP over systems with one solver object per
    thread; returns seconds."""
    n = N
    sl = slice(0, nsys_sample * n)
    a, b, c, d = (np.ascontiguousarray(v[sl]) for v in
                  (bt.a, bt.b, bt.c, bt.d))
    t0 = time.perf_counter()
    if hasattr(port_or_ref, "batch_tpr"):
        port_or_ref.batch_tpr(0, nsys_sample, n, SLICE, a, b, c, d, threads)
    else:
        port_or_ref.batch(0, nsys_sample, n, SLICE, a, b, c, d, threads)
    return time.perf_counter() - t0


def cpu_impl():
    from oracle import oracle as O
    r = O.ref("f32")
    if r is not None:
        return r, "reference"
    return O.port(), "port"


def cpu_solver(kind, sample, threads):
    return {"kind": f"reference PTPR, FP32, no refinement ({kind})",
            "s": SLICE, "sample_systems_per_step": sample,
            "threads": threads,
            "parallelism": "OpenMP over systems, one solver object per "
                           "thread (the reference's multi-thread test)"}


def cpu_sample_size(rate, steps):
    """Systems per CPU step: CPU_SAMPLE, raised (in CPU_SAMPLE multiples,
    up to the whole batch) so that the timed steps together take about a
    second at the measured rate."""
    want = rate * 1.0 / max(1, steps)
    k = max(1, min(NSYS // CPU_SAMPLE, int(np.ceil(want / CPU_SAMPLE))))
    return k * CPU_SAMPLE


def plain_row(iters=1000):
    """The plain single-system configuration (N=2048, S=512, FP32, seed
    42): the GPU class path (host arrays in and out, as the reference's
    timed loop, src/pm.cpp:160-194, and the device-only kernel time) beside
    the reference's CPU PTPR / TPR timed the same way on this machine's host
    cores with their solver-internal OpenMP (one thread and all cores)."""
    from tpr_gb300 import workloads as W
    from tpr_gb300 import generate as G
    gpu = W.plain(iters)
    impl, kind = cpu_impl()
    from oracle import oracle as O
    port = O.port()
    a, b, c, d, xt = G.one_system(2048, 42, "dominant")
    an, cn, rn = port.normalize(a, b, c, d)
    cores = os.cpu_count() or 1
    cpu = {"kind": kind, "cores": cores, "iters": iters}
    for kid, name in ((0, "ptpr"), (1, "tpr")):
        res = {}
        for threads in sorted({1, cores}):
            impl.time_plain(kid, an, cn, rn, 512, 10, threads)  # warm-up
            t, x = impl.time_plain(kid, an, cn, rn, 512, iters, threads)
            res[f"us_per_solve_{threads}t"] = t * 1e6 / iters
            res["rel_l2_vs_xt"] = float(
                np.linalg.norm(x.astype(np.float64) - xt) / np.linalg.norm(xt))
        cpu[name] = res
    gpu.pop("workload", None)
    return {"workload": "one system N=2048, S=512, FP32, seed 42, "
                        f"{iters} solves", "gpu": gpu, "cpu_reference": cpu}


def other_rows():
    """The uneven-batch, precision-stress and serving configurations,
    measured after the bench's timed region (compact fields; the full
    records come from python -m tpr_gb300.workloads / serve_bench)."""
    from tpr_gb300 import serve_bench as SB
    from tpr_gb300 import workloads as W
    un = W.uneven()
    un.pop("plan", None)
    pr = W.precision()
    sv = SB.run(20000)
    serving = {"workload": sv["workload"], "saturated": sv["saturated"],
               "loads": [{k: ld[k] for k in ("load", "p50_ms", "p99_ms",
                                             "p99_over_p50", "systems_per_s", "rc")}
                         for ld in sv["loads"]]}
    return {"uneven": un, "precision": pr, "serving": serving}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    from tpr_gb300 import generate as G
    impl, kind = cpu_impl()
    threads = os.cpu_count() or 1
    bt = G.uniform_batch(NSYS, N, 1_000_000, "dominant")
    t = cpu_reference_sample(impl, bt, CPU_SAMPLE, threads)
    sample = cpu_sample_size(CPU_SAMPLE / t, args.steps)
    for _ in range(args.warmup):
        cpu_reference_sample(impl, bt, sample, threads)
    times = [cpu_reference_sample(impl, bt, sample, threads)
             for _ in range(args.steps)]
    total = sum(times)
    value = sample * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "systems/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded generator, dominant)",
        "config": dict(CONFIG),
        "solver": cpu_solver(kind, sample, threads),
        "cpu_baseline": {"value": value, "unit": "systems/s",
                         "cores": threads, "kind": kind,
                         "sample": f"{sample} systems x N={N}, S={SLICE} "
                                   f"per step, {args.steps} steps, OpenMP "
                                   f"over systems"},
        "e2e": {"value": value, "unit": "systems/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def solver_desc(B, n, tuned, world):
    """How this arm solves the workload: the kernel's tile and what plays
    the reference's slice.  The hierarchical solver has no slice size S:
    a thread reduces its chunk of L equations, a warp segment of 32 lanes
    (32 L equations, the in-slice reduction) and the warps of a system
    (the inter-slice system) in turn."""
    L, nt, variant = B.tile_for(n)
    tps = min(nt, n // L)  # threads per system
    return {"kind": "hierarchical TPR, FP32 + 1 refinement step with a "
                    "compensated FP32 (double-float) residual",
            "refine_steps": REFINE, "residual": "compensated FP32",
            "x": "FP64",
            "tile": {"eq_per_thread": L, "threads_per_cta": nt,
                     "variant": variant, "threads_per_system": tps,
                     "systems_per_cta": max(1, nt // tps)},
            "levels_eq": {"thread_chunk": L,
                          "warp_segment": L * min(32, tps),
                          "system": n},
            "tuned_entries": tuned,
            "parallelism": f"replicas x{world}",
            "e2e_host_layout": "a, b, c, d in one pinned block, x pinned; "
                               "chunks of 4 M equations"}


def run_ours(args):
    import torch

    import tpr_gb300 as T
    from tpr_gb300 import batch as B
    from tpr_gb300 import generate as G

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    T.load(build_if_missing=False) if os.path.exists(T.LIB_PATH) else T.load()
    from tpr_gb300 import autotune
    tuned = autotune.apply()

    bt = G.uniform_batch(NSYS, N, 1_000_000 * (rank + 1), "dominant")
    dev = [torch.from_numpy(v).cuda() for v in (bt.a, bt.b, bt.c, bt.d)]
    x = torch.empty(NSYS * N, dtype=torch.float64, device="cuda")
    o = B.opts(refine_steps=REFINE)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def step():
        B.solve_into(x, *dev, N, o, sptr)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    # accuracy gate of the metric: every system vs FP64 Thomas
    from oracle import oracle as O
    port = O.port()
    truth = port.batch_thomas(bt)
    worst, _ = port.batch_rel_l2(bt, x.cpu().numpy(), truth)

    # device-resident timing: two events on the launching stream around the
    # K back-to-back launches (one launch per step).  Events between the
    # launches would add their own gap to every step (measured 2.2 us per
    # step on GB300), so the average launch duration is the timed region
    # divided by K: inter-launch gaps count against the kernel.
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        clk.wait_ready()
        m0 = clk.mark()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(args.steps):
            step()
        t1.record(stream)
        torch.cuda.synchronize()
        m1 = clk.mark()
        if dist:
            dist.barrier()
        total_ms = t0.elapsed_time(t1)

        # end to end through the host-array C ABI call
        # a, b, c, d one after the other in one pinned block (structure of
        # arrays): the pipeline uploads each chunk with one 2D copy
        neq = NSYS * N
        blk = torch.empty(4 * neq, dtype=torch.float32).pin_memory()
        for i, v in enumerate((bt.a, bt.b, bt.c, bt.d)):
            blk[i * neq:(i + 1) * neq].copy_(torch.from_numpy(v))
        pin = [blk[i * neq:(i + 1) * neq] for i in range(4)]
        xh = torch.empty(NSYS * N, dtype=torch.float64).pin_memory()
        ctx = B.HostContext(chunk_eq=1 << 22)
        for _ in range(2):
            ctx.solve(NSYS, N, *pin, xh, o)
        torch.cuda.synchronize()
        e2e_steps = max(3, args.steps // 10)
        if dist:
            dist.barrier()
        # each step queued behind the previous one (the asynchronous host
        # call): step k's downloads overlap step k+1's uploads; every step
        # still uploads its inputs and downloads its x, and the timed
        # region ends when the last x is in host memory
        te = time.perf_counter()
        for _ in range(e2e_steps):
            ctx.solve_async(NSYS, N, *pin, xh, o)
        ctx.wait()
        e2e_s = time.perf_counter() - te
        ctx.close()
    worst_e2e, _ = port.batch_rel_l2(bt, xh.numpy(), truth)

    if dist:
        from tpr_gb300 import replicas
        total_ms, e2e_s, worst, worst_e2e = replicas.aggregate(
            [total_ms, e2e_s, worst, worst_e2e])

    ms_per_step = total_ms / args.steps
    value = world * NSYS / (ms_per_step * 1e-3)
    e2e_value = world * NSYS * e2e_steps / e2e_s
    kernel_ms = total_ms / args.steps  # average launch, gaps included
    algo_bytes = ALGO_BYTES_PER_EQ * NSYS * N
    achieved = algo_bytes / (kernel_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak()

    cpu = plain = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        impl, kind = cpu_impl()
        threads = os.cpu_count() or 1
        sample = CPU_SAMPLE
        cpu_reference_sample(impl, bt, sample, threads)
        reps, spent = 0, 0.0
        while spent < args.cpu_seconds:
            spent += cpu_reference_sample(impl, bt, sample, threads)
            reps += 1
        cpu = {"value": sample * reps / spent, "unit": "systems/s",
               "cores": threads, "kind": kind,
               "sample": f"{reps} steps x {sample} systems of the same "
                         f"workload (N={N}, S={SLICE}, PTPR FP32, no "
                         f"refinement), OpenMP over systems"}
        plain = plain_row()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "systems/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator: a,c~U(-1,1), "
                    "b=|a|+|c|+U(1,2), d=A x_t)",
            "config": dict(CONFIG),
            "solver": solver_desc(B, N, tuned, world),
            "rel_l2_max": worst, "rel_l2_max_e2e": worst_e2e,
            "gb_per_s": achieved,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind,
                         "traffic": profiled_traffic(),
                         "algorithmic_bytes_per_launch": algo_bytes},
            "e2e": {"value": e2e_value, "unit": "systems/s",
                    "h2d_bytes_per_step": 16 * NSYS * N,
                    "d2h_bytes_per_step": 8 * NSYS * N},
            "gpu_launches": args.steps,
            "clocks": clk.summary(m0, m1),
        }
        if cpu:
            line["cpu_baseline"] = cpu
        if plain:
            line["plain_single_system"] = plain
        if world == 1 and not args.no_rows:
            line["rows"] = other_rows()
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-rows", action="store_true",
                   help="leave out the uneven / precision / serving rows")
    args = p.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
