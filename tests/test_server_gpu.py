"""Serving loop (continuous batching): results alone and in the mix are the
same bits, solutions meet the refined tolerance (relative L2 <= 1e-9 vs the
FP64 Thomas oracle), admission respects the device budget, failures are
statuses."""
import threading

import numpy as np
import pytest

import tpr_gb300 as T
from tpr_gb300 import devgen
from tpr_gb300 import generate as G
from tpr_gb300.server import Server

pytestmark = pytest.mark.gpu


def _req(rng, nmax=24, kmin=8, kmax=14):
    m = int(rng.integers(1, nmax + 1))
    ns = (1 << rng.integers(kmin, kmax + 1, m)).astype(np.int32)
    seeds = rng.integers(1, 2 ** 63, m, dtype=np.int64).astype(np.uint64)
    return ns, seeds


def _solve_alone(ns, seeds, kind="uneven"):
    with Server(budget_bytes=1 << 30) as s:
        t = s.submit_seeded(ns, seeds, kind)
        info = s.wait(t)
        assert info["rc"] == 0
        return s.fetch(t, int(ns.sum())), s.fetch_system(t, int(ns.sum()))


def test_device_generator_matches_host_mirror(cuda):
    rng = np.random.default_rng(1)
    ns, seeds = _req(rng, 6)
    for kind in ("dominant", "uneven"):
        with Server(budget_bytes=1 << 28) as s:
            t = s.submit_seeded(ns, seeds, kind)
            assert s.wait(t)["rc"] == 0
            a, b, c, d = s.fetch_system(t, int(ns.sum()))
        o = 0
        for n, sd in zip(ns, seeds):
            ha, hb, hc, hd = devgen.system(int(n), int(sd), kind)
            for dev, host in ((a, ha), (b, hb), (c, hc), (d, hd)):
                np.testing.assert_array_equal(dev[o:o + n], host)
            o += n


def test_alone_equals_mixed_and_accuracy(cuda, port):
    rng = np.random.default_rng(7)
    target = _req(rng, 16)
    x_alone, sysdata = _solve_alone(*target)
    others = [_req(rng) for _ in range(60)]
    with Server(budget_bytes=2 << 30) as s:
        tickets = []
        for k, r in enumerate(others):
            tickets.append(s.submit_seeded(*r))
            if k == 30:
                tt = s.submit_seeded(*target)   # arrives mid-stream
        infos = [s.wait(t) for t in tickets]
        info = s.wait(tt)
        assert info["rc"] == 0 and all(i["rc"] == 0 for i in infos)
        x_mixed = s.fetch(tt, int(target[0].sum()))
        steps = {i["step"] for i in infos} | {info["step"]}
    np.testing.assert_array_equal(x_alone, x_mixed)
    assert len(steps) >= 1
    # accuracy against FP64 Thomas on the resident system
    a, b, c, d = sysdata
    bt = G.Batch(target[0], a, b, c, d, np.zeros(len(a)))
    truth = port.batch_thomas(bt)
    worst, _ = port.batch_rel_l2(bt, x_mixed, truth)
    assert worst <= 1e-9, worst


def test_host_request_round_trip(cuda, port):
    bt = G.batch([256, 4096, 64, 1024], 5, "uneven")
    x = np.zeros(bt.neq, np.float64)
    with Server(budget_bytes=1 << 28) as s:
        t = s.submit_host(bt.ns, bt.a, bt.b, bt.c, bt.d, x)
        info = s.wait(t)
        assert info["rc"] == 0 and info["neq"] == bt.neq
        s.release(t)
    worst, _ = port.batch_rel_l2(bt, x, port.batch_thomas(bt))
    assert worst <= 1e-9


def test_budget_admission_and_release(cuda):
    """Requests larger in total than the budget all complete; memory in use
    never exceeds the budget; completion steps follow submission order."""
    rng = np.random.default_rng(3)
    budget = 48 << 20            # 2M equations
    reqs = [_req(rng, 64, 11, 13) for _ in range(80)]
    assert sum(int(r[0].sum()) for r in reqs) * 24 > 4 * budget
    with Server(budget_bytes=budget) as s:
        cap = s.stats()["arena_cap_eq"]
        peak = [0]
        stop = threading.Event()

        def watch():
            while not stop.is_set():
                peak[0] = max(peak[0], s.stats()["arena_used_eq"])

        th = threading.Thread(target=watch)
        th.start()
        tickets = [s.submit_seeded(*r) for r in reqs]
        steps = []
        for t in tickets:
            info = s.wait(t)
            assert info["rc"] == 0
            steps.append(info["step"])
            s.release(t)
        stop.set()
        th.join()
        st = s.stats()
    assert peak[0] <= cap
    assert steps == sorted(steps)
    assert st["requests_done"] == len(reqs) and st["arena_used_eq"] == 0


def test_oversized_and_bad_requests(cuda):
    with Server(budget_bytes=1 << 24) as s:
        with pytest.raises(T.TprError) as e:
            s.submit_seeded(np.array([1 << 20], np.int32),
                            np.array([1], np.uint64))
        assert e.value.code == T.EBUSY
        with pytest.raises(T.TprError):
            s.submit_seeded(np.array([100], np.int32), np.array([1], np.uint64))


def test_nonfinite_request_status(cuda):
    bt = G.batch([128, 128], 2, "dominant")
    bt.a[128:], bt.b[128:], bt.c[128:] = 0.0, 0.0, 0.0   # singular system
    x = np.zeros(bt.neq)
    with Server(budget_bytes=1 << 26) as s:
        t = s.submit_host(bt.ns, bt.a, bt.b, bt.c, bt.d, x)
        info = s.wait(t)
    assert info["rc"] == T.ENONFINITE and info["nonfinite_systems"] == 1


def test_load_driver_small(cuda):
    with Server(budget_bytes=1 << 30) as s:
        lat, el, nsys, rc = s.run_load(200, 2000.0, seed=4, max_sys=32)
        det = s.last_detail
    assert rc == 0 and (lat > 0).all() and el > 0 and nsys >= 200
    # queue time and the finishing step's device time both fit inside the
    # latency; every request has equations
    assert (det[:, 0] >= 0).all() and (det[:, 1] > 0).all()
    assert (det[:, 0] + det[:, 1] <= lat + 50.0).all()
    assert (det[:, 2] >= 256).all()


def test_one_step_in_flight_same_bits(cuda):
    rng = np.random.default_rng(21)
    target = _req(rng, 12)
    x_alone, _ = _solve_alone(*target)
    with Server(budget_bytes=1 << 30, max_inflight=1) as s:
        tickets = [s.submit_seeded(*_req(rng)) for _ in range(20)]
        tt = s.submit_seeded(*target)
        assert all(s.wait(t)["rc"] == 0 for t in tickets)
        assert s.wait(tt)["rc"] == 0
        np.testing.assert_array_equal(x_alone,
                                      s.fetch(tt, int(target[0].sum())))
    with pytest.raises(T.TprError) as e:
        Server(budget_bytes=1 << 24, max_inflight=3)
    assert e.value.code == T.EINVAL


def test_routed_and_queue_only_steps(cuda, port):
    """Steps whose size groups go to the staged / cluster kernels and steps
    kept on the queue kernel both meet 1e-9 against FP64 Thomas."""
    rng = np.random.default_rng(33)
    reqs = [_req(rng, 8, 8, 14) for _ in range(6)]
    out = {}
    for routes in (True, False):
        with Server(budget_bytes=1 << 30, kernel_routes=routes) as s:
            ts = [s.submit_seeded(*r) for r in reqs]
            infos = [s.wait(t) for t in ts]
            assert all(i["rc"] == 0 for i in infos)
            out[routes] = [(s.fetch(t, int(r[0].sum())),
                            s.fetch_system(t, int(r[0].sum())))
                           for t, r in zip(ts, reqs)]
    for routes in (True, False):
        for (x, (a, b, c, d)), r in zip(out[routes], reqs):
            bt = G.Batch(r[0], a, b, c, d, np.zeros(len(a)))
            worst, _ = port.batch_rel_l2(bt, x, port.batch_thomas(bt))
            assert worst <= 1e-9, (routes, worst)
