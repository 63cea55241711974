"""Uneven batches and multi-CTA systems through the plan API -- routed by
size to the staged, cluster and persistent queue kernels, or all on the
queue kernel (variant REGISTERS) -- against the FP64 Thomas oracle.
Tolerance: refined <= 1e-9 relative L2 per system, plain FP32 <= 1e-5."""
import numpy as np
import pytest

from tpr_gb300 import batch as B
from tpr_gb300 import generate as G

pytestmark = pytest.mark.gpu


def _check(port, bt, x, tol):
    truth = port.batch_thomas(bt)
    worst, per = port.batch_rel_l2(bt, x, truth)
    assert worst <= tol, (worst, np.argmax(per), bt.ns[np.argmax(per)])
    return worst


@pytest.mark.parametrize("variant", [0, B.REGISTERS])
@pytest.mark.parametrize("nt", [256, 512])
def test_uneven_sizes_refined(cuda, port, nt, variant):
    ns = G.uneven_sizes(300, 4, 14, 21)          # 16 .. 16384
    bt = G.batch(ns, 300, "uneven")
    x, (rc, st, code) = B.solve_plan_host(bt, refine_steps=1,
                                          threads_per_cta=nt, variant=variant)
    assert rc == 0 and code == 0 and not st.any()
    _check(port, bt, x, 1e-9)


def test_uneven_plain_fp32(cuda, port):
    ns = G.uneven_sizes(200, 4, 13, 5)
    bt = G.batch(ns, 900, "uneven")
    x, (rc, _, _) = B.solve_plan_host(bt, refine_steps=0, x_f64=False)
    assert rc == 0 and x.dtype == np.float32
    _check(port, bt, x, 1e-5)


@pytest.mark.parametrize("variant", [0, B.REGISTERS])
@pytest.mark.parametrize("n", [16384, 32768, 65536])
def test_multi_cta_systems(cuda, port, n, variant):
    """Systems split over several CTAs: one thread-block cluster per system
    (routed), or 8..32 queue-kernel CTAs meeting in global scratch."""
    bt = G.uniform_batch(5, n, 40 + n, "uneven")
    info = {}
    x, (rc, st, code) = B.solve_plan_host(bt, refine_steps=1, variant=variant,
                                          info=info)
    assert rc == 0 and code == 0
    assert info["cluster_systems"] == (5 if variant == 0 else 0)
    _check(port, bt, x, 1e-9)


def test_precision_stress_sample(cuda, port):
    """Weakly dominant N=32768 systems (cond up to ~1e4), 2 refinement
    steps, against FP64 Thomas."""
    bt = G.uniform_batch(4, 32768, 3, "weak")
    x, (rc, _, _) = B.solve_plan_host(bt, refine_steps=2)
    assert rc == 0
    _check(port, bt, x, 1e-9)


def test_graph_replay_and_repeat(cuda, port):
    ns = G.uneven_sizes(64, 6, 16, 8)
    bt = G.batch(ns, 64, "uneven")
    x1, _ = B.solve_plan_host(bt, graph=False)
    x2, (rc, _, _) = B.solve_plan_host(bt, graph=True, repeats=3)
    assert rc == 0
    np.testing.assert_array_equal(x1, x2)
    _check(port, bt, x2, 1e-9)


def test_non_contiguous_offsets_and_order(cuda, port):
    """Systems at arbitrary (16-byte aligned) offsets, out of size order."""
    ns = np.array([1024, 64, 8192, 128, 16], np.int32)
    gaps = np.array([12, 0, 4, 100, 8], np.int64)
    offsets = np.zeros(len(ns), np.int64)
    pos = 0
    for k in range(len(ns)):
        pos += int(gaps[k])
        offsets[k] = pos
        pos += int(ns[k])
    ref = G.batch(ns, 77, "dominant")
    a, b, c, d = (np.zeros(pos, np.float32) for _ in range(4))
    b[:] = 1.0
    for k in range(len(ns)):
        o, n, ro = offsets[k], ns[k], ref.offsets[k]
        for dst, src in ((a, ref.a), (b, ref.b), (c, ref.c), (d, ref.d)):
            dst[o:o + n] = src[ro:ro + n]
    bt = G.Batch(ns, a, b, c, d, np.zeros(pos), offsets)
    x, (rc, _, _) = B.solve_plan_host(bt)
    assert rc == 0
    _check(port, bt, x, 1e-9)


def test_non_finite_system_is_flagged(cuda):
    """A singular system yields a per-system status, not a trap."""
    ns = np.array([256, 256, 256], np.int32)
    bt = G.batch(ns, 1, "dominant")
    bt.b[256:512] = 0.0           # zero diagonal ...
    bt.a[256:512] = 0.0
    bt.c[256:512] = 0.0           # ... and no couplings: singular
    x, (rc, st, code) = B.solve_plan_host(bt, refine_steps=1)
    import tpr_gb300 as T
    assert rc == T.ENONFINITE
    assert st.tolist() == [0, 1, 0]
    assert np.isfinite(x[:256]).all() and np.isfinite(x[512:]).all()


def test_routes_by_size(cuda, port):
    """Sizes 2^6..2^16 back to back: sizes whose tile is a cluster tile
    (and all of 8192..65536) on the cluster kernel, the other sizes of
    256..4096 on the staged kernel, 64 and 128 on the queue kernel; one
    launch per routed size plus one queue launch; graph replay gives the
    same bits."""
    ns = G.uneven_sizes(120, 6, 16, 17)
    bt = G.batch(ns, 120, "uneven")
    info = {}
    x, (rc, st, code) = B.solve_plan_host(bt, refine_steps=1, info=info)
    assert rc == 0 and code == 0 and not st.any()
    on_cluster = {n: n >= 8192 or (n >= 2048 and B.tile_for(n)[2] == B.CLUSTER)
                  for n in set(int(v) for v in ns)}
    clus = int(sum(on_cluster[int(n)] for n in ns))
    staged = int(sum((256 <= n <= 4096) and not on_cluster[int(n)] for n in ns))
    assert info["staged_systems"] == staged
    assert info["cluster_systems"] == clus
    assert info["queue_systems"] == len(ns) - staged - clus
    routed_sizes = len(set(int(n) for n in ns if n >= 256))
    assert info["launches"] == routed_sizes + (1 if (ns < 256).any() else 0)
    _check(port, bt, x, 1e-9)
    xg, _ = B.solve_plan_host(bt, refine_steps=1, graph=True, repeats=3)
    np.testing.assert_array_equal(x, xg)
    xp, _ = B.solve_plan_host(bt, refine_steps=0, x_f64=False)
    _check(port, bt, xp, 1e-5)


def test_unaligned_offsets_stay_on_queue(cuda, port):
    """Offsets that are multiples of 4 but not of 32 cannot be loaded as
    tensor-map rows: those systems stay on the queue kernel."""
    ns = np.array([1024, 1024, 8192], np.int32)
    offsets = np.array([4, 1024 + 8, 2048 + 12], np.int64)
    pos = int(offsets[-1] + ns[-1])
    ref = G.batch(ns, 5, "dominant")
    a, b, c, d = (np.zeros(pos, np.float32) for _ in range(4))
    b[:] = 1.0
    for k in range(len(ns)):
        o, n, ro = offsets[k], ns[k], ref.offsets[k]
        for dst, src in ((a, ref.a), (b, ref.b), (c, ref.c), (d, ref.d)):
            dst[o:o + n] = src[ro:ro + n]
    bt = G.Batch(ns, a, b, c, d, np.zeros(pos), offsets)
    info = {}
    x, (rc, _, _) = B.solve_plan_host(bt, info=info)
    assert rc == 0
    assert info["queue_systems"] == 3 and info["launches"] == 1
    _check(port, bt, x, 1e-9)


@pytest.mark.parametrize("n", [512, 16384])
def test_non_finite_routed_system_is_flagged(cuda, n):
    """Per-system status from the staged (512) and cluster (16384) routes."""
    ns = np.array([n, n, n], np.int32)
    bt = G.batch(ns, 2, "dominant")
    bt.a[n:2 * n], bt.b[n:2 * n], bt.c[n:2 * n] = 0.0, 0.0, 0.0
    info = {}
    x, (rc, st, code) = B.solve_plan_host(bt, refine_steps=1, info=info)
    import tpr_gb300 as T
    assert info["queue_systems"] == 0
    assert rc == T.ENONFINITE and code == 0
    assert st.tolist() == [0, 1, 0]
    assert np.isfinite(x[:n]).all() and np.isfinite(x[2 * n:]).all()


def test_plan_rejects_bad_input(cuda):
    import tpr_gb300 as T
    with pytest.raises(T.TprError):
        B.Plan([100])                          # not a power of two
    with pytest.raises(T.TprError):
        B.Plan([64, 64], offsets=[0, 66])      # misaligned offset
