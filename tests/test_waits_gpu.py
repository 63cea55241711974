"""Bounded device waits: each kind of wait the solver kernels use (the
mbarrier wait for a TMA load, the cluster row-exchange wait, the
global-memory barrier between the CTAs of one system) is run on a condition
that never comes true.  It must give up, record TPRGB_ETIMEOUT with its
site, and leave the context usable: a batch solved right after still meets
the refined solver's 1e-9 bound.  Nothing faults or hangs; the waits just
run out (the third after its fixed limit of about a second)."""
import ctypes
import time

import pytest

import tpr_gb300 as T
from tpr_gb300 import batch as B
from tpr_gb300 import generate as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which,site,detail", [(0, 0, 0), (1, 1, 0), (2, 2, 7)])
def test_wait_gives_up_and_reports(cuda, port, which, site, detail):
    st = (ctypes.c_uint * 3)()
    t0 = time.perf_counter()
    assert T.load().tprgb_selftest_wait_timeout(which, 1 << 14, st) == T.OK
    waited = time.perf_counter() - t0
    # 2^14 polls: about 0.06 s; the global barrier's fixed limit: about 1.1 s
    assert waited < 5.0, waited
    assert st[0] == T.ETIMEOUT
    assert st[1] == site
    assert st[2] == detail
    bt = G.uniform_batch(8, 1024, 11 + which, "dominant")
    x = B.solve_host(bt, refine_steps=1)
    truth = port.batch_thomas(bt)
    worst, _ = port.batch_rel_l2(bt, x, truth)
    assert worst <= 1e-9, worst


def test_selftest_rejects_bad_arguments(cuda):
    st = (ctypes.c_uint * 3)()
    L = T.load()
    assert L.tprgb_selftest_wait_timeout(3, 16, st) == T.EINVAL
    assert L.tprgb_selftest_wait_timeout(0, 0, st) == T.EINVAL
    assert L.tprgb_selftest_wait_timeout(0, 16, None) == T.EINVAL
