"""Front ends: the tpr_pm-compatible CLI and the GPU stability harness
(the reference's nstab) against the oracle."""
import numpy as np
import pytest

from tpr_gb300 import nstab, pm

pytestmark = pytest.mark.gpu


def test_nstab_matches_oracle(cuda, port, golden):
    lines = []
    rows = nstab.run(npz="tests/golden/nstab.npz", out=lines.append)
    assert len(rows) == 20 * (2 * 6 + 1) and len(lines) == len(rows)
    z = np.load("tests/golden/nstab.npz")
    xt = z["xt"]
    for name, solver, n, s, err in rows:
        if solver == "PCR" or s not in (16, 64, 512):
            continue
        k = name[2:-4]
        x = golden[f"nstab_eq{k}_{solver.lower()}_s{s}_f32"]
        ref = nstab.norm(x, xt)
        assert (np.isnan(ref) and np.isnan(err)) or ref == err, (name, solver, s)
    # the dominant fixtures are accurate; eq1 (cond ~4e3) loses digits
    good = [r for r in rows if r[0] in ("eq18.txt", "eq19.txt", "eq6.txt")]
    assert all(r[4] < 1e-5 for r in good)


def test_pm_cli(cuda, tmp_path):
    out = tmp_path / "x.csv"
    for solver in ("ptpr", "tpr", "pcr", "cuptpr", "cutpr"):
        times, x = pm.run(1024, 128, 3, solver, str(out))
        assert len(times) == 3 and np.isfinite(x).all()
        vals = np.array(out.read_text().strip().split(","), np.float64)
        assert vals.shape == (1024,)
    times, x = pm.run(1024, 128, 64, "batch")
    assert len(times) == 64
    times, x = pm.run(1024, 128, 3, "cusparse", str(out))
    assert len(times) == 3 and np.isfinite(x).all() and min(times) > 0


def test_cusparse_comparator(cuda, port, ans1024):
    """The cuSPARSE gtsv2_nopivot comparison solver (the reference's
    "cusparse" benchmark option) on the reference's fixed N=1024 system and
    a random dominant one."""
    import ctypes
    import tpr_gb300 as T
    from tpr_gb300 import generate as G
    L = T.load()
    n = 1024
    a, diag, c, rhs = (v.astype(np.float32) for v in G.fixed_system(n))
    x = np.empty(n, np.float32)
    ms = ctypes.c_float()
    ptr = lambda v: v.ctypes.data_as(ctypes.c_void_p)
    T.check(L.tprgb_cusparse_gtsv(T.F32, n, ptr(a), None, ptr(c), ptr(rhs),
                                  ptr(x), ctypes.byref(ms)))
    ans = ans1024
    # the reference's known-answer tolerances (test/examples.cpp:36-56)
    assert np.all(np.abs(x - ans) <= 1e-2)
    assert np.max((x - ans) ** 2) <= 1e-3
    assert ms.value > 0
    bt = G.batch(np.array([4096]), 3, "dominant")
    for prec, dt, tol in ((T.F32, np.float32, 1e-5), (T.F64, np.float64, 1e-12)):
        av, bv, cv, dv = (v.astype(dt) for v in (bt.a, bt.b, bt.c, bt.d))
        xv = np.empty(4096, dt)
        T.check(L.tprgb_cusparse_gtsv(prec, 4096, ptr(av), ptr(bv), ptr(cv),
                                      ptr(dv), ptr(xv), None))
        worst, _ = port.batch_rel_l2(bt, xv.astype(np.float64),
                                     port.batch_thomas(bt))
        assert worst <= tol, (prec, worst)
