"""Host-side logic that needs no GPU: tuning table, generators, fixture
reader, CLI argument handling, replica partitioning edge cases."""
import json
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN
import tpr_gb300 as T
from tpr_gb300 import autotune, devgen
from tpr_gb300 import generate as G
from tpr_gb300 import nstab, pm


def test_tune_table_apply_and_get(lib, tmp_path):
    from tpr_gb300 import batch as B
    lib.tprgb_tune_clear()
    assert B.tile_for(1024) == (16, 64, 4)           # built-in default
    doc = {"device": "TEST-GPU", "tiles": {
        "1024": {"eq_per_thread": 4, "threads_per_cta": 512, "variant": 2},
        "64": {"eq_per_thread": 8, "threads_per_cta": 128, "variant": 1}}}
    p = tmp_path / "t.json"
    p.write_text(json.dumps(doc))
    assert autotune.apply(str(p), device_name="OTHER-GPU") == 0
    assert autotune.apply(str(p), device_name="TEST-GPU") == 2
    assert B.tile_for(1024) == (4, 512, 2)
    assert B.tile_for(64) == (8, 128, 1)
    lib.tprgb_tune_clear()
    assert B.tile_for(1024) == (16, 64, 4)


def test_tune_set_rejects_bad_tiles(lib):
    import tpr_gb300 as T
    assert lib.tprgb_tune_set(1024, 3, 256, 1) == T.EINVAL      # L
    assert lib.tprgb_tune_set(1024, 8, 64, 1) == T.EUNSUPPORTED  # T > nt
    assert lib.tprgb_tune_set(1024, 8, 1024, 2) == T.EINVAL     # staged nt
    assert lib.tprgb_tune_set(1000, 8, 256, 1) == T.EINVAL      # n
    assert lib.tprgb_tune_set(16, 8, 64, 3) == T.EINVAL        # swizzled n < 32
    assert lib.tprgb_tune_set(1024, 16, 512, 4) == T.EINVAL    # swizzled nt
    assert lib.tprgb_tune_set(1024, 16, 128, 1) == T.EINVAL    # L=16 registers
    assert lib.tprgb_tune_set(65536, 16, 128, 5) == T.EINVAL   # 32 CTAs
    assert lib.tprgb_tune_set(1024, 16, 64, 5) == T.EINVAL     # one CTA
    assert lib.tprgb_tune_set(32768, 8, 256, 5) == T.EINVAL    # cluster L
    assert lib.tprgb_tune_set(32768, 16, 256, 5) == T.OK
    assert lib.tprgb_tune_set(65536, 16, 512, 5) == T.OK       # 8 CTAs of 512
    assert lib.tprgb_tune_set(8192, 16, 512, 5) == T.EINVAL    # one CTA of 512
    assert lib.tprgb_tune_set(1024, 16, 64, 4) == T.OK
    lib.tprgb_tune_clear()


def test_committed_table_is_valid():
    path = autotune.TABLE
    if not os.path.exists(path):
        pytest.skip("no tuned table committed")
    doc = json.load(open(path))
    for n, ent in doc["tiles"].items():
        n = int(n)
        assert n & (n - 1) == 0
        assert ent["eq_per_thread"] in (4, 8, 16)
        assert autotune.fits(n, ent["eq_per_thread"], ent["threads_per_cta"],
                             ent.get("variant", 1))
        # the library accepts the entry (checked without a GPU)
        lib = T.load()
        assert lib.tprgb_tune_set(n, ent["eq_per_thread"],
                                  ent["threads_per_cta"],
                                  ent.get("variant", 1)) == T.OK
    T.load().tprgb_tune_clear()


def test_generators_deterministic_and_dominant():
    for kind in G.KINDS:
        a1, b1, c1, d1, x1 = G.one_system(256, 9, kind)
        a2, b2, c2, d2, x2 = G.one_system(256, 9, kind)
        for u, v in ((a1, a2), (b1, b2), (c1, c2), (d1, d2), (x1, x2)):
            np.testing.assert_array_equal(u, v)
        assert a1[0] == 0 and c1[-1] == 0
        assert np.all(np.abs(b1) > np.abs(a1) + np.abs(c1))
    ns = G.uneven_sizes(1000, 6, 16, 1)
    assert set(np.unique(ns)) <= {1 << k for k in range(6, 17)}
    bt = G.batch([64, 128], 3)
    assert bt.neq == 192 and list(bt.offsets) == [0, 64]


def test_device_generator_mirror_properties():
    for kind in ("dominant", "uneven", "weak"):
        a, b, c, d = devgen.system(512, 1234, kind)
        assert a.dtype == np.float32 and a[0] == 0 and c[-1] == 0
        assert np.all(b > np.abs(a) + np.abs(c))
        a2, *_ = devgen.system(512, 1234, kind)
        np.testing.assert_array_equal(a, a2)
        a3, *_ = devgen.system(512, 1235, kind)
        assert not np.array_equal(a, a3)


def test_nstab_reader_matches_bundled_bands(tmp_path):
    z = np.load(os.path.join(GOLDEN, "nstab.npz"))
    a, diag, c, rhs = z["eq18"]
    n = len(a)
    # write the band back in the reference's dense-row format
    rows = []
    for i in range(n):
        row = np.zeros(n + 1)
        if i > 0:
            row[i - 1] = a[i]
        row[i] = diag[i]
        if i < n - 1:
            row[i + 1] = c[i]
        row[n] = rhs[i]
        rows.append(",".join(repr(float(v)) for v in row))
    f = tmp_path / "eq18.txt"
    f.write_text("\n".join(rows) + "\n")
    got = nstab.read_fixture(str(f), n)
    for u, v in zip(got, (a, diag, c, rhs)):
        np.testing.assert_array_equal(u, v)
    assert nstab.norm(z["xt"], z["xt"]) == 0.0


def test_pm_cli_usage_and_unknown_solver(capsys):
    assert pm.main([]) == 1
    assert "Usage" in capsys.readouterr().err
    with pytest.raises(SystemExit):
        pm.run(64, 8, 1, "lapack")


def test_bench_clock_window():
    """bench.py's clock summary covers the samples taken between two marks
    plus the nearest one on each side, and reports throttle reasons seen
    there only."""
    import bench
    clk = bench.ClockSampler(0)
    idle = ["2070", "2070", "500", "Not Active", "Not Active", "Not Active",
            "Not Active", "Not Active"]
    hot = ["1900", "2070", "1300", "Active", "Not Active", "Not Active",
           "Not Active", "Active"]
    clk.rows = [idle, idle, hot, hot, hot, idle, idle]
    s = clk.summary(3, 4)             # rows 2..4 (one before, one after)
    assert s["samples"] == 3
    assert s["sm_mhz"] == 1900.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    s = clk.summary(6, 6)             # a window between two samples
    assert s["samples"] == 2 and s["reasons"] == []
    assert clk.summary()["samples"] == 7


def test_bench_reads_committed_profile_and_peak():
    """bench.py takes roofline.traffic from the committed ncu summary of the
    bench kernel and the peak from the measured-peaks file; both parse, and
    the traffic is the kernel's DRAM bytes (no more than the algorithmic
    24 B per equation, no less than the 16 B of inputs it must read)."""
    import bench
    traffic = bench.profiled_traffic()
    assert traffic is not None
    eq = 16384 * 1024
    assert 16 * eq <= traffic <= 24 * eq, traffic
    peak, kind = bench.measured_peak()
    assert peak > 1000 and kind in ("measured", "fallback")
