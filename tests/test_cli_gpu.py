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
