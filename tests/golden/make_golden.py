"""Regenerate the golden fixtures in this directory.

Run where the reference tree is present: TPR_REFERENCE_ROOT names it
(default: a `reference` directory beside this repository's root):

    TPR_REFERENCE_ROOT=<reference tree> python tests/golden/make_golden.py

It writes
  ans1024.npy      the reference's known answer test/ans1024.txt (solution
                   of the fixed N=1024 system a=c=-1/6, b=1, rhs=i+1)
  nstab.npz        the tridiagonal bands of the reference's 20 stability
                   fixtures src/inputs/eq{1..20}.txt (N=512, dense rows +
                   rhs column), x_t from src/inputs/xt.txt and cond.dat
  ref_outputs.npz  outputs of the reference's own CPU solvers, compiled
                   from its sources by oracle/Makefile (oracle/_ref), on
                   the fixed system, on the seeded N=2048 plain-solve
                   system, and on the stability fixtures

Nothing at test time reads the reference tree; the tests read these files.
"""
from __future__ import annotations

import glob
import hashlib
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tpr_gb300 import generate as G  # noqa: E402

REF = O.REFERENCE_ROOT


def read_ans1024() -> np.ndarray:
    txt = open(os.path.join(REF, "test", "ans1024.txt")).read()
    vals = [float(t) for t in re.split(r"[,\s]+", txt) if t.strip()]
    assert len(vals) == 1024, len(vals)
    return np.array(vals, np.float64)


def read_fixture(path: str, n: int):
    """Bands of one dense-row fixture, read in FP64 as the reference's
    reader does (src/system.cpp:54-116)."""
    a = np.zeros(n)
    diag = np.zeros(n)
    c = np.zeros(n)
    rhs = np.zeros(n)
    with open(path) as f:
        for i in range(n):
            row = np.array(f.readline().strip().split(","), np.float64)
            assert row.shape[0] == n + 1
            if i > 0:
                a[i] = row[i - 1]
            diag[i] = row[i]
            if i < n - 1:
                c[i] = row[i + 1]
            rhs[i] = row[n]
    return a, diag, c, rhs


def digest(*arrs) -> str:
    h = hashlib.sha256()
    for x in arrs:
        h.update(np.ascontiguousarray(x).tobytes())
    return h.hexdigest()


def main() -> None:
    O.build(reference=True)
    r32, r64 = O.ref("f32"), O.ref("f64")
    out = {}

    ans = read_ans1024()
    np.save(os.path.join(HERE, "ans1024.npy"), ans)

    # fixed N=1024 system, reference test sweep s = 4..1024
    # (test/examples.cpp:59-102; the 4-arg setter divides by diag == 1)
    a, diag, c, rhs = G.fixed_system(1024)
    for prec, R in (("f32", r32), ("f64", r64)):
        dt = R.dtype
        af, cf, rf = a.astype(dt), c.astype(dt), rhs.astype(dt)
        out[f"fixed_cr_{prec}"] = R.cr(af, cf, rf)[0]
        out[f"fixed_pcr_{prec}"] = R.pcr(af, cf, rf)[0]
        for s in [4, 8, 16, 32, 64, 128, 256, 512, 1024]:
            out[f"fixed_ptpr_s{s}_{prec}"] = R.ptpr(af, cf, rf, s)[0]
            out[f"fixed_tpr_s{s}_{prec}"] = R.tpr(af, cf, rf, s)[0]

    # seeded plain single-system workload: N=2048, S=512, seed 42
    a, b, c, d, xt = G.one_system(2048, 42, "dominant")
    out["plain_input_sha256"] = np.frombuffer(
        digest(a, b, c, d).encode(), np.uint8)
    P = O.port()
    for prec, R in (("f32", r32), ("f64", r64)):
        an, cn, rn = P.normalize(a, b, c, d, R.dtype)
        for s in [64, 128, 256, 512, 1024, 2048]:
            out[f"plain_ptpr_s{s}_{prec}"] = R.ptpr(an, cn, rn, s)[0]
            out[f"plain_tpr_s{s}_{prec}"] = R.tpr(an, cn, rn, s)[0]

    # stability fixtures, s in {16, 64, 512}, FP32
    # (src/numerical_stability.cpp:172-195)
    files = sorted(glob.glob(os.path.join(REF, "src", "inputs", "eq*.txt")),
                   key=lambda p: int(re.findall(r"\d+", os.path.basename(p))[0]))
    bands = {}
    for path in files:
        k = int(re.findall(r"\d+", os.path.basename(path))[0])
        a, diag, c, rhs = read_fixture(path, 512)
        bands[f"eq{k}"] = np.stack([a, diag, c, rhs])
        an, cn, rn = P.normalize(a, diag, c, rhs, np.float32)
        with np.errstate(all="ignore"):
            for s in (16, 64, 512):
                out[f"nstab_eq{k}_ptpr_s{s}_f32"] = r32.ptpr(an, cn, rn, s)[0]
                out[f"nstab_eq{k}_tpr_s{s}_f32"] = r32.tpr(an, cn, rn, s)[0]
    xt = np.loadtxt(os.path.join(REF, "src", "inputs", "xt.txt"))
    cond = np.loadtxt(os.path.join(REF, "src", "inputs", "cond.dat"))
    np.savez_compressed(os.path.join(HERE, "nstab.npz"), xt=xt, cond=cond,
                        **bands)
    np.savez_compressed(os.path.join(HERE, "ref_outputs.npz"), **out)
    print(f"wrote {len(out)} reference outputs, {len(bands)} fixtures")


if __name__ == "__main__":
    main()
