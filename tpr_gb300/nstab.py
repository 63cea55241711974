"""Numerical-stability harness on the GPU solvers
(src/numerical_stability.cpp:172-195).

    python -m tpr_gb300.nstab [--inputs DIR] [--npz FILE]

For every fixture matrix (the reference's dense-row eq*.txt files in DIR,
read in FP64 as src/system.cpp:54-116 does, or the bands of the same
fixtures stored in FILE) it solves with PTPR and TPR for s = 16 .. N and
with PCR, through the 4-argument setter, and prints
"Input,Solver,N,S,relL2" -- relL2 = ||x - x_t||_2 / ||x_t||_2
(src/numerical_stability.cpp:100-115) against the true solution (xt.txt).
Non-finite solutions print as nan/inf as the reference's do.
"""
from __future__ import annotations

import argparse
import glob
import os
import re

import numpy as np

import tpr_gb300 as T


def read_fixture(path: str, n: int):
    a, diag, c, rhs = (np.zeros(n) for _ in range(4))
    with open(path) as f:
        for i in range(n):
            row = np.array(f.readline().strip().split(","), np.float64)
            if i > 0:
                a[i] = row[i - 1]
            diag[i] = row[i]
            if i < n - 1:
                c[i] = row[i + 1]
            rhs[i] = row[n]
    return a, diag, c, rhs


def norm(x, xt) -> float:
    x = np.asarray(x, np.float64)
    xt = np.asarray(xt, np.float64)
    with np.errstate(all="ignore"):
        return float(np.sqrt(np.sum((x - xt) ** 2)) / np.sqrt(np.sum(xt ** 2)))


def fixtures(inputs=None, npz=None):
    if inputs:
        files = sorted(glob.glob(os.path.join(inputs, "eq*.txt")),
                       key=lambda p: int(re.findall(r"\d+", os.path.basename(p))[0]))
        xt = np.loadtxt(os.path.join(inputs, "xt.txt"))
        for p in files:
            yield os.path.basename(p), read_fixture(p, len(xt)), xt
    else:
        z = np.load(npz)
        xt = z["xt"]
        keys = sorted((k for k in z.files if k.startswith("eq")),
                      key=lambda k: int(k[2:]))
        for k in keys:
            yield f"{k}.txt", tuple(z[k]), xt


def run(inputs=None, npz=None, out=print):
    rows = []
    for name, (a, diag, c, rhs), xt in fixtures(inputs, npz):
        n = len(xt)
        a32, d32, c32, r32 = (v.astype(np.float32) for v in (a, diag, c, rhs))
        s = 16
        while s <= n:
            for cls, label in ((T.PTPR, "PTPR"), (T.TPR, "TPR")):
                t = cls(n, s)
                t.set_tridiagonal_system(a32, d32, c32, r32)
                t.solve()
                rows.append((name, label, n, s, norm(t.get_ans(), xt)))
            s *= 2
        p = T.PCR(n)
        p.set_tridiagonal_system(a32, d32, c32, r32)
        p.solve()
        rows.append((name, "PCR", n, 0, norm(p.get_ans(), xt)))
    for r in rows:
        out(f"{r[0]},{r[1]},{r[2]},{r[3]},{r[4]:e}")
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--inputs", help="directory with eq*.txt and xt.txt")
    ap.add_argument("--npz", default=os.path.join(
        os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
        "tests", "golden", "nstab.npz"))
    a = ap.parse_args()
    run(a.inputs, None if a.inputs else a.npz)


if __name__ == "__main__":
    main()
