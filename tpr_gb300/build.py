"""Build libtprgb.so in-tree with nvcc for sm_103a (GB300).

    python -m tpr_gb300.build            # incremental
    python -m tpr_gb300.build --force    # rebuild everything

Each translation unit compiles in parallel to tpr_gb300/_build/*.o, then one
shared library is linked to tpr_gb300/libtprgb.so.  No cmake, no torch.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtprgb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler",
                 "-fPIC,-fvisibility=hidden", "-I" + INCLUDE, "-I" + CSRC,
                 "--expt-relaxed-constexpr"]

# translation unit -> extra flags
SOURCES = {
    "api.cu": [],
    # reference-semantics kernels: no FMA contraction, IEEE division, so the
    # results match the reference CPU solvers bit for bit
    "ref_kernels.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"],
    "batch_kernels.cu": [],
    "batch_tma.cu": [],
    "batch_sw.cu": [],
    "batch_api.cu": [],
    "plan_kernels.cu": [],
    "gen_kernels.cu": [],
    "server.cu": [],
    "cusparse_cmp.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps(src: str) -> list[str]:
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
            if f.endswith((".cuh", ".h"))]
    hdrs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return [src] + hdrs


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, obj: str, extra: list[str], verbose: bool) -> str:
    cmd = [nvcc()] + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n"
                           f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose: bool = False, jobs: int = 0) -> str:
    os.makedirs(BUILD, exist_ok=True)
    todo = []
    objs = []
    for name, extra in SOURCES.items():
        src = os.path.join(CSRC, name)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        objs.append(obj)
        if force or verbose or _stale(obj, _deps(src)):
            todo.append((src, obj, extra))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or len(todo)) as ex:
            futs = [ex.submit(_compile, s, o, e, verbose) for s, o, e in todo]
            for f in futs:
                log = f.result()
                if verbose and log:
                    sys.stderr.write(log)
    if todo or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + \
              ["-lcudart", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
