"""The C ABI library builds, loads and exports every symbol that
include/*.h declares.  No compute call: this runs without a GPU."""
import ctypes
import glob
import os
import re

import pytest

from tests.conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        for m in re.finditer(r"TPRGB_API\s+[\w\s\*]+?\b(tprgb_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "tprgb_ref_solve_device" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_no_unexpected_exports(lib):
    """Only tprgb_* symbols are visible (hidden visibility elsewhere)."""
    import subprocess
    from tpr_gb300 import LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH],
                         capture_output=True, text=True).stdout
    ours = [l.split()[-1] for l in out.splitlines() if " T " in l]
    assert ours and all(n.startswith("tprgb_") for n in ours), ours[:10]


def test_error_paths_without_gpu(lib):
    """Argument validation answers with status codes before touching the
    device."""
    from tpr_gb300 import EINVAL
    f = ctypes.c_int()
    assert lib.tprgb_flops(0, 2048, 512, ctypes.byref(f)) == 0
    assert f.value == 4 * (14 * 512 * 9) + 14 * 4 + 9 * 3 + 14 * 4 * 2 + 4 * 4 * 511
    assert lib.tprgb_flops(0, 1000, 8, ctypes.byref(f)) == EINVAL
    assert b"powers of two" in lib.tprgb_last_error()
    sz = ctypes.c_size_t()
    assert lib.tprgb_ref_workspace_bytes(0, 1, 2048, 512, 0, ctypes.byref(sz)) == 0
    assert sz.value == 0  # fits one CTA
    assert lib.tprgb_ref_workspace_bytes(0, 2, 1 << 16, 256, 0, ctypes.byref(sz)) == 0
    assert sz.value == 2 * (3 * 65536 + 3 * 256) * 4
    assert lib.tprgb_ref_workspace_bytes(0, 1, 1024, 3, 0, ctypes.byref(sz)) == EINVAL
    # standalone CR / PCR: none while n fits one CTA (8192 FP32, 4096 FP64),
    # then one set of a, c, rhs per system for CR and two for PCR
    for kind, prec, n, want in [(2, 0, 8192, 0), (3, 1, 4096, 0),
                                (2, 1, 8192, 3 * 8192 * 8),
                                (3, 0, 16384, 6 * 16384 * 4),
                                (3, 1, 1 << 20, 6 * (1 << 20) * 8)]:
        assert lib.tprgb_ref_workspace_bytes(kind, 2, n, 0, prec,
                                             ctypes.byref(sz)) == 0
        assert sz.value == 2 * want, (kind, prec, n)
    assert lib.tprgb_ref_solve_device(9, 1, 1024, 4, 0, None, None, None, None,
                                      None, 0, None) == EINVAL
    assert lib.tprgb_ref_solve_device(0, 1, 1024, 4, 0, None, None, None, None,
                                      None, 0, None) == EINVAL
    assert b"null device pointer" in lib.tprgb_last_error()


def test_cpp_sources_compile_against_headers(tmp_path):
    """The C++ drop-in headers and the C++ test programs compile (syntax and
    types) without a GPU, so a header change that breaks a caller shows up
    on CPU already."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    cuda_inc = None
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "include", "cuda_runtime.h")):
            cuda_inc = os.path.join(root, "include")
    if not gxx or not cuda_inc:
        pytest.skip("g++ or the CUDA headers are absent")
    cpp = os.path.join(ROOT, "tests", "cpp")
    for name in sorted(os.listdir(cpp)):
        if not name.endswith(".cpp"):
            continue
        r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall",
                            "-I" + os.path.join(ROOT, "include"), "-I" + cuda_inc,
                            os.path.join(cpp, name)],
                           capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, f"{name}:\n{r.stderr}"
