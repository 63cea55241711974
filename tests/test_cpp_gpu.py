"""Builds tests/cpp/test_classes.cpp against include/tpr_gb.hpp and
libtprgb.so (float and double `real`) and runs it: the reference's own
example cases through the C++ class surface."""
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("double", [False, True])
def test_cpp_class_surface(cuda, lib, tmp_path, double):
    import tpr_gb300
    ans = np.load(os.path.join(GOLDEN, "ans1024.npy"))
    ans_txt = tmp_path / "ans1024.txt"
    np.savetxt(ans_txt, ans)
    exe = tmp_path / "test_classes"
    cmd = ["g++", "-O2", "-std=c++17", "-pthread",
           "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_classes.cpp"),
           "-o", str(exe), tpr_gb300.LIB_PATH,
           "-Wl,-rpath," + os.path.dirname(tpr_gb300.LIB_PATH)]
    if double:
        cmd.insert(1, "-D_REAL_IS_DOUBLE_")
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe), str(ans_txt)], capture_output=True,
                       text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout


def test_cpp_batched_surface(cuda, lib, tmp_path):
    """tests/cpp/test_batched.cpp: the C++ wrappers of the batched APIs
    (HostPipeline, Plan, Server) against FP64 Thomas in C++, <= 1e-9."""
    import tpr_gb300
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = tmp_path / "test_batched"
    cmd = ["g++", "-O2", "-std=c++17", "-pthread",
           "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(cuda_home, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_batched.cpp"),
           "-o", str(exe), tpr_gb300.LIB_PATH,
           "-L" + os.path.join(cuda_home, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.dirname(tpr_gb300.LIB_PATH)]
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout
