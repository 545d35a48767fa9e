"""A C++ program with no Python in between calls the GPU solver through the
C ABI (tests/cpp/box_solve.cpp, over xflow_gb300/host/xf_box_system.h):
xf_create, xf_grid_create, xf_op_create and xf_solve_host on a 32^3
pressure-type system, checked against the program's own restatement of the
reference's Laplace rows; a bad point code must throw the reference's way."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_caller_solves_through_the_c_abi(tmp_path):
    exe = os.path.join(tmp_path, "box_solve")
    lib = os.path.join(ROOT, "xflow_gb300")
    subprocess.run(["g++", "-std=c++11", "-O2", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "xflow_gb300", "host"), os.path.join(ROOT, "tests", "cpp", "box_solve.cpp"),
                    "-L" + lib, "-lxflow", "-Wl,-rpath," + lib, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(out.stdout)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("OK")
