"""The drop-in for the reference's TSLAE (xflow_gb300/host/xslae_gpu.cpp)
compiles against the reference's own, unchanged headers and links with the
reference's compiled objects in place of XSLAE.o: every TSLAE member the
time loop calls resolves to the GPU implementation.  Needs the reference tree
(XFLOW_REF) and its objects built by `make -C oracle ref REF=$XFLOW_REF`;
skipped otherwise (the program only links, it runs nothing)."""
import glob
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("XFLOW_REF", "")
OBJS = sorted(p for p in glob.glob(os.path.join(ROOT, "oracle", "_ref", "*.o")) if not p.endswith("XSLAE.o"))
LIB = os.path.join(ROOT, "xflow_gb300", "libxflow.so")


@pytest.mark.skipif(not (REF and os.path.isdir(REF) and len(OBJS) >= 10 and os.path.exists(LIB)),
                    reason="needs XFLOW_REF, the reference objects (make -C oracle ref) and libxflow.so")
def test_tslae_drop_in_links_with_the_reference_objects(tmp_path):
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")),
                            "include")
    cuda_lib = os.path.join(os.path.dirname(cuda_inc), "lib64")
    obj = os.path.join(tmp_path, "xslae_gpu.o")
    subprocess.run(["g++", "-std=c++11", "-O2", "-w", "-I" + REF, "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "xflow_gb300", "host"), "-I" + cuda_inc, "-c",
                    os.path.join(ROOT, "xflow_gb300", "host", "xslae_gpu.cpp"), "-o", obj], check=True)
    exe = os.path.join(tmp_path, "tslae_link")
    out = subprocess.run(["g++", "-fopenmp", "-o", exe, os.path.join(ROOT, "tests", "cpp", "tslae_link_main.cpp"), obj]
                         + OBJS + ["-L" + os.path.dirname(LIB), "-lxflow", "-L" + cuda_lib, "-lcudart", "-lz"],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr[-3000:]
