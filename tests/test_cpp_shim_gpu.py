"""The C++ drop-in shim (include/portblas_gb.h): the samples compile with g++
against the blas:: templates alone and verify themselves on the GPU."""
import os
import subprocess

import pytest

from portblas_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _compile(src, out):
    lib_dir = os.path.dirname(build.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           src, "-o", out, "-L", lib_dir, "-lgbblas", f"-Wl,-rpath,{lib_dir}", "-L", os.path.join(CUDA, "lib64"),
           "-lcudart"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_shim_compiles_without_gpu(tmp_path):
    build.build()
    for s in ("gemm.cpp", "gemv.cpp", "blas_ext.cpp", "gemm_grouped.cpp"):
        _compile(os.path.join(ROOT, "samples", s), str(tmp_path / s.replace(".cpp", "")))


@pytest.mark.gpu
@pytest.mark.parametrize("sample", ["gemm", "gemv", "blas_ext", "gemm_grouped"])
def test_shim_samples_run(torch_cuda, tmp_path, sample):
    build.build()
    exe = str(tmp_path / sample)
    _compile(os.path.join(ROOT, "samples", sample + ".cpp"), exe)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
