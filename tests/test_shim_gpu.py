"""The C++ drop-in header (include/gb300kf/KalmanFitter.hpp): a program
written in the reference driver's shape — its typedefs
(Run/Common/FitData.hpp:26-43), its object construction and its OpenMP fit
loop (Run/GPU/KalmanFitterGPUTest.cu:539-560) and GPU launch arrays
(Run/GPU/Kernels.cu:6-45) — compiles against it, and on the GPU its
per-track fit() calls and its fitBatch() call give bitwise the fits of a
direct kf_fit_batch_host call, with and without surface material."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "driver_fit_loop.cpp"
FLAGS = ["-std=c++17", "-O2", "-fopenmp", "-I", "/usr/local/cuda/include"]


def test_driver_shaped_program_compiles():
    # compile only (no GPU): the header is self-contained C++17
    res = subprocess.run(["g++", *FLAGS, "-fsyntax-only", str(SRC)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


@pytest.mark.gpu
def test_driver_fit_loop_matches_c_abi(kf, tmp_path):
    lib = kf.load()
    libdir = Path(lib._name).parent
    exe = tmp_path / "driver_fit_loop"
    cmd = ["g++", *FLAGS, str(SRC), "-o", str(exe), f"-L{libdir}", "-lgb300kf",
           f"-Wl,-rpath,{libdir}", "-L/usr/local/cuda/lib64", "-lcudart",
           "-Wl,-rpath,/usr/local/cuda/lib64"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "mismatches=0" in res.stdout
