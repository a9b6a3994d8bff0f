"""The C++ drop-in shim (reference-shaped KalmanFitter API) builds against the
C ABI and gives the same fits as a direct kf_fit_batch_host call."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _compile(kf, out: Path) -> Path:
    lib = kf.load()
    libdir = Path(lib._name).parent
    cmd = ["g++", "-std=c++17", "-O2", "-I", "/usr/local/cuda/include",
           str(ROOT / "tests" / "cpp" / "shim_fit.cpp"), "-o", str(out),
           f"-L{libdir}", "-lgb300kf", f"-Wl,-rpath,{libdir}",
           "-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_shim_compiles(kf, tmp_path):
    # compile only (no GPU): the header is self-contained C++17
    res = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", "/usr/local/cuda/include",
                          str(ROOT / "tests" / "cpp" / "shim_fit.cpp")],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr


@pytest.mark.gpu
def test_shim_matches_c_abi(kf, tmp_path):
    exe = _compile(kf, tmp_path / "shim_fit")
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "mismatches=0" in res.stdout
