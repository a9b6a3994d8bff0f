"""The adjoint's vector-Jacobian products against central finite differences
(CPU; tests/cpp/adjoint_vjp.cpp includes the same header the kernel uses)."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def vjp_report(tmp_path_factory):
    exe = tmp_path_factory.mktemp("adj") / "adjoint_vjp"
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", str(ROOT / "gpukalmanfitter_gb300" / "csrc"),
                    str(ROOT / "tests" / "cpp" / "adjoint_vjp.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}


@pytest.mark.parametrize("name", ["stages", "accept", "transport", "jtapply", "path", "scale",
                                  "bound", "filter", "update", "leg", "smooth", "start", "align",
                                  "polyequiv", "poly", "polyfast", "trigadd"])
def test_vjp_matches_finite_differences(vjp_report, name):
    # worst |analytic - central difference| over the largest gradient component,
    # 20 random points and random output adjoints per primitive
    assert vjp_report[name] < 1e-5, vjp_report
