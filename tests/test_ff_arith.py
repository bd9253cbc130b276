"""Float-float arithmetic of the node evaluations (``csrc/pes_ff.cuh``),
compiled for the host and checked against long double: relative errors of
+, *, /, sqrt, cbrt and exp near 2^-46, absolute errors of log, sin, cos,
atan, sin(x)/x and the 2 pi wraps (moduli) near 1e-14 .. 1e-13.  The device
build runs the same source (with a fast reciprocal estimate refined by the same Newton
step); its end-to-end effect is covered by the mixed-plan parity tests."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
BOUNDS = {"add": 2e-14, "mul": 3e-14, "div": 6e-14, "sqrt": 3e-14, "cbrt": 6e-14, "log": 3e-14, "sin": 3e-14,
          "cos": 3e-14, "sinc": 3e-14, "wrap": 1e-12, "wrap_wide": 1e-11, "exp": 6e-14, "atan": 6e-14}


@pytest.fixture(scope="module")
def errors(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("ff") / "ff_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-w", "-o", exe,
                    os.path.join(HERE, "native", "ff_check.cu")], check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}


@pytest.mark.parametrize("name", sorted(BOUNDS))
def test_ff_error_bound(errors, name):
    assert errors[name] <= BOUNDS[name], (name, errors[name])
