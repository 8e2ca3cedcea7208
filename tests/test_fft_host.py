"""The in-register DFTs (radix 2, 3, 4, 5, their composites up to 20, and 17) and
the four-step line plans of every supported line length, compiled for the
host from the same header the kernels use and checked against a plain FP64
DFT (tests/fft_host_check.cu).  No GPU needed; nvcc compiles the host code."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "phase-field-microstructure-evolution_gb300" / "csrc"
TOL = 3e-7  # FP32 round-off of a <= 256-point transform, relative to the largest output


@pytest.fixture(scope="module")
def fft_report(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path_factory.mktemp("fft") / "fft_host_check"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", str(CSRC), str(ROOT / "tests" / "fft_host_check.cu"), "-o",
                    str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    rep = {}
    for line in out.splitlines():
        f = line.split()
        rep[(f[0], int(f[1]))] = [float(v) for v in f[2:]]
    return rep


@pytest.mark.parametrize("radix", [2, 3, 4, 5, 6, 8, 10, 12, 16, 17, 20])
def test_register_dft_matches_fp64(fft_report, radix):
    fwd, inv = fft_report[("dft", radix)]
    assert fwd < TOL and inv < TOL, (radix, fwd, inv)


@pytest.mark.parametrize("length", [4, 8, 12, 16, 24, 32, 40, 48, 51, 64, 80, 96, 100, 102, 128, 160, 192, 200, 256])
def test_line_plan_matches_fp64(fft_report, length):
    (err,) = fft_report[("line", length)]
    assert err < TOL, (length, err)


def test_x_pass_line_of_128_as_8_by_16(fft_report):
    """The x pass factors its 128-point lines (Nx = 256) as 8 x 16, not as the
    plan's 16 x 8."""
    (err,) = fft_report[("xline", 128)]
    assert err < TOL, err
