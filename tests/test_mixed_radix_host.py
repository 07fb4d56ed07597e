"""The mixed-radix register FFT of the smooth-size kernels (msf_mixed.cuh),
checked on the host: every register radix and the two-pass split of every
supported length (2^a 3^b 5^c from 16 to 256, and 512) against a direct FP64
DFT, at 1e-5 relative to the largest output."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "md-structure-factor_gb300", "csrc")


def test_mixed_radix_register_fft_matches_dft(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "mixed_radix_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
                    "-I", CSRC, os.path.join(HERE, "native", "mixed_radix_check.cu"), "-o", exe],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    last = r.stdout.strip().splitlines()[-1]
    assert r.returncode == 0, r.stdout[-2000:]
    assert last.startswith("max_rel_err")
    assert float(last.split()[1]) < 1e-5
