"""The float64 multiply prodover's chain runs on the integer pipe
(pdl_gb300/csrc/prod_int.cuh, `nmul`), compiled for the host and checked
against the CPU's IEEE multiply: 4 M random normal pairs of every exponent
and significands near rounding ties, and 62 K chains of 64 products
(tests/native/nmul_check.cu)."""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent


def test_nmul_is_the_ieee_product(tmp_path):
    if not shutil.which("nvcc"):
        pytest.skip("no nvcc")
    exe = tmp_path / "nmul_check"
    subprocess.run(["nvcc", "-O2", "-std=c++17", "-x", "cu", str(HERE / "native" / "nmul_check.cu"),
                    "-o", str(exe)], check=True, capture_output=True)
    r = subprocess.run([str(exe), "4000000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip() == "0", r.stdout + r.stderr
