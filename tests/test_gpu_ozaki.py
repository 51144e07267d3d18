"""The bf16 tensor-core digit products of the FP64 profile spectrum
(galario_gb300/csrc/gb_ozaki.cuh), tested on their own by
tests/cpp/ozaki_test.cu: the kernel's per-element integer sums (the eight
levels of every K tile folded into units of 2^-35 and reduced over the K
tiles) against int64 arithmetic, bit for bit (ragged tiles, every digit at
+-64, 32 K tiles), and FP64 products through the digits against long
double (error below 2^-50 of K max|a| max|b|)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_ozaki_level_products(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "ozaki_test")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                    "-I", os.path.join(ROOT, "galario_gb300", "csrc"), "-o", exe,
                    os.path.join(HERE, "cpp", "ozaki_test.cu")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
