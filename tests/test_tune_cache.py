"""The batched path's launch-shape tuner on the CPU (no GPU): the choice of
the fastest candidate from fake timings and the cache file that keeps the
choices across processes (galario_gb300/csrc/gb_tune.h), through a small C++
program built with the host compiler."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_tuner_choice_and_cache_file(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "tune_test"
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "galario_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "tune_test.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok"
    lines = (tmp_path / "sub" / "dir" / "autotune.txt").read_text().splitlines()
    assert lines[0].startswith("NVIDIA_GB300 f32 4096 240 482 684 64 21 1 4096 0 : ")
