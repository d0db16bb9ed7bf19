"""The gathered energy fill (per node and per filling edge, lf_fill.cuh)
against the scattered form, on the host for every registry kernel: same
accumulators, constant term and submodularity flag (CPU only: the check is
compiled with nvcc for the host and nothing runs on a GPU)."""
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "latticeflow_gb300", "csrc")

import pytest


def test_gathered_fill_equals_scattered_fill(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not present")
    exe = tmp_path / "fill_forms_check"
    cmd = [nvcc, "-std=c++17", "-O1", "-I" + CSRC,
           os.path.join(ROOT, "tests", "native", "fill_forms_check.cu"),
           os.path.join(CSRC, "lf_registry.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "0 mismatches" in r.stdout
