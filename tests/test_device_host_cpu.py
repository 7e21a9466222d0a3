"""Host-side checks of device.cuh, built with nvcc and run on the CPU: the
compile-time shared-memory layouts (every exchange between register windows
of the persistent kernel's variants with at least 32 threads per polynomial is
free of bank conflicts on both sides, and every padded layout fits its
buffer), and the canonical reduction (x mod q for any int32 x)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run_host_check(tmp_path, name):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if not nvcc:
        pytest.skip("nvcc not found")
    exe = tmp_path / name
    subprocess.run([nvcc, "-std=c++17", os.path.join(ROOT, "tests", "cpp", name + ".cu"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert " 0 failures" in out.stdout


def test_exchange_layouts_conflict_free(tmp_path):
    _run_host_check(tmp_path, "exchange_layouts")


def test_canonical_reduction(tmp_path):
    _run_host_check(tmp_path, "canon_reduce")
