"""The compile-time shared-memory layouts of the transform kernels (device.cuh),
checked on the host: every exchange between register windows of the
persistent kernel's variants with at least 32 threads per polynomial is free
of bank conflicts on both sides, and every padded layout fits its buffer."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exchange_layouts_conflict_free(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if not nvcc:
        pytest.skip("nvcc not found")
    exe = tmp_path / "exchange_layouts"
    subprocess.run([nvcc, "-std=c++17", os.path.join(ROOT, "tests", "cpp", "exchange_layouts.cu"), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "0 failures" in out.stdout
