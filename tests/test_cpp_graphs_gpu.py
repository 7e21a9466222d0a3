"""The C++ graph classes (include/gb300_ntt.hpp) driven like src/project.cpp."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_graph_mirror(tmp_path, orc):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    pkg = os.path.join(ROOT, "ntts_on_amd_ai_engines_aie1_gb300")
    exe = str(tmp_path / "graph_mirror")
    subprocess.run(["nvcc", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "graph_mirror.cu"),
                    "-o", exe, "-L", pkg, "-lgb300ntt", f"-Xlinker=-rpath={pkg}"], check=True)
    out = str(tmp_path / "y.bin")
    r = subprocess.run([exe, out], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "graph mirror ok" in r.stdout
    y = np.fromfile(out, dtype=np.int16).reshape(100, 4096)
    # regenerate the program's inputs: std::mt19937_64(20261203) % 12289
    x = np.array([v % 12289 for v in _mt19937_64(20261203, 4096 * 100)], dtype=np.int16).reshape(100, 4096)
    want = orc.Plan(orc.R2_I16_FWD, 4096, 12289, 41)(x)
    assert np.array_equal(y, want)


def _mt19937_64(seed, count):
    """std::mt19937_64 output sequence (the published MT19937-64 recurrence)."""
    n, m = 312, 156
    mt = [0] * n
    mt[0] = seed & 0xFFFFFFFFFFFFFFFF
    for i in range(1, n):
        mt[i] = (6364136223846793005 * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i) & 0xFFFFFFFFFFFFFFFF
    idx = n
    out = []
    upper, lower = 0xFFFFFFFF80000000, 0x7FFFFFFF
    a = 0xB5026F5AA96619E9
    for _ in range(count):
        if idx >= n:
            for i in range(n):
                x = (mt[i] & upper) | (mt[(i + 1) % n] & lower)
                xa = x >> 1
                if x & 1:
                    xa ^= a
                mt[i] = mt[(i + m) % n] ^ xa
            idx = 0
        y = mt[idx]
        idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        out.append(y & 0xFFFFFFFFFFFFFFFF)
    return out
