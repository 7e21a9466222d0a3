"""The reference harness's quarter-file format (src/project.cpp:111-132,
src/kernels/io_kernels.cc): reading, writing, the C++ header, and the harness
run on the GPU against the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIX = os.path.join(ROOT, "tests", "golden", "quarters")


@pytest.fixture(scope="module")
def qf():
    from ntts_on_amd_ai_engines_aie1_gb300 import quarter_files
    return quarter_files


def _streams(sub):
    out = []
    for k in range(4):
        with open(os.path.join(FIX, sub, f"input_data_q{k}.txt")) as f:
            out.append(np.array([int(t) for t in f.read().split()], dtype=np.int64))
    return out


@pytest.mark.parametrize("sub,n,dt", [("data", 4096, np.int16), ("data_int32", 2048, np.int32)])
def test_read_assembles_quarters(qf, sub, n, dt):
    x = qf.read_quarters(os.path.join(FIX, sub), n, dt)
    assert x.shape == (4, n) and x.dtype == dt
    s = _streams(sub)
    qn = n // 4
    for i in range(4):
        for k in range(4):
            assert np.array_equal(x[i, k * qn:(k + 1) * qn], s[k][i * qn:(i + 1) * qn])
    assert np.array_equal(x[0], np.arange(n))            # the reference's ramp
    with pytest.raises(ValueError):
        qf.read_quarters(os.path.join(FIX, sub), n, dt, count=5)


def test_write_read_round_trip_and_timestamps(qf, tmp_path):
    rng = np.random.default_rng(1)
    for dt, per in ((np.int16, 8), (np.int32, 4)):
        y = rng.integers(np.iinfo(dt).min, np.iinfo(dt).max, (3, 64)).astype(dt)
        d = tmp_path / np.dtype(dt).name
        qf.write_quarters(str(d), y)
        lines = (d / "output_data_q2.txt").read_text().splitlines()
        assert len(lines) == 3 * 16 // per and all(len(l.split()) == per for l in lines)
        assert np.array_equal(qf.read_quarters(str(d), 64, dt, prefix="output_data"), y)
    # the cycle-accurate simulator's timestamp lines are skipped
    d = tmp_path / "ts"
    qf.write_quarters(str(d), np.arange(32, dtype=np.int16)[None])
    for k in range(4):
        p = d / f"output_data_q{k}.txt"
        p.write_text("T 1200 ns\n" + p.read_text())
    assert np.array_equal(qf.read_quarters(str(d), 32, np.int16, prefix="output_data")[0], np.arange(32))


def test_cpp_header_matches(qf, tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    exe = tmp_path / "quarters_io"
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "quarters_io.cpp"), "-o", str(exe)], check=True)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(exe), os.path.join(FIX, "data"), os.path.join(FIX, "data_int32"), str(out)],
                       check=True, capture_output=True, text=True)
    assert r.stdout.split() == ["0", "4095", "0", "2047"]
    for sub, n, dt, pre in (("data", 4096, np.int16, "i16"), ("data_int32", 2048, np.int32, "i32")):
        x = qf.read_quarters(os.path.join(FIX, sub), n, dt)
        assert np.array_equal(qf.read_quarters(str(out), n, dt, prefix=pre), x)
        ref = tmp_path / ("py_" + pre)
        qf.write_quarters(str(ref), x, prefix=pre)
        for k in range(4):      # byte-identical to the Python writer
            assert (out / f"{pre}_q{k}.txt").read_text() == (ref / f"{pre}_q{k}.txt").read_text()


ORACLE_OF_CONFIG = {  # NTT_CONFIG -> (oracle kind, n, q, root, factor)  (src/project.cpp:139-157)
    0: ("R2_I16_FWD", 4096, 12289, 41, 0), 1: ("R2_I16_INV", 4096, 12289, 41, 0),
    2: ("R4_I16_FWD", 4096, 12289, 41, 0), 3: ("R8_I16_STAGE", 4096, 12289, 41, 0),
    4: ("R2_I32_FWD", 2048, 1073707009, 992735929, 0), 5: ("R2_I32_INV", 2048, 1073707009, 992735929, 0),
    6: ("BITREV_I16", 4096, 0, 0, 0), 7: ("FULL_BARRETT_I16", 4096, 12289, 0, 12286)}


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", range(8))
def test_harness_run_matches_oracle(qf, orc, cfg, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    sub = "data_int32" if cfg in (4, 5) else "data"
    kind, n, q, root, factor = ORACLE_OF_CONFIG[cfg]
    y = qf.run_dut(cfg, os.path.join(FIX, sub), str(tmp_path), ITERATIONS=4)
    x = qf.read_quarters(os.path.join(FIX, sub), n, np.int32 if cfg in (4, 5) else np.int16)
    want = orc.Plan(getattr(orc, kind), n, q, root, factor=factor)(x)
    assert np.array_equal(y, want)
    back = qf.read_quarters(str(tmp_path), n, y.dtype, prefix="output_data")
    assert np.array_equal(back, want)
