"""The reference harness's quarter-file format, and a driver like its test harness.

The reference streams every polynomial into the AIE array through four PLIOs,
each carrying one quarter of the coefficients (src/project.cpp:111-132,
src/kernels/io_kernels.cc INPUT_KERNEL_INT16 / OUTPUT_KERNEL_INT16, README.md
"Every design is wrapped in the same test harness"):

* ``<folder>/input_data_q{0..3}.txt`` hold four independent streams of
  whitespace-separated integers, one 128-bit PLIO word per line: 8 int16 or
  4 int32 values.  Polynomial i is the concatenation of coefficients
  [i n/4, (i+1) n/4) of stream q0, q1, q2 and q3, in that order.
* ``<folder>/output_data_q{0..3}.txt`` receive the results split the same way.
  The cycle-accurate simulator writes a ``T <time> ns`` line before every block
  of data; such lines are skipped when reading.

``run_dut`` is the harness itself: the design NTT_CONFIG selects
(src/project.cpp:139-157), ITERATIONS polynomials read from the input quarter
files, transformed on the GPU, written back as output quarter files.
"""
import os

import numpy as np

PER_LINE = {np.dtype(np.int16): 8, np.dtype(np.int32): 4}


def _stream(path):
    vals = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or s[0] == "T":          # blank or simulator timestamp line
                continue
            vals.extend(int(t) for t in s.split())
    return np.asarray(vals, dtype=np.int64)


def read_quarters(folder, n, dtype=np.int16, count=None, prefix="input_data"):
    """(count, n) polynomials assembled from the four quarter streams.

    count=None takes every whole polynomial the shortest stream holds.  Values
    are stored like the 16- or 32-bit PLIO lanes (two's-complement wrap)."""
    if n % 4:
        raise ValueError("n must be a multiple of 4")
    qn = n // 4
    streams = [_stream(os.path.join(folder, f"{prefix}_q{k}.txt")) for k in range(4)]
    avail = min(len(s) for s in streams) // qn
    if count is None:
        count = avail
    if count > avail:
        raise ValueError(f"the quarter files hold {avail} polynomials of n = {n}, {count} requested")
    out = np.empty((count, n), dtype=np.int64)
    for k, s in enumerate(streams):
        out[:, k * qn:(k + 1) * qn] = s[:count * qn].reshape(count, qn)
    return out.astype(dtype)


def write_quarters(folder, polys, prefix="output_data", per_line=None):
    """Writes (count, n) polynomials as four quarter files, like the output PLIOs."""
    polys = np.asarray(polys)
    if polys.ndim == 1:
        polys = polys[None, :]
    count, n = polys.shape
    if n % 4:
        raise ValueError("n must be a multiple of 4")
    per_line = per_line or PER_LINE.get(polys.dtype, 8)
    qn = n // 4
    os.makedirs(folder, exist_ok=True)
    for k in range(4):
        flat = polys[:, k * qn:(k + 1) * qn].reshape(-1)
        with open(os.path.join(folder, f"{prefix}_q{k}.txt"), "w") as f:
            for i in range(0, len(flat), per_line):
                f.write(" ".join(str(int(v)) for v in flat[i:i + per_line]) + "\n")


def run_dut(NTT_CONFIG, in_folder, out_folder, ITERATIONS=100, BITREV_N=None, stream=None):
    """graph_dut.init(); graph_dut.run(ITERATIONS); graph_dut.end() of
    src/project.cpp:161-167, with the PLIO quarter files of the harness.
    Returns the (ITERATIONS, n) output array that was written."""
    import torch

    from . import BITREV_N as DEFAULT_BITREV_N
    from . import dut_for_config

    dut = dut_for_config(NTT_CONFIG, BITREV_N or DEFAULT_BITREV_N)
    dt = np.int32 if NTT_CONFIG in (4, 5) else np.int16
    x = read_quarters(in_folder, dut.NTT_LENGTH, dt, ITERATIONS)
    dut.init()
    try:
        d_in = torch.from_numpy(x).cuda()
        d_out = dut.run(ITERATIONS, d_in, torch.empty_like(d_in), stream)
        torch.cuda.synchronize()
        y = d_out.cpu().numpy()
    finally:
        dut.end()
    write_quarters(out_folder, y)
    return y
