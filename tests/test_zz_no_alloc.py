"""gbntt_batch_execute_noalloc: the batch entry point that allocates no device
memory, for callers that cannot call cudaMalloc while they transform (their
device memory comes from their own allocator, or a device allocation would
stall a latency-bound serving loop).  It must give the same outputs as the
allocating entry points, call after call, and leave the device's free memory
unchanged.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _segments(gb, specs, rng):
    plans, xs = [], []
    for kind, n, q, root, count, dt in specs:
        plans.append(gb.Plan(kind, n, q, root))
        hi = q if q else 30000
        xs.append(torch.from_numpy(rng.integers(0, hi, (count, n)).astype(dt)).cuda())
    return plans, xs


def test_noalloc_batch_matches_existing_entry_point():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    lib = gb.lib()
    lib.gbntt_batch_execute_noalloc.argtypes = [ctypes.POINTER(gb.Segment), ctypes.c_uint32, ctypes.c_void_p]
    assert hasattr(lib, "gbntt_batch_execute_noalloc")
    rng = np.random.default_rng(99)
    specs = [
        (2, 1024, 12289, pow(41, 4, 12289), 333, np.int16),        # radix-4
        (2, 256, 7681, pow(17, 30, 7681), 77, np.int16),           # radix-4, other modulus
        (4, 4096, 998244353, pow(3, (998244353 - 1) // 4096, 998244353), 9, np.int32),   # int32 forward
        (6, 1024, 0, 0, 5, np.int16),                               # bit-reversal: a plain plan launch
    ]
    plans, xs = _segments(gb, specs, rng)
    stream = torch.cuda.current_stream()
    for call in range(2):
        if call == 1:                                     # new inputs for the second call
            plans, xs = plans, [torch.from_numpy(rng.integers(0, max(s[2], 30000), tuple(x.shape)).astype(
                np.int16 if x.dtype == torch.int16 else np.int32)).cuda() for s, x in zip(specs, xs)]
        ys = [torch.full_like(x, 7) for x in xs]
        want = [torch.empty_like(x) for x in xs]
        arr = (gb.Segment * len(specs))()
        for i, (p, x, y) in enumerate(zip(plans, xs, ys)):
            arr[i].plan, arr[i].d_in, arr[i].d_out, arr[i].count = p.handle, x.data_ptr(), y.data_ptr(), x.shape[0]
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = lib.gbntt_batch_execute_noalloc(arr, len(specs), stream.cuda_stream)
        assert rc == 0, lib.gbntt_last_error()
        torch.cuda.synchronize()
        if call == 1:                                     # set-up happened on the first call
            assert torch.cuda.mem_get_info()[0] == free_before
        for p, x, w in zip(plans, xs, want):              # the existing entry point
            p(x, out=w)
        torch.cuda.synchronize()
        for i, (y, w) in enumerate(zip(ys, want)):
            assert torch.equal(y, w), f"segment {i}, call {call}"
    # more segments than the static array holds are refused
    big = (gb.Segment * 17)()
    for i in range(17):
        big[i].plan, big[i].d_in, big[i].d_out, big[i].count = plans[0].handle, xs[0].data_ptr(), ys[0].data_ptr(), 1
    assert lib.gbntt_batch_execute_noalloc(big, 17, stream.cuda_stream) == 1
    assert b"at most 16" in lib.gbntt_last_error()
