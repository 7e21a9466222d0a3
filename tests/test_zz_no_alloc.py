"""gbntt_batch_execute_noalloc: the batch entry point that allocates no device
memory, for callers that cannot call cudaMalloc while they transform (their
device memory comes from their own allocator, or a device allocation would
stall a latency-bound serving loop).  It must give the same outputs as the
allocating entry points, call after call, leave the device's free memory
unchanged, and report a bounded wait that ran out (gbntt_noalloc_status).
This file is collected last on purpose."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

R4 = pow(41, 4, 12289)
SPECS = [  # (kind, n, q, root, count, dtype, flags, in place)
    (2, 1024, 12289, R4, 333, np.int16, 0, False),                                       # radix-4
    (2, 256, 7681, pow(17, 30, 7681), 77, np.int16, 0, False),                           # radix-4, other modulus
    (4, 4096, 998244353, pow(3, (998244353 - 1) // 4096, 998244353), 9, np.int32, 0, False),   # int32 forward
    (0, 1024, 12289, R4, 50, np.int16, 1, False),                                        # canonical radix-2
    (6, 1024, 0, 0, 5, np.int16, 0, False),                    # bit-reversal: a plain plan launch
    (2, 1024, 12289, R4, 0, np.int16, 0, False),               # empty segment: nothing runs
    (0, 512, 12289, pow(41, 8, 12289), 20, np.int16, 0, True), # in place: a plan launch
]
# per call: the descriptor kernel, three persistent launches (int16 lanes,
# int32 lanes, canonical int16), two plan launches (bit-reversal, in place)
LAUNCHES_PER_CALL = 1 + 3 + 2


@pytest.fixture(scope="module")
def gb():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    return gb


def _inputs(rng):
    xs = []
    for kind, n, q, root, count, dt, flags, inplace in SPECS:
        hi = q if q else 30000
        xs.append(torch.from_numpy(rng.integers(0, hi, (count, n)).astype(dt)).cuda())
    return xs


def _segment_array(gb, plans, xs, ys):
    arr = (gb.Segment * len(SPECS))()
    for i, (p, x, y) in enumerate(zip(plans, xs, ys)):
        arr[i].plan, arr[i].d_in, arr[i].d_out, arr[i].count = p.handle, x.data_ptr(), y.data_ptr(), x.shape[0]
    return arr


def test_noalloc_batch_matches_existing_entry_point(gb):
    lib = gb.lib()
    rng = np.random.default_rng(99)
    plans = [gb.Plan(k, n, q, r, 0, fl) for k, n, q, r, _, _, fl, _ in SPECS]
    stream = torch.cuda.current_stream()
    for call in range(2):
        xs = _inputs(rng)                                 # new inputs on every call
        want = [torch.empty_like(x) for x in xs]
        for p, x, w in zip(plans, xs, want):              # the existing entry point
            if x.shape[0]:
                p(x, out=w)
        ys = [x if spec[7] else torch.full_like(x, 7) for spec, x in zip(SPECS, xs)]
        arr = _segment_array(gb, plans, xs, ys)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        c0 = gb.launch_count()
        rc = lib.gbntt_batch_execute_noalloc(arr, len(SPECS), stream.cuda_stream)
        assert rc == 0, lib.gbntt_last_error()
        torch.cuda.synchronize()
        assert gb.launch_count() - c0 == LAUNCHES_PER_CALL
        if call == 1:                                     # set-up happened on the first call
            assert torch.cuda.mem_get_info()[0] == free_before
        gb.noalloc_status()
        for i, (y, w) in enumerate(zip(ys, want)):
            assert torch.equal(y, w), f"segment {i}, call {call}"
    # more segments than the static array holds are refused, before any launch
    big = (gb.Segment * 17)()
    x0, y0 = _inputs(rng)[0], None
    y0 = torch.empty_like(x0)
    for i in range(17):
        big[i].plan, big[i].d_in, big[i].d_out, big[i].count = plans[0].handle, x0.data_ptr(), y0.data_ptr(), 1
    c0 = gb.launch_count()
    assert lib.gbntt_batch_execute_noalloc(big, 17, stream.cuda_stream) == 1
    assert b"at most 16" in lib.gbntt_last_error()
    assert gb.launch_count() == c0


def test_noalloc_timeout_is_reported(gb):
    """A tile-load wait that runs out (a limit of 0 polls, no fault) is reported
    by gbntt_noalloc_status, which clears it; the next call is correct."""
    lib = gb.lib()
    rng = np.random.default_rng(7)
    plans = [gb.Plan(k, n, q, r, 0, fl) for k, n, q, r, _, _, fl, _ in SPECS]
    xs = _inputs(rng)
    want = [torch.empty_like(x) for x in xs]
    for p, x, w in zip(plans, xs, want):
        if x.shape[0]:
            p(x, out=w)
    stream = torch.cuda.current_stream()
    try:
        gb.set_wait_limit(0)
        ys = [torch.full_like(x, 7) if not s[7] else x.clone() for s, x in zip(SPECS, xs)]
        assert lib.gbntt_batch_execute_noalloc(_segment_array(gb, plans, xs, ys), len(SPECS),
                                               stream.cuda_stream) == 0
        torch.cuda.synchronize()
        with pytest.raises(gb.NTTError) as err:
            gb.noalloc_status()
        assert err.value.code == 9                        # GBNTT_ERR_TIMEOUT
    finally:
        gb.set_wait_limit()
    gb.noalloc_status()                                   # cleared by the report
    ys = [x if s[7] else torch.full_like(x, 7) for s, x in zip(SPECS, xs)]
    assert lib.gbntt_batch_execute_noalloc(_segment_array(gb, plans, xs, ys), len(SPECS),
                                           stream.cuda_stream) == 0
    torch.cuda.synchronize()
    gb.noalloc_status()
    for i, (y, w) in enumerate(zip(ys, want)):
        assert torch.equal(y, w), i
