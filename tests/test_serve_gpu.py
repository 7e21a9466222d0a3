"""Serving loop: continuous batching of mixed forward/inverse requests of
mixed sizes and storage types; every result equals the same request run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from test_parity_gpu import root_for  # noqa: E402


@pytest.fixture(scope="module")
def gb():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    return gb


def _plans(gb):
    specs = []
    for n in (256, 1024, 4096):
        specs += [(0, n, 12289), (1, n, 12289)]
    for n, q in ((256, 998244353), (4096, 754974721), (65536, 469762049), (2048, 167772161)):
        specs += [(4, n, q), (5, n, q)]
    specs += [(2, 1024, 12289), (9, 1024, 12289), (8, 512, 12289)]
    plans = [gb.Plan(k, n, q, root_for(q, n)) for k, n, q in specs]
    # output options travel with the plan: natural order + n^-1 scaling on an inverse
    specs.append((1, 2048, 12289))
    plans.append(gb.Plan(1, 2048, 12289, root_for(12289, 2048), 0, gb.FLAG_NATURAL_ORDER | gb.FLAG_SCALE_NINV))
    return specs, plans


def test_mix_equals_alone(gb):
    specs, plans = _plans(gb)
    srv = gb.Server(plans, slots=4, device_bytes=64 << 20, max_requests_per_batch=64)
    rng = np.random.default_rng(123)
    reqs = []
    for _ in range(300):                              # buffers first, then one burst of submissions
        i = int(rng.integers(0, len(specs)))
        kind, n, q = specs[i]
        dt = np.int32 if kind in (4, 5) else np.int16
        cnt = int(rng.integers(1, 4))
        h_in = torch.from_numpy(rng.integers(0, q, (cnt, n)).astype(dt)).pin_memory()
        reqs.append((i, h_in, torch.empty_like(h_in).pin_memory()))
    tickets = srv.submit_schedule([r[0] for r in reqs], [r[1] for r in reqs], [r[2] for r in reqs],
                                  [r[1].shape[0] for r in reqs], [0.0] * len(reqs))
    reqs = [r + (t,) for r, t in zip(reqs, tickets)]
    for _, _, _, t in reqs:
        srv.wait(t, 60000)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["refused"] == 0
    assert st["microbatches"] < len(reqs)            # requests were batched together
    assert st["p99_us"] >= st["p50_us"] > 0
    for i, h_in, h_out, _ in reqs:                    # the same request alone
        alone = plans[i](h_in.cuda())
        torch.cuda.synchronize()
        assert torch.equal(alone.cpu(), h_out), specs[i]
    srv.close()


def test_admission_refuses_oversized_and_times_out(gb):
    plan = gb.Plan(0, 1024, 12289, root_for(12289, 1024))
    srv = gb.Server([plan], slots=2, device_bytes=64 << 10)      # 64 KiB arena: 32 polynomials
    big = torch.zeros(64, 1024, dtype=torch.int16).pin_memory()
    t_big = srv.submit(0, big, torch.empty_like(big).pin_memory())
    assert srv.try_wait(t_big, 1000) == 10                        # GBNTT_ERR_ADMISSION
    small = torch.ones(4, 1024, dtype=torch.int16).pin_memory()
    out = torch.empty_like(small).pin_memory()
    srv.wait(srv.submit(0, small, out), 10000)
    assert torch.equal(out, plan(small.cuda()).cpu())
    assert srv.try_wait(10 ** 9, 50) == 9                         # unknown ticket: bounded wait
    srv.close()


def test_open_loop_schedule(gb):
    specs, plans = _plans(gb)
    srv = gb.Server(plans, slots=4)
    rng = np.random.default_rng(9)
    n_req = 2000
    idx = [int(rng.integers(0, 6)) for _ in range(n_req)]          # int16 plans
    ins = [torch.from_numpy(rng.integers(0, 12289, (1, specs[i][1])).astype(np.int16)).pin_memory() for i in range(6)]
    outs = [torch.empty_like(x).pin_memory() for x in ins]
    arrivals = np.cumsum(rng.exponential(20.0, n_req))              # mean 20 us apart
    tickets = srv.submit_schedule(idx, [ins[i] for i in idx], [outs[i] for i in idx], [1] * n_req,
                                  arrivals.tolist())
    srv.drain()
    st = srv.stats()
    assert st["completed"] == n_req
    assert len(tickets) == n_req
    srv.close()


def test_pageable_and_pinned_requests(gb):
    """Pageable buffers go through the copy engine, pinned ones through the
    gather/scatter kernels; a micro-batch may mix both."""
    specs, plans = _plans(gb)
    srv = gb.Server(plans, slots=2)
    rng = np.random.default_rng(77)
    reqs = []
    for k in range(120):
        i = int(rng.integers(0, len(specs)))
        kind, n, q = specs[i]
        dt = np.int32 if kind in (4, 5) else np.int16
        x = rng.integers(0, q, (2, n)).astype(dt)
        if k % 2:
            h_in, h_out = x, np.empty_like(x)
        else:
            h_in = torch.from_numpy(x).pin_memory()
            h_out = torch.empty_like(h_in).pin_memory()
        # the caller keeps both buffers alive until the request completes: a
        # freed pinned tensor goes back to torch's host cache and may be handed
        # out again as another request's buffer while this one is in flight
        reqs.append((i, x, h_in, h_out, srv.submit(i, h_in, h_out)))
    for *_, t in reqs:
        srv.wait(t, 60000)
    for i, x, _, h_out, _ in reqs:
        got = h_out if isinstance(h_out, np.ndarray) else h_out.numpy()
        assert np.array_equal(plans[i](torch.from_numpy(x).cuda()).cpu().numpy(), got), specs[i]
    srv.close()
