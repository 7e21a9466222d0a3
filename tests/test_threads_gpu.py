"""Plans shared by several host threads at once, each on its own stream: the
C ABI's concurrency contract (plans are immutable after creation; the
host-buffer call is serialised per plan; each thread owns its batches)."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from test_parity_gpu import root_for  # noqa: E402

THREADS = 4
ROUNDS = 12


@pytest.fixture(scope="module")
def gb():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    return gb


def test_plans_shared_across_threads(gb):
    # (kind, n, q, count, dtype, flags): canonical radix-2 int16, lane int32,
    # the canonical four-step (several launches per call)
    specs = [(0, 1024, 12289, 300, np.int16, gb.FLAG_CANONICAL), (4, 4096, 998244353, 40, np.int32, 0),
             (4, 1 << 16, 469762049, 3, np.int32, gb.FLAG_CANONICAL)]
    plans = [gb.Plan(k, n, q, root_for(q, n), 0, fl) for k, n, q, _, _, fl in specs]
    host_plan = gb.Plan(2, 256, 7681, root_for(7681, 256), 0, gb.FLAG_CANONICAL)   # shared host-buffer calls
    rng = np.random.default_rng(515)
    inputs, wants, host_in, host_want = [], [], [], []
    for t in range(THREADS):
        xs = [torch.from_numpy(rng.integers(0, q, (c, n)).astype(dt)).cuda() for _, n, q, c, dt, _ in specs]
        inputs.append(xs)
        wants.append([p(x) for p, x in zip(plans, xs)])
        h = rng.integers(0, 7681, (64, 256)).astype(np.int16)
        host_in.append(h)
        host_want.append(host_plan(torch.from_numpy(h).cuda()).cpu().numpy())
    torch.cuda.synchronize()
    errors = []

    def worker(t):
        try:
            stream = torch.cuda.Stream()
            with torch.cuda.stream(stream):                          # this thread's torch work too
                xs = inputs[t]
                ys = [torch.empty_like(x) for x in xs]
                bx = torch.from_numpy(rng_local[t].integers(0, 12289, (500, 1024)).astype(np.int16)).cuda()
                by = torch.empty_like(bx)
                stream.synchronize()
                batch = gb.Batch([(plans[0], bx, by)])               # this thread's own batch
                for r in range(ROUNDS):
                    for p, x, y in zip(plans, xs, ys):
                        y.fill_(0)
                        p.execute(x, y, x.shape[0], stream)
                    batch.execute(stream)
                    ho = np.zeros_like(host_in[t])
                    host_plan.execute_host(host_in[t], ho)
                    stream.synchronize()
                    for i, (y, w) in enumerate(zip(ys, wants[t])):
                        assert torch.equal(y, w), (t, r, i)
                    assert np.array_equal(ho, host_want[t]), (t, r, "host")
                batch.status()
                bw = torch.empty_like(bx)
                plans[0].execute(bx, bw, bx.shape[0], stream)
                stream.synchronize()
                assert torch.equal(by, bw), (t, "batch")
        except Exception as e:   # reported by the main thread
            errors.append(e)

    rng_local = [np.random.default_rng(600 + t) for t in range(THREADS)]
    ts = [threading.Thread(target=worker, args=(t,)) for t in range(THREADS)]
    for th in ts:
        th.start()
    for th in ts:
        th.join()
    assert not errors, errors[0]
    for p in plans:
        p.status()
