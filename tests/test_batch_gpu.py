"""Persistent batched launches: mixed designs, moduli and lengths in one
launch per storage type, bit-exact against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from test_parity_gpu import root_for  # noqa: E402

SEED = 4242


@pytest.fixture(scope="module")
def gb():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    return gb


SEGS = [
    # (kind, oracle kind, n, q, count, dtype, flags, oracle kwargs)
    (2, 2, 256, 7681, 700, np.int16, 0, {}),
    (2, 2, 256, 10753, 513, np.int16, 0, {}),
    (2, 2, 1024, 12289, 999, np.int16, 0, {}),
    (0, 0, 1024, 12289, 77, np.int16, 0, {}),
    (1, 1, 512, 12289, 65, np.int16, 0, {}),
    (0, 0, 4096, 12289, 9, np.int16, 0, {}),
    (1, 1, 8, 12289, 300, np.int16, 0, {}),
    (8, 8, 4096, 12289, 11, np.int16, 0, {"r8_exact": True}),
    (8, 8, 256, 12289, 37, np.int16, 0, {"r8_exact": True}),
    (2, 2, 16, 12289, 1000, np.int16, 1, {}),
    (4, 4, 4096, 998244353, 13, np.int32, 0, {}),
    (5, 5, 2048, 754974721, 21, np.int32, 0, {}),
    (4, 4, 8192, 469762049, 3, np.int32, 0, {}),
    (5, 5, 4, 167772161, 999, np.int32, 0, {}),
    (6, 6, 1024, 0, 10, np.int16, 0, {}),          # bit-reversal: separate launch
    (3, 3, 512, 12289, 12, np.int16, 0, {}),       # radix-8 stage: separate launch
]


def _make(gb, rng, spec):
    kind, okind, n, q, count, dt, flags, okw = spec
    root = root_for(q, n) if q else 0
    plan = gb.Plan(kind, n, q, root, 0, flags)
    hi = q if q else 30000
    x = rng.integers(-hi if dt == np.int16 else 0, hi, (count, n)).astype(dt)
    want = __import__("oracle.oracle", fromlist=["Plan"]).Plan(okind, n, q, root, **okw)(x)
    if flags & 1:
        want = (want.astype(np.int64) % q).astype(dt)
    return plan, x, want


def test_mixed_batch(gb):
    rng = np.random.default_rng(SEED)
    made = [_make(gb, rng, s) for s in SEGS]
    xs = [torch.from_numpy(x).cuda() for _, x, _ in made]
    ys = [torch.full_like(x, 12345) for x in xs]
    b = gb.Batch([(p, x, y) for (p, _, _), x, y in zip(made, xs, ys)])
    # persistent launches: int16 and int32 lane arithmetic, the canonical int16
    # segment's own; then the bit-reversal and radix-8 stage plan launches
    assert b.launches == 3 + 2
    for rep in range(3):                # the tile counter re-arms itself
        for y in ys:
            y.fill_(12345)
        b.execute()
        torch.cuda.synchronize()
        b.status()
        for i, ((_, _, want), y) in enumerate(zip(made, ys)):
            got = y.cpu().numpy()
            assert np.array_equal(got, want), f"segment {i} ({SEGS[i][:5]}), repetition {rep}"


def test_mixed_batch_graph_replay(gb):
    """The mixed batch (persistent launches, then the bit-reversal and radix-8
    stage plan launches, which are programmatic dependent launches) captured
    in the batch's CUDA graph and replayed."""
    rng = np.random.default_rng(SEED + 5)
    made = [_make(gb, rng, s) for s in SEGS]
    xs = [torch.from_numpy(x).cuda() for _, x, _ in made]
    ys = [torch.full_like(x, 12345) for x in xs]
    b = gb.Batch([(p, x, y) for (p, _, _), x, y in zip(made, xs, ys)])
    s = torch.cuda.Stream()
    for rep in range(3):
        with torch.cuda.stream(s):
            for y in ys:
                y.fill_(12345)
        b.graph_launch(s)
        s.synchronize()
        b.status()
        for i, ((_, _, want), y) in enumerate(zip(made, ys)):
            assert np.array_equal(y.cpu().numpy(), want), f"segment {i} ({SEGS[i][:5]}), replay {rep}"


def test_graph_launch_and_rebind(gb):
    rng = np.random.default_rng(SEED + 1)
    made = [_make(gb, rng, s) for s in SEGS[:4]]
    xs = [torch.from_numpy(x).cuda() for _, x, _ in made]
    ys = [torch.zeros_like(x) for x in xs]
    b = gb.Batch([(p, x, y) for (p, _, _), x, y in zip(made, xs, ys)])
    assert b.launches == 1
    s = torch.cuda.Stream()
    for _ in range(4):
        b.graph_launch(s)
    s.synchronize()
    for (_, _, want), y in zip(made, ys):
        assert np.array_equal(y.cpu().numpy(), want)
    # rebind segment 2 to new buffers; the graph picks the new descriptor up
    x2 = torch.from_numpy(rng.integers(0, 12289, (999, 1024)).astype(np.int16)).cuda()
    y2 = torch.zeros_like(x2)
    b.set_io(2, x2, y2)
    b.graph_launch(s)
    s.synchronize()
    from oracle import oracle
    want2 = oracle.Plan(2, 1024, 12289, root_for(12289, 1024))(x2.cpu().numpy())
    assert np.array_equal(y2.cpu().numpy(), want2)


def test_batch_counts_launches(gb):
    plan = gb.Plan(2, 1024, 12289, root_for(12289, 1024))
    x = torch.zeros(4096, 1024, dtype=torch.int16, device="cuda")
    y = torch.empty_like(x)
    b = gb.Batch([(plan, x, y)])
    c0 = gb.launch_count()
    b.execute()
    torch.cuda.synchronize()
    assert gb.launch_count() == c0 + 1
    el = b.query(4)                       # coefficients per thread chosen by the autotuner
    assert el in (4, 5, 6)
    assert b.tiles == 4096 // (256 >> (10 - el))
    b2 = gb.Batch([(plan, x, y)], flags=1)   # autotuner off
    assert b2.query(4) == 6


def test_autotune_force(gb, monkeypatch):
    """GBNTT_TUNE_FORCE pins the autotuner's choice (used for reproducible profiles)."""
    plan = gb.Plan(2, 1024, 12289, root_for(12289, 1024))
    x = torch.randint(0, 12289, (512, 1024), dtype=torch.int16, device="cuda")
    y = torch.empty_like(x)
    want = plan(x)
    for el in (6, 5, 4):
        monkeypatch.setenv("GBNTT_TUNE_FORCE", f"{el},0")
        b = gb.Batch([(plan, x, y)])
        assert b.query(4) == el and b.query(6) == 256
        y.zero_()
        b.graph_launch()
        torch.cuda.synchronize()
        assert torch.equal(y, want)


@pytest.mark.parametrize("Ls", [(12, 8, 2), (13, 12, 5)])
def test_int32_batch_widths(gb, monkeypatch, Ls):
    """int32 batches: 16 coefficients per thread carry n <= 2^12; a batch with
    n = 2^13 must keep to the 32-coefficient kernel, even when 16 is requested."""
    monkeypatch.setenv("GBNTT_TUNE_FORCE", "4,0")
    q = 998244353
    rng = np.random.default_rng(5 + Ls[0])
    segs, wants = [], []
    for i, L in enumerate(Ls):
        n = 1 << L
        kind = 4 if i % 2 == 0 else 5
        plan = gb.Plan(kind, n, q, root_for(q, n))
        x = torch.from_numpy(rng.integers(0, q, (37, n)).astype(np.int32)).cuda()
        segs.append((plan, x, torch.empty_like(x)))
        wants.append(plan(x))
    b = gb.Batch(segs)
    b.execute()
    torch.cuda.synchronize()
    for (_, _, y), w in zip(segs, wants):
        assert torch.equal(y, w)


def _ragged_r8(gb, rng, flags, count=2000):
    """The ragged radix-8 workload: `count` polynomials of n = 2^U, U uniform
    in 8..12, q = 12289, natural-order output (bit reversal fused)."""
    q = 12289
    U = rng.integers(8, 13, count)
    segs, xs = [], []
    for L in range(8, 13):
        n = 1 << L
        c = int((U == L).sum())
        plan = gb.Plan(8, n, q, pow(41, 4096 // n, q), 0, gb.FLAG_NATURAL_ORDER | flags)
        x = rng.integers(0, q, (c, n)).astype(np.int16)
        xs.append(x)
        d = torch.from_numpy(x).cuda()
        segs.append((plan, d, torch.full_like(d, 777)))
    return segs, xs


@pytest.mark.parametrize("canonical", [False, True])
def test_ragged_radix8_natural_order_one_launch(gb, orc, canonical):
    """2000 ragged radix-8 polynomials with the bit reversal fused, in ONE
    persistent launch, every polynomial against the oracle's radix-8 chain
    (exact multipliers) followed by its bit-reversal unit (reference:
    src/kernels/ntt_r8_kernels.cc:214-404 then bitreverse_kernels.cc:54-143)."""
    rng = np.random.default_rng(SEED + 30 + canonical)
    segs, xs = _ragged_r8(gb, rng, gb.FLAG_CANONICAL if canonical else 0)
    b = gb.Batch(segs)
    assert b.launches == 1
    b.execute()
    torch.cuda.synchronize()
    b.status()
    q = 12289
    for (plan, _, y), x in zip(segs, xs):
        n = x.shape[1]
        root = pow(41, 4096 // n, q)
        want = orc.Plan(orc.R8_I16_FWD, n, q, root, r8_exact=True)(x)
        bo = orc.Plan(orc.BITREV_I16, n)
        want = bo(want)
        if canonical:
            want = want.astype(np.int64) % q
            assert np.array_equal(want, orc.ntt_exact(x, q, root)[:, orc.bitrev_perm(n)])
        assert np.array_equal(y.cpu().numpy().astype(np.int64), want.astype(np.int64)), n


def test_canonical_batch_every_family(gb, orc):
    """Canonical segments of both storage types and directions beside lane
    segments: four persistent launches, each output against the exact transform
    (canonical) or the oracle (lanes)."""
    rng = np.random.default_rng(SEED + 40)
    specs = [  # (kind, n, q, count, dtype, flags)
        (2, 1024, 12289, 300, np.int16, 1), (0, 256, 7681, 201, np.int16, 1), (1, 4096, 12289, 7, np.int16, 1),
        (9, 64, 12289, 99, np.int16, 1 | 0x10), (8, 512, 10753, 45, np.int16, 1 | 0x8),
        (4, 8192, 998244353, 5, np.int32, 1), (5, 4096, 754974721, 19, np.int32, 1 | 0x10),
        (4, 4, 469762049, 1000, np.int32, 1), (5, 1024, 167772161, 66, np.int32, 1 | 0x8),
        (2, 256, 12289, 100, np.int16, 0), (4, 2048, 998244353, 9, np.int32, 0),
    ]
    segs, wants = [], []
    for kind, n, q, count, dt, fl in specs:
        root = root_for(q, n)
        lo, hi = (-32768, 32768) if dt == np.int16 else (-(1 << 31), 1 << 31)
        x = rng.integers(lo, hi, (count, n)).astype(dt) if fl & 1 else rng.integers(0, q, (count, n)).astype(dt)
        d = torch.from_numpy(x).cuda()
        segs.append((gb.Plan(kind, n, q, root, 0, fl), d, torch.full_like(d, 5)))
        inverse = kind in (1, 5, 9)
        if fl & 1:
            xin = np.ascontiguousarray(x[:, orc.bitrev_perm(n)]) if (fl & 0x8 and inverse) else x
            w = orc.ntt_exact(xin, q, root, inverse=inverse)
            if fl & 0x10:
                w = w * pow(n, -1, q) % q
            if fl & 0x8 and not inverse:
                w = w[:, orc.bitrev_perm(n)]
        else:
            w = orc.Plan(kind, n, q, root)(x)
        wants.append(w)
    b = gb.Batch(segs)
    assert b.launches == 4
    for rep in range(2):
        b.graph_launch()
        torch.cuda.synchronize()
        b.status()
        for i, ((_, _, y), w) in enumerate(zip(segs, wants)):
            assert np.array_equal(y.cpu().numpy().astype(np.int64), w.astype(np.int64)), (i, rep)


def test_bounded_wait_timeout_is_reported(gb):
    """A tile load whose bounded wait runs out: the launch records
    GBNTT_ERR_TIMEOUT (the CTA lets its copies in flight land and stops), the
    status call reports and clears it, and the next launch is correct.  The
    wait is made to run out by a limit of 0 polls, not by any fault."""
    rng = np.random.default_rng(SEED + 50)
    plan = gb.Plan(2, 1024, 12289, root_for(12289, 1024))
    cplan = gb.Plan(4, 4096, 998244353, root_for(998244353, 4096), 0, gb.FLAG_CANONICAL)
    x = torch.from_numpy(rng.integers(0, 12289, (2000, 1024)).astype(np.int16)).cuda()
    x32 = torch.from_numpy(rng.integers(0, 998244353, (300, 4096)).astype(np.int32)).cuda()
    y, y32 = torch.zeros_like(x), torch.zeros_like(x32)
    b = gb.Batch([(plan, x, y), (cplan, x32, y32)])
    want, want32 = plan(x), cplan(x32)
    try:
        gb.set_wait_limit(0)
        b.execute()
        torch.cuda.synchronize()
        with pytest.raises(gb.NTTError) as err:
            b.status()
        assert err.value.code == 9              # GBNTT_ERR_TIMEOUT
    finally:
        gb.set_wait_limit()
    b.status()                                  # the error was cleared by the report
    y.zero_()
    y32.zero_()
    b.execute()
    torch.cuda.synchronize()
    b.status()
    assert torch.equal(y, want) and torch.equal(y32, want32)


@pytest.mark.parametrize("force", ["4,6", "4,5", "4,0", "5,0", "5,4", "4,12", "4,10", "5,12"])
def test_canonical_batch_every_configuration(gb, orc, monkeypatch, force):
    """Every compiled canonical int16 configuration, pinned with
    GBNTT_TUNE_FORCE (16 or 32 coefficients per thread, CTAs of 256, 128 or
    64 threads), on a radix-4 / radix-2 batch of n = 256 and 1024, forward and
    inverse: outputs against the exact transform."""
    monkeypatch.setenv("GBNTT_TUNE_FORCE", force)
    rng = np.random.default_rng(SEED + 60)
    segs, wants = [], []
    for kind, n, q, count in ((2, 1024, 12289, 301), (2, 256, 7681, 513), (1, 1024, 12289, 77), (0, 512, 10753, 40)):
        root = root_for(q, n)
        x = rng.integers(-32768, 32768, (count, n)).astype(np.int16)
        d = torch.from_numpy(x).cuda()
        segs.append((gb.Plan(kind, n, q, root, 0, gb.FLAG_CANONICAL), d, torch.full_like(d, 3)))
        wants.append(orc.ntt_exact(x, q, root, inverse=kind == 1))
    b = gb.Batch(segs)
    el, occ = (int(v) for v in force.split(","))
    assert b.query(4) == el and b.query(7) == occ
    b.graph_launch()
    torch.cuda.synchronize()
    b.status()
    for (_, _, y), w in zip(segs, wants):
        assert np.array_equal(y.cpu().numpy().astype(np.int64), w)


def test_many_segments_one_launch_per_part(gb):
    """300 small segments (radix-2/4, forward/inverse, lane and canonical
    arithmetic, n = 16 .. 1024, 1-9 polynomials each, some empty) in one
    persistent launch per part: every CTA finds its first tile's segment and
    later segments by search, not by walking the list; outputs against the
    per-plan launches."""
    rng = np.random.default_rng(SEED + 70)
    plans = {}
    segs, wants = [], []
    for i in range(300):
        kind = int(rng.choice([0, 1, 2]))
        L = int(rng.integers(4, 11))
        if kind == 2 and L % 2:
            L -= 1
        n, q = 1 << L, int(rng.choice([12289, 12289, 7681])) if L <= 8 else 12289
        flags = int(rng.integers(0, 2))              # lane or canonical arithmetic
        key = (kind, n, q, flags)
        if key not in plans:
            plans[key] = gb.Plan(kind, n, q, root_for(q, n), 0, flags)
        count = 0 if i % 37 == 5 else int(rng.integers(1, 10))
        x = torch.from_numpy(rng.integers(-32768, 32768, (count, n)).astype(np.int16)).cuda()
        segs.append((plans[key], x, torch.full_like(x, 11)))
        wants.append(plans[key](x) if count else x.clone())
    b = gb.Batch(segs)
    assert b.launches == 2                           # int16 lanes, int16 canonical
    for rep in range(2):
        b.graph_launch()
        torch.cuda.synchronize()
        b.status()
        for i, ((_, x, y), w) in enumerate(zip(segs, wants)):
            if x.shape[0]:
                assert torch.equal(y, w), (i, rep)


def test_batch_graph_with_two_pass_segments(gb):
    """Segments that run their plan's own launches inside a batch's CUDA graph:
    the canonical int32 four-step (n = 2^16) and the lane two-pass (n = 2^17),
    whose launches after the first are programmatic dependent launches, beside
    a persistent int16 segment; replayed twice, against the plans' own calls."""
    rng = np.random.default_rng(SEED + 80)
    specs = [(4, 1 << 16, 998244353, 5, gb.FLAG_CANONICAL), (5, 1 << 17, 469762049, 3, 0),
             (2, 1024, 12289, 700, gb.FLAG_CANONICAL)]
    segs, wants = [], []
    for kind, n, q, count, fl in specs:
        dt = np.int16 if q == 12289 else np.int32
        plan = gb.Plan(kind, n, q, root_for(q, n), 0, fl)
        x = torch.from_numpy(rng.integers(0, q, (count, n)).astype(dt)).cuda()
        segs.append((plan, x, torch.full_like(x, 9)))
        wants.append(plan(x))
    b = gb.Batch(segs)
    s = torch.cuda.Stream()
    for rep in range(2):
        for _, _, y in segs:
            y.fill_(9)
        torch.cuda.synchronize()
        b.graph_launch(s)
        s.synchronize()
        b.status()
        for i, ((_, _, y), w) in enumerate(zip(segs, wants)):
            assert torch.equal(y, w), (i, rep)


@pytest.mark.parametrize("force", ["5,0", "4,0", "4,4"])
def test_canonical_int32_batch_every_configuration(gb, orc, monkeypatch, force):
    """Every compiled canonical int32 configuration, pinned with
    GBNTT_TUNE_FORCE (32 or 16 coefficients per thread; registers for 2 or 4
    CTAs/SM).  Forward and inverse, natural order, n^-1 scaling, n = 4 .. 4096,
    full-range inputs: outputs against the exact transform."""
    monkeypatch.setenv("GBNTT_TUNE_FORCE", force)
    rng = np.random.default_rng(SEED + 90)
    specs = [(4, 4096, 998244353, 37, 0), (5, 2048, 754974721, 21, 0x10), (4, 256, 469762049, 301, 0x8),
             (5, 1024, 167772161, 45, 0x8), (5, 4, 998244353, 777, 0)]
    segs, wants = [], []
    for kind, n, q, count, fl in specs:
        root = root_for(q, n)
        x = rng.integers(-(1 << 31), 1 << 31, (count, n)).astype(np.int32)
        d = torch.from_numpy(x).cuda()
        segs.append((gb.Plan(kind, n, q, root, 0, gb.FLAG_CANONICAL | fl), d, torch.full_like(d, 3)))
        inverse = kind == 5
        xin = np.ascontiguousarray(x[:, orc.bitrev_perm(n)]) if (fl & 0x8 and inverse) else x
        w = orc.ntt_exact(xin, q, root, inverse=inverse)
        if fl & 0x10:
            w = w * pow(n, -1, q) % q
        if fl & 0x8 and not inverse:
            w = w[:, orc.bitrev_perm(n)]
        wants.append(w)
    b = gb.Batch(segs)
    assert b.launches == 1
    for rep in range(2):
        b.graph_launch()
        torch.cuda.synchronize()
        b.status()
        for i, ((_, _, y), w) in enumerate(zip(segs, wants)):
            assert np.array_equal(y.cpu().numpy().astype(np.int64), w.astype(np.int64)), (force, i, rep)
