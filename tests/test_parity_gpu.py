"""GPU parity: every design, through the C ABI, bit-exact against the oracle
(the reference's algorithm restated on the CPU) on the same seeded inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SEED = 20261203


@pytest.fixture(scope="module")
def gb():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    return gb


def root_for(q, n):
    if q == 12289:
        return pow(41, 4096 // n, q)
    if q == 1073707009:
        return pow(992735929, 2048 // n, q)
    g = {7681: 17, 10753: 11, 998244353: 3, 469762049: 3, 167772161: 3, 754974721: 11}[q]
    return pow(g, (q - 1) // n, q)


def gpu_run(gb, kind, n, q, root, x, factor=0, flags=0, inplace=False):
    plan = gb.Plan(kind, n, q, root, factor, flags)
    t = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    if inplace:
        plan(t, out=t)
        out = t
    else:
        out = plan(t)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def inputs(rng, batch, n, lo, hi, dtype):
    return rng.integers(lo, hi, size=(batch, n)).astype(dtype)


def check(gb, orc, kind, okind, n, q, root, x, factor=0, flags=0, oflags=None, **kw):
    want = orc.Plan(okind, n, q, root, factor=factor, **(oflags or {}))(x)
    got = gpu_run(gb, kind, n, q, root, x, factor, flags)
    assert got.dtype == want.dtype
    bad = np.argwhere(got != want)
    assert bad.size == 0, f"{len(bad)} mismatches, first at {bad[0]}: gpu {got[tuple(bad[0])]} oracle {want[tuple(bad[0])]}"
    return want


N16 = [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096]


@pytest.mark.parametrize("n", N16)
def test_r2_i16_forward(gb, orc, n):
    rng = np.random.default_rng(SEED + n)
    q = 12289
    for lo, hi in ((0, q), (-32768, 32768)):
        x = inputs(rng, 37, n, lo, hi, np.int16)
        check(gb, orc, gb.Kind.R2_I16_FWD, orc.R2_I16_FWD, n, q, root_for(q, n), x)


@pytest.mark.parametrize("n", N16)
def test_r2_i16_inverse(gb, orc, n):
    rng = np.random.default_rng(SEED + 100 + n)
    q = 12289
    for lo, hi in ((-q, q), (-32768, 32768)):
        x = inputs(rng, 29, n, lo, hi, np.int16)
        check(gb, orc, gb.Kind.R2_I16_INV, orc.R2_I16_INV, n, q, root_for(q, n), x)


@pytest.mark.parametrize("n,q", [(4, 12289), (16, 12289), (64, 12289), (256, 12289), (1024, 12289),
                                 (4096, 12289), (256, 7681), (64, 10753), (256, 10753)])
def test_r4_forward(gb, orc, n, q):
    rng = np.random.default_rng(SEED + 200 + n + q)
    for lo, hi in ((0, q), (-32768, 32768)):
        x = inputs(rng, 41, n, lo, hi, np.int16)
        check(gb, orc, gb.Kind.R4_I16_FWD, orc.R4_I16_FWD, n, q, root_for(q, n), x)


@pytest.mark.parametrize("n", [4, 16, 256, 1024, 4096])
def test_r4_inverse(gb, orc, n):
    rng = np.random.default_rng(SEED + 300 + n)
    q = 12289
    x = inputs(rng, 9, n, -q, q, np.int16)
    check(gb, orc, gb.Kind.R4_I16_INV, orc.R4_I16_INV, n, q, root_for(q, n), x)


@pytest.mark.parametrize("n", [16, 32, 64, 512, 1024, 4096])
def test_r8_stage_reference_multipliers(gb, orc, n):
    """The reference's one radix-8 stage with its float K=31 multipliers:
    bit-exact, including the outputs those multipliers get wrong."""
    rng = np.random.default_rng(SEED + 400 + n)
    q = 12289
    for lo, hi in ((0, q), (-32768, 32768)):
        x = inputs(rng, 23, n, lo, hi, np.int16)
        check(gb, orc, gb.Kind.R8_I16_STAGE, orc.R8_I16_STAGE, n, q, root_for(q, n), x)


@pytest.mark.parametrize("n", [8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096])
def test_r8_chained(gb, orc, n):
    rng = np.random.default_rng(SEED + 500 + n)
    q = 12289
    x = inputs(rng, 19, n, -32768, 32768, np.int16)
    check(gb, orc, gb.Kind.R8_I16_FWD, orc.R8_I16_FWD, n, q, root_for(q, n), x, oflags={"r8_exact": True})
    check(gb, orc, gb.Kind.R8_I16_FWD, orc.R8_I16_FWD, n, q, root_for(q, n), x, flags=gb.FLAG_R8_FLOAT)


Q32 = [998244353, 469762049, 167772161, 754974721, 1073707009]


@pytest.mark.parametrize("n", [2, 4, 16, 64, 256, 1024, 2048, 4096, 8192, 16384, 32768])
@pytest.mark.parametrize("q", Q32)
def test_r2_i32(gb, orc, n, q):
    if q == 1073707009 and n > 2048:
        pytest.skip("root order 2048")
    rng = np.random.default_rng(SEED + 600 + n + q % 1000)
    batch = 7 if n >= 8192 else 33
    root = root_for(q, n)
    x = inputs(rng, batch, n, 0, q, np.int32)
    y = check(gb, orc, gb.Kind.R2_I32_FWD, orc.R2_I32_FWD, n, q, root, x)
    check(gb, orc, gb.Kind.R2_I32_INV, orc.R2_I32_INV, n, q, root, y)
    xf = inputs(rng, batch, n, -(1 << 31), 1 << 31, np.int32)
    check(gb, orc, gb.Kind.R2_I32_FWD, orc.R2_I32_FWD, n, q, root, xf)
    check(gb, orc, gb.Kind.R2_I32_INV, orc.R2_I32_INV, n, q, root, xf)


@pytest.mark.parametrize("n", [2, 8, 64, 128, 256, 512, 1024, 2048, 4096, 8192, 65536])
def test_bitrev(gb, orc, n):
    """Out of place and in place; n = 64 .. 4096 run the tiled transpose
    kernel, the others the staged gather."""
    rng = np.random.default_rng(SEED + 700 + n)
    x = inputs(rng, 5, n, -32768, 32768, np.int16)
    got = gpu_run(gb, gb.Kind.BITREV_I16, n, 0, 0, x)
    want = orc.Plan(orc.BITREV_I16, n)(x)
    assert np.array_equal(got, want)
    got2 = gpu_run(gb, gb.Kind.BITREV_I16, n, 0, 0, x, inplace=True)
    assert np.array_equal(got2, want)


@pytest.mark.parametrize("n", [64, 128, 256, 2048, 4096])
def test_bitrev_many_polynomials(gb, orc, n):
    """The tiled kernel with several tiles per CTA and a partly filled last
    CTA (301 polynomials), out of place and in place."""
    rng = np.random.default_rng(SEED + 750 + n)
    x = inputs(rng, 301, n, -32768, 32768, np.int16)
    want = orc.Plan(orc.BITREV_I16, n)(x)
    assert np.array_equal(gpu_run(gb, gb.Kind.BITREV_I16, n, 0, 0, x), want)
    assert np.array_equal(gpu_run(gb, gb.Kind.BITREV_I16, n, 0, 0, x, inplace=True), want)


@pytest.mark.parametrize("n,batch", [(4096, 3), (1024, 17), (7, 5)])
def test_full_barrett(gb, orc, n, batch):
    rng = np.random.default_rng(SEED + 800 + n)
    q = 12289
    F = pow(4096, -1, q)
    x = inputs(rng, batch, n, -32768, 32768, np.int16)
    got = gpu_run(gb, gb.Kind.FULL_BARRETT_I16, n, q, 0, x, factor=F)
    want = orc.Plan(orc.FULL_BARRETT_I16, n, q, 0, factor=F)(x)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("kind,okind,q,n,dt", [(0, 0, 12289, 1024, np.int16), (1, 1, 12289, 1024, np.int16),
                                               (2, 2, 12289, 1024, np.int16), (4, 4, 998244353, 4096, np.int32),
                                               (5, 5, 754974721, 4096, np.int32)])
def test_canonical_outputs(gb, orc, kind, okind, q, n, dt):
    rng = np.random.default_rng(SEED + 900 + kind)
    x = inputs(rng, 11, n, 0, q, dt)
    want = orc.Plan(okind, n, q, root_for(q, n))(x).astype(np.int64) % q
    got = gpu_run(gb, kind, n, q, root_for(q, n), x, flags=gb.FLAG_CANONICAL)
    assert np.array_equal(got.astype(np.int64), want)


@pytest.mark.parametrize("kind,okind,q,n,dt", [(0, 0, 12289, 4096, np.int16), (5, 5, 998244353, 4096, np.int32),
                                               (8, 8, 12289, 2048, np.int16)])
def test_in_place(gb, orc, kind, okind, q, n, dt):
    rng = np.random.default_rng(SEED + 950 + kind)
    x = inputs(rng, 6, n, 0, q, dt)
    want = orc.Plan(okind, n, q, root_for(q, n), r8_exact=True)(x)
    got = gpu_run(gb, kind, n, q, root_for(q, n), x, inplace=True)
    assert np.array_equal(got, want)


def test_config1_roundtrip(gb, orc):
    """n = 1024, q = 12289: forward then inverse; bit-exact and x * n mod q."""
    q, n = 12289, 1024
    root = root_for(q, n)
    x = np.random.default_rng(SEED).integers(0, q, n).astype(np.int16)
    y = check(gb, orc, gb.Kind.R2_I16_FWD, orc.R2_I16_FWD, n, q, root, x[None])
    z = check(gb, orc, gb.Kind.R2_I16_INV, orc.R2_I16_INV, n, q, root, y)
    assert np.array_equal(z[0].astype(np.int64) % q, x.astype(np.int64) * n % q)
    fb = gpu_run(gb, gb.Kind.FULL_BARRETT_I16, n, q, 0, z, factor=pow(n, -1, q))
    assert np.array_equal(fb[0].astype(np.int64) % q, x.astype(np.int64))


@pytest.mark.parametrize("q", [998244353, 469762049, 167772161, 754974721])
def test_config2_dft(gb, orc, q):
    """n = 256 against the O(n^2) DFT, n = 4096 round trip."""
    rng = np.random.default_rng(SEED + q % 997)
    x = rng.integers(0, q, 256)
    y = gpu_run(gb, gb.Kind.R2_I32_FWD, 256, q, root_for(q, 256), x.astype(np.int32)[None], flags=gb.FLAG_CANONICAL)
    X = orc.dft(x, q, root_for(q, 256))
    assert np.array_equal(y[0].astype(np.int64), X[orc.bitrev_perm(256)])
    x = rng.integers(0, q, 4096).astype(np.int32)[None]
    y = gpu_run(gb, gb.Kind.R2_I32_FWD, 4096, q, root_for(q, 4096), x)
    z = gpu_run(gb, gb.Kind.R2_I32_INV, 4096, q, root_for(q, 4096), y)
    assert np.array_equal(z.astype(np.int64) % q, x.astype(np.int64) * 4096 % q)


def test_graph_mirror_and_configs(gb, orc):
    """dut_for_config selects the design of src/project.cpp:139-157."""
    rng = np.random.default_rng(SEED + 1)
    for cfg in range(8):
        g = gb.dut_for_config(cfg).init()
        p = g.plan
        n = p.n
        dt = np.int32 if p.elem_bytes == 4 else np.int16
        x = rng.integers(0, min(p.q, 30000) if p.q else 30000, (3, n)).astype(dt)
        out = g.run(3, torch.from_numpy(x).cuda())
        torch.cuda.synchronize()
        ok = orc.Plan(int(p.kind), n, p.q, p.root, factor=p.factor)(x)
        assert np.array_equal(out.cpu().numpy(), ok), cfg
        g.end()


def test_batch_zero_and_launch_counter(gb):
    plan = gb.Plan(gb.Kind.R2_I16_FWD, 1024, 12289, root_for(12289, 1024))
    x = torch.zeros(4, 1024, dtype=torch.int16, device="cuda")
    c0 = gb.launch_count()
    plan.execute(x, x, 0)
    assert gb.launch_count() == c0
    plan(x)
    assert gb.launch_count() == c0 + 1


def test_execute_host(gb, orc):
    q, n = 12289, 1024
    x = np.random.default_rng(3).integers(-32768, 32768, (64, n)).astype(np.int16)
    out = np.empty_like(x)
    plan = gb.Plan(gb.Kind.R4_I16_FWD, n, q, root_for(q, n))
    plan.execute_host(x, out)
    assert np.array_equal(out, orc.Plan(orc.R4_I16_FWD, n, q, root_for(q, n))(x))
    st = gb.Plan(gb.Kind.R8_I16_STAGE, n, q, root_for(q, n))
    st.execute_host(x, out)
    assert np.array_equal(out, orc.Plan(orc.R8_I16_STAGE, n, q, root_for(q, n))(x))


HOST_CASES = [  # (kind, n, q, factor, flags, dtype) -- every design
    (0, 1024, 12289, 0, 0, np.int16), (1, 1024, 12289, 0, 0x8 | 0x10, np.int16), (2, 256, 7681, 0, 0, np.int16),
    (9, 4096, 12289, 0, 0, np.int16), (3, 512, 12289, 0, 0, np.int16), (8, 2048, 12289, 0, 0x8, np.int16),
    (6, 1024, 0, 0, 0, np.int16), (7, 1024, 12289, 12277, 0, np.int16), (4, 4096, 998244353, 0, 0x1, np.int32),
    (5, 2048, 754974721, 0, 0x8, np.int32), (4, 1 << 16, 469762049, 0, 0, np.int32)]


@pytest.mark.parametrize("kind,n,q,factor,flags,dt", HOST_CASES)
def test_execute_host_every_design(gb, kind, n, q, factor, flags, dt):
    """Host buffers, pinned and pageable, equal the device-memory launch, also in place."""
    root = root_for(q, n) if q and kind != 7 else 0
    plan = gb.Plan(kind, n, q, root, factor, flags)
    rng = np.random.default_rng(SEED + 77 + kind + n)
    lo, hi = (0, q) if q else (-32768, 32768)
    x = rng.integers(lo, hi, (5, n)).astype(dt)
    want = plan(torch.from_numpy(x).cuda()).cpu().numpy()
    pin_in = torch.from_numpy(x).pin_memory()
    pin_out = torch.empty_like(pin_in).pin_memory()
    plan.execute_host(pin_in, pin_out)
    assert np.array_equal(pin_out.numpy(), want)
    page_out = np.empty_like(x)
    plan.execute_host(x, page_out)
    assert np.array_equal(page_out, want)
    if kind != 3:                                        # the radix-8 stage cannot run in place
        plan.execute_host(pin_in, pin_in)
        assert np.array_equal(pin_in.numpy(), want)


def test_batch_execute_host_zero_copy(gb):
    """Pinned buffers: one zero-copy persistent launch per storage type (the
    radix-8 stage segment is copied through its device buffers); pageable
    buffers: copies and the graph.  Ragged counts leave partial tiles."""
    specs = [(2, 1024, 12289), (0, 256, 12289), (1, 64, 12289), (8, 4096, 12289), (5, 4096, 998244353),
             (4, 8192, 998244353), (3, 512, 12289)]
    rng = np.random.default_rng(SEED + 99)
    plans, ins, d_in, d_out = [], [], [], []
    for kind, n, q in specs:
        dt = np.int32 if kind in (4, 5) else np.int16
        plans.append(gb.Plan(kind, n, q, root_for(q, n)))
        ins.append(rng.integers(0, q, (37 + 3 * len(ins), n)).astype(dt))
        d_in.append(torch.from_numpy(ins[-1]).cuda())
        d_out.append(torch.empty_like(d_in[-1]))
    batch = gb.Batch([(plans[i], d_in[i], d_out[i]) for i in range(len(specs))])
    batch.execute()
    torch.cuda.synchronize()
    want = [t.cpu().numpy() for t in d_out]
    pin_in = [torch.from_numpy(x).pin_memory() for x in ins]
    pin_out = [torch.empty_like(t).pin_memory() for t in pin_in]
    c0 = gb.launch_count()
    batch.execute_host(pin_in, pin_out)                  # zero copy: int16 + int32 launches, + r8 stage
    assert gb.launch_count() - c0 == 3
    assert all(np.array_equal(a.numpy(), b) for a, b in zip(pin_out, want))
    batch.execute_host(pin_in, pin_in)                   # in place on the host buffers
    assert all(np.array_equal(a.numpy(), b) for a, b in zip(pin_in, want))
    page_out = [np.empty_like(x) for x in ins]
    batch.execute_host(ins, page_out)                    # copies + one persistent launch
    assert all(np.array_equal(a, b) for a, b in zip(page_out, want))


FORM_CASES = [  # (kind, oracle kind, q, L, dtype, oracle options) -- designs with a latency form
    (0, 0, 12289, 9, np.int16, {}), (0, 0, 12289, 10, np.int16, {}), (0, 0, 12289, 11, np.int16, {}),
    (1, 1, 12289, 10, np.int16, {}), (1, 1, 12289, 12, np.int16, {}), (2, 2, 12289, 10, np.int16, {}),
    (9, 9, 12289, 10, np.int16, {}), (8, 8, 12289, 10, np.int16, {"r8_exact": True}),
    (8, 8, 12289, 11, np.int16, {"r8_exact": True}), (4, 4, 998244353, 9, np.int32, {}),
    (4, 4, 998244353, 11, np.int32, {}), (5, 5, 998244353, 10, np.int32, {})]


@pytest.mark.parametrize("kind,okind,q,L,dt,ok", FORM_CASES)
def test_latency_and_throughput_forms(gb, orc, kind, okind, q, L, dt, ok):
    """A per-plan launch of at most one CTA per SM takes the latency form (one
    polynomial per CTA, up to 256 threads); a larger one the throughput form.
    Both equal the oracle."""
    n = 1 << L
    root = root_for(q, n)
    rng = np.random.default_rng(SEED + 300 + kind + L)
    for batch in (1, 3, 400):
        x = inputs(rng, batch, n, 0, q, dt)
        check(gb, orc, kind, okind, n, q, root, x, oflags=ok)


def test_zero_copy_buffer_switches(gb):
    """Zero-copy calls alternating between two sets of pinned buffers (A, B, A,
    B with different inputs): each call transforms the buffers it is given,
    so device descriptors reused from the previous call stay correct."""
    rng = np.random.default_rng(SEED + 101)
    specs = [(2, 1024, 12289, np.int16), (4, 4096, 998244353, np.int32)]
    plans = [gb.Plan(k, n, q, root_for(q, n)) for k, n, q, _ in specs]
    sets = []
    for _ in range(2):
        xs = [rng.integers(0, q, (19, n)).astype(dt) for _, n, q, dt in specs]
        want = [p(torch.from_numpy(x).cuda()).cpu().numpy() for p, x in zip(plans, xs)]
        ins = [torch.from_numpy(x).pin_memory() for x in xs]
        outs = [torch.empty_like(t).pin_memory() for t in ins]
        sets.append((ins, outs, want))
    batch = gb.Batch([(p, torch.from_numpy(x.numpy()).cuda(), torch.empty_like(torch.from_numpy(x.numpy())).cuda())
                      for p, x in zip(plans, sets[0][0])])
    for rep in range(4):
        ins, outs, want = sets[rep % 2]
        for t in outs:
            t.zero_()
        batch.execute_host(ins, outs)
        assert all(np.array_equal(o.numpy(), w) for o, w in zip(outs, want)), rep
        for t in outs:
            t.zero_()
        plans[0].execute_host(ins[0], outs[0])
        assert np.array_equal(outs[0].numpy(), want[0]), rep


# ---------------------------------------------------------------------------
# fused bit reversal (natural order) and fused n^-1 epilogue
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("kind,okind,q,n,dt,ok", [
    (0, 0, 12289, 1024, np.int16, {}), (2, 2, 12289, 4096, np.int16, {}), (2, 2, 7681, 256, np.int16, {}),
    (8, 8, 12289, 2048, np.int16, {"r8_exact": True}), (4, 4, 998244353, 4096, np.int32, {}),
    (0, 0, 12289, 16, np.int16, {})])
def test_natural_order_forward(gb, orc, kind, okind, q, n, dt, ok):
    rng = np.random.default_rng(SEED + 1000 + n + kind)
    x = inputs(rng, 13, n, 0, q, dt)
    want = orc.Plan(okind, n, q, root_for(q, n), **ok)(x)[:, orc.bitrev_perm(n)]
    got = gpu_run(gb, kind, n, q, root_for(q, n), x, flags=gb.FLAG_NATURAL_ORDER)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("kind,q,n,dt", [(1, 12289, 1024, np.int16), (1, 12289, 8, np.int16),
                                         (9, 12289, 4096, np.int16), (5, 754974721, 2048, np.int32)])
def test_natural_order_inverse_and_scale(gb, orc, kind, q, n, dt):
    rng = np.random.default_rng(SEED + 1100 + n + kind)
    x = inputs(rng, 7, n, -q, q, dt)
    br = orc.bitrev_perm(n)
    want = orc.Plan(kind, n, q, root_for(q, n))(np.ascontiguousarray(x[:, br]))
    got = gpu_run(gb, kind, n, q, root_for(q, n), x, flags=gb.FLAG_NATURAL_ORDER)
    assert np.array_equal(got, want)
    if dt == np.int16:
        fb = orc.Plan(orc.FULL_BARRETT_I16, n, q, 0, factor=pow(n, -1, q))
        got = gpu_run(gb, kind, n, q, root_for(q, n), x, flags=gb.FLAG_SCALE_NINV)
        assert np.array_equal(got, fb(orc.Plan(kind, n, q, root_for(q, n))(x)))


def test_fused_roundtrip_returns_input(gb):
    """natural-order forward, then natural-order inverse with the n^-1 epilogue: x back."""
    q, n = 12289, 1024
    x = np.random.default_rng(5).integers(0, q, (64, n)).astype(np.int16)
    y = gpu_run(gb, 0, n, q, root_for(q, n), x, flags=gb.FLAG_NATURAL_ORDER)
    z = gpu_run(gb, 1, n, q, root_for(q, n), y, flags=gb.FLAG_NATURAL_ORDER | gb.FLAG_SCALE_NINV)
    assert np.array_equal(z.astype(np.int64) % q, x)
    assert z.min() >= 0 and z.max() <= q


def test_flags_in_a_batch(gb, orc):
    q = 12289
    rng = np.random.default_rng(77)
    specs = [(2, 1024, gb.FLAG_NATURAL_ORDER), (1, 1024, gb.FLAG_SCALE_NINV),
             (1, 256, gb.FLAG_NATURAL_ORDER | gb.FLAG_SCALE_NINV), (0, 512, gb.FLAG_NATURAL_ORDER)]
    plans, xs, ys, wants = [], [], [], []
    for kind, n, fl in specs:
        x = rng.integers(0, q, (300, n)).astype(np.int16)
        xin = np.ascontiguousarray(x[:, orc.bitrev_perm(n)]) if (fl & gb.FLAG_NATURAL_ORDER and kind == 1) else x
        w = orc.Plan(kind, n, q, root_for(q, n))(xin)
        if fl & gb.FLAG_SCALE_NINV:
            w = orc.Plan(orc.FULL_BARRETT_I16, n, q, 0, factor=pow(n, -1, q))(w)
        if fl & gb.FLAG_NATURAL_ORDER and kind != 1:
            w = w[:, orc.bitrev_perm(n)]
        plans.append(gb.Plan(kind, n, q, root_for(q, n), 0, fl))
        xs.append(torch.from_numpy(x).cuda())
        ys.append(torch.empty_like(xs[-1]))
        wants.append(w)
    b = gb.Batch(list(zip(plans, xs, ys)))
    b.execute()
    torch.cuda.synchronize()
    for i, (y, w) in enumerate(zip(ys, wants)):
        assert np.array_equal(y.cpu().numpy(), w), i


@pytest.mark.parametrize("L", [16, 17, 19, 20, 21, 22])
@pytest.mark.parametrize("q", [998244353, 754974721])
def test_r2_i32_two_pass(gb, orc, q, L):
    """n = 2^16 .. 2^22: column pass + row pass, bit-exact with the reference's layers
    (2^21 and 2^22: fewer columns per CTA in the column pass)."""
    n = 1 << L
    rng = np.random.default_rng(SEED + 1200 + L)
    batch = 1 if L >= 21 else 3 if L >= 19 else 5
    root = root_for(q, n)
    x = inputs(rng, batch, n, 0, q, np.int32)
    y = check(gb, orc, gb.Kind.R2_I32_FWD, orc.R2_I32_FWD, n, q, root, x)
    z = check(gb, orc, gb.Kind.R2_I32_INV, orc.R2_I32_INV, n, q, root, y)
    assert np.array_equal(z.astype(np.int64) % q, x.astype(np.int64) * n % q)
    got = gpu_run(gb, gb.Kind.R2_I32_FWD, n, q, root, x, flags=gb.FLAG_CANONICAL)
    assert np.array_equal(got.astype(np.int64), y.astype(np.int64) % q)
    got = gpu_run(gb, gb.Kind.R2_I32_INV, n, q, root, y, inplace=True)
    assert np.array_equal(got, z)


def test_r2_i32_two_pass_many_chunks(gb):
    """50 polynomials of 2^20 (three 96 MiB chunks, programmatic dependent
    launches between the passes and the chunks), forward and inverse: the
    polynomials at the chunk boundaries equal their single-polynomial calls."""
    q, n = 998244353, 1 << 20
    root = root_for(q, n)
    x = torch.from_numpy(np.random.default_rng(SEED + 1300).integers(0, q, (50, n)).astype(np.int32)).cuda()
    for kind in (gb.Kind.R2_I32_FWD, gb.Kind.R2_I32_INV):
        plan = gb.Plan(kind, n, q, root)
        y = plan(x)
        for i in (0, 23, 24, 47, 48, 49):
            assert torch.equal(y[i:i + 1], plan(x[i:i + 1])), (kind, i)


def test_r2_i32_two_pass_dft_column(gb, orc):
    """n = 2^16 against the modular DFT at a few output positions."""
    q, n = 469762049, 1 << 16
    root = root_for(q, n)
    x = np.random.default_rng(11).integers(0, q, n)
    y = gpu_run(gb, gb.Kind.R2_I32_FWD, n, q, root, x.astype(np.int32)[None], flags=gb.FLAG_CANONICAL)[0]
    br = n.bit_length() - 1
    for k in (0, 1, 12345, n - 1):
        want = sum(int(x[j]) * pow(root, j * k, q) for j in range(n)) % q
        pos = int(format(k, f"0{br}b")[::-1], 2)
        assert int(y[pos]) == want
