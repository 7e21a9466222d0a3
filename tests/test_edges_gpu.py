"""Edge cases: the largest moduli each storage type allows (q < 2^16/3 for the
int16 designs, q < 2^32/3 for int32), the full input range, and empty work
(zero polynomials) on every entry point."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from test_parity_gpu import SEED, check, inputs  # noqa: E402

# the largest NTT-friendly primes below the lazy-reduction bounds, with a generator
Q16_MAX = [(19457, 3, 1024), (18433, 5, 2048)]          # (q, generator, largest power-of-two n)
Q32_MAX = [(1431580673, 3, 4096), (1431576577, 5, 8192)]


@pytest.fixture(scope="module")
def gb():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    return gb


@pytest.mark.parametrize("q,g,n", Q16_MAX)
@pytest.mark.parametrize("lo", [0, -32768])
def test_int16_largest_moduli(gb, orc, q, g, n, lo):
    root = pow(g, (q - 1) // n, q)
    rng = np.random.default_rng(SEED + q + lo)
    x = inputs(rng, 9, n, lo, q if lo == 0 else 32768, np.int16)
    y = check(gb, orc, gb.Kind.R2_I16_FWD, orc.R2_I16_FWD, n, q, root, x)
    check(gb, orc, gb.Kind.R2_I16_INV, orc.R2_I16_INV, n, q, root, y)
    if (n.bit_length() - 1) % 2 == 0:
        check(gb, orc, gb.Kind.R4_I16_FWD, orc.R4_I16_FWD, n, q, root, x)
    if lo == 0:   # canonical round trip
        z = orc.Plan(orc.R2_I16_INV, n, q, root)(y)
        assert np.array_equal(z.astype(np.int64) % q, x.astype(np.int64) * n % q)


@pytest.mark.parametrize("q,g,n", Q32_MAX)
@pytest.mark.parametrize("lo", [0, -(1 << 31)])
def test_int32_largest_moduli(gb, orc, q, g, n, lo):
    root = pow(g, (q - 1) // n, q)
    rng = np.random.default_rng(SEED + (q % 1000) + (lo & 7))
    x = inputs(rng, 5, n, lo, q if lo == 0 else (1 << 31), np.int32)
    y = check(gb, orc, gb.Kind.R2_I32_FWD, orc.R2_I32_FWD, n, q, root, x)
    check(gb, orc, gb.Kind.R2_I32_INV, orc.R2_I32_INV, n, q, root, y)


def test_largest_moduli_in_one_batch(gb, orc):
    """The persistent kernel with the largest moduli of both storage types."""
    segs, wants = [], []
    rng = np.random.default_rng(SEED + 5)
    for kind, okind, q, g, n, dt in ((0, 0, 19457, 3, 1024, np.int16), (1, 1, 18433, 5, 2048, np.int16),
                                     (4, 4, 1431580673, 3, 4096, np.int32), (5, 5, 1431576577, 5, 8192, np.int32)):
        root = pow(g, (q - 1) // n, q)
        x = rng.integers(0, q, (33, n)).astype(dt)
        dx = torch.from_numpy(x).cuda()
        segs.append((gb.Plan(kind, n, q, root), dx, torch.empty_like(dx)))
        wants.append(orc.Plan(okind, n, q, root)(x))
    b = gb.Batch(segs)
    b.execute()
    torch.cuda.synchronize()
    for (_, _, y), w in zip(segs, wants):
        assert np.array_equal(y.cpu().numpy(), w)


def test_empty_work(gb):
    """Zero polynomials: no launch, no error, outputs untouched."""
    plan = gb.Plan(gb.Kind.R2_I16_FWD, 1024, 12289, pow(41, 4, 12289))
    x = torch.ones(4, 1024, dtype=torch.int16, device="cuda")
    y = torch.full_like(x, 7)
    c0 = gb.launch_count()
    plan.execute(x, y, 0)
    h = np.ones((4, 1024), dtype=np.int16)
    ho = np.full_like(h, 7)
    plan.execute_host(h, ho, batch=0)
    torch.cuda.synchronize()
    assert gb.launch_count() == c0
    assert bool((y == 7).all()) and bool((ho == 7).all())
    # a batch with an empty segment next to a full one
    other = gb.Plan(gb.Kind.R4_I16_FWD, 256, 7681, pow(17, (7681 - 1) // 256, 7681))
    z_in = torch.randint(0, 7681, (64, 256), dtype=torch.int16, device="cuda")
    z_out = torch.empty_like(z_in)
    b = gb.Batch([(plan, x[:0], y[:0]), (other, z_in, z_out)])
    b.execute()
    torch.cuda.synchronize()
    assert torch.equal(z_out, other(z_in))
    # the server refuses an empty request at submission
    srv = gb.Server([plan])
    with pytest.raises(gb.NTTError):
        srv.submit(0, h, ho, count=0)
    srv.close()
