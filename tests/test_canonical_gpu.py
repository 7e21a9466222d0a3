"""GPU parity of the canonical families (GBNTT_FLAG_CANONICAL): Shoup
multiplication, lazily reduced lanes, one final reduction.

Every output is checked against the exact transform (oracle.ntt_exact, itself
pinned to the O(n^2) modular DFT in test_oracle.py) of the inputs taken mod q.
Where the reference's own lanes do not wrap -- residue inputs at the
reference's moduli, and full-range int16 inputs to its forward designs -- the
same outputs are also checked against the oracle's restatement of the
reference's kernels reduced mod q, i.e. the reference's residues.  Where its
lanes do wrap, GBNTT_FLAG_CANONICAL | GBNTT_FLAG_LANE_EXACT reproduces the
reference's residues bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from test_parity_gpu import SEED, gpu_run, inputs, root_for  # noqa: E402

FWD16 = [(0, 0), (2, 2), (8, 8)]     # (library kind, oracle kind): radix-2, radix-4, radix-8 chain
INV16 = [(1, 1), (9, 9)]             # radix-2 inverse, radix-4 inverse
REF_Q16 = [12289, 7681, 10753]       # the reference's modulus and the benchmark's other two
MAX_L16 = {12289: 12, 7681: 9, 10753: 9, 19457: 10, 18433: 11}
GEN16 = {19457: 3, 18433: 5}
Q32 = [998244353, 469762049, 167772161, 754974721, 1073707009]


@pytest.fixture(scope="module")
def gb():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    return gb


def root16(q, n):
    if q in GEN16:
        return pow(GEN16[q], (q - 1) // n, q)
    return root_for(q, n)


def supports(kind, L):
    if kind in (2, 9):
        return L % 2 == 0
    if kind == 8:
        return L >= 3
    return True


def canon_check(gb, orc, kind, okind, n, q, root, x, inverse, flags=0, lanes=False, batch_forms=True):
    """The canonical output of x (and of x's first polynomials alone, which
    takes the latency form) against the exact transform; against the oracle's
    residues when `lanes` says the reference's lanes do not wrap."""
    got = gpu_run(gb, kind, n, q, root, x, flags=gb.FLAG_CANONICAL | flags)
    assert got.min() >= 0 and int(got.max()) < q
    want = orc.ntt_exact(x, q, root, inverse=inverse)
    bad = np.argwhere(got.astype(np.int64) != want)
    assert bad.size == 0, f"{len(bad)} mismatches, first at {bad[0]}: gpu {got[tuple(bad[0])]} exact {want[tuple(bad[0])]}"
    if batch_forms and x.shape[0] > 3:
        few = gpu_run(gb, kind, n, q, root, x[:3], flags=gb.FLAG_CANONICAL | flags)
        assert np.array_equal(few, got[:3])
    if lanes:
        ref = orc.Plan(okind, n, q, root, r8_exact=True)(x).astype(np.int64) % q
        assert np.array_equal(got.astype(np.int64), ref)
    return got


@pytest.mark.parametrize("L", list(range(1, 13)))
@pytest.mark.parametrize("kind,okind", FWD16 + INV16)
def test_canonical_int16_every_length(gb, orc, kind, okind, L):
    if not supports(kind, L):
        pytest.skip("length not a design of this kind")
    n = 1 << L
    inverse = (kind, okind) in INV16
    for q in REF_Q16:
        if L > MAX_L16[q]:
            continue
        rng = np.random.default_rng(SEED + 3000 + 17 * L + kind + q)
        root = root16(q, n)
        x = inputs(rng, 170, n, 0, q, np.int16)    # more than one polynomial per SM: throughput form
        canon_check(gb, orc, kind, okind, n, q, root, x, inverse, lanes=True)
        # the full int16 range: the reference's forward lanes stay exact; its
        # radix-2 inverse sums raw inputs in its first layer and wraps
        x = inputs(rng, 19, n, -32768, 32768, np.int16)
        canon_check(gb, orc, kind, okind, n, q, root, x, inverse, lanes=not inverse)


@pytest.mark.parametrize("q", [19457, 18433])
@pytest.mark.parametrize("kind,okind", FWD16 + INV16)
def test_canonical_int16_largest_moduli(gb, orc, kind, okind, q):
    """q near 2^16/3: the reference's radix-4 and inverse lanes wrap there; the
    canonical family still returns the exact transform, and LANE_EXACT the
    reference's own residues."""
    inverse = (kind, okind) in INV16
    for L in (2, 4, 7, MAX_L16[q]):
        if not supports(kind, L):
            continue
        n = 1 << L
        root = root16(q, n)
        rng = np.random.default_rng(SEED + 3100 + L + kind + q)
        for lo, hi in ((0, q), (-32768, 32768)):
            x = inputs(rng, 23, n, lo, hi, np.int16)
            canon_check(gb, orc, kind, okind, n, q, root, x, inverse)
            lane = gpu_run(gb, kind, n, q, root, x, flags=gb.FLAG_CANONICAL | gb.FLAG_LANE_EXACT)
            ref = orc.Plan(okind, n, q, root, r8_exact=True)(x).astype(np.int64) % q
            assert np.array_equal(lane.astype(np.int64), ref)


@pytest.mark.parametrize("n", [2, 4, 16, 256, 1024, 2048, 4096, 8192, 16384, 32768])
@pytest.mark.parametrize("q", Q32)
def test_canonical_int32(gb, orc, n, q):
    rng = np.random.default_rng(SEED + 3200 + n + q % 997)
    root = root_for(q, n) if q != 1073707009 or n <= 2048 else None
    if root is None:
        pytest.skip("q = 1073707009 has no root of unity of order above 2048")
    batch = 160 if n <= 4096 else 5
    for kind, okind, inverse in ((4, 4, False), (5, 5, True)):
        x = inputs(rng, batch, n, 0, q, np.int32)
        canon_check(gb, orc, kind, okind, n, q, root, x, inverse, lanes=True)
        x = inputs(rng, batch, n, -(1 << 31), 1 << 31, np.int32)
        canon_check(gb, orc, kind, okind, n, q, root, x, inverse, lanes=not inverse)


@pytest.mark.parametrize("q,g,n", [(1431580673, 3, 4096), (1431576577, 5, 8192)])
def test_canonical_int32_above_2_30_takes_the_lane_form(gb, orc, q, g, n):
    """Moduli in [2^30, 2^32/3) leave no room for lazy lanes: GBNTT_FLAG_CANONICAL
    runs the reference's lane arithmetic there and reduces it."""
    root = pow(g, (q - 1) // n, q)
    rng = np.random.default_rng(SEED + 3300 + n)
    for kind in (4, 5):
        x = inputs(rng, 5, n, 0, q, np.int32)
        got = gpu_run(gb, kind, n, q, root, x, flags=gb.FLAG_CANONICAL)
        assert np.array_equal(got.astype(np.int64), orc.Plan(kind, n, q, root)(x).astype(np.int64) % q)


@pytest.mark.parametrize("kind,n,q,dt", [(0, 1024, 12289, np.int16), (2, 4096, 12289, np.int16),
                                         (8, 2048, 12289, np.int16), (0, 8, 12289, np.int16),
                                         (4, 4096, 998244353, np.int32), (4, 16384, 754974721, np.int32)])
def test_canonical_natural_order_forward(gb, orc, kind, n, q, dt):
    rng = np.random.default_rng(SEED + 3400 + n + kind)
    lo, hi = (-32768, 32768) if dt == np.int16 else (-(1 << 31), 1 << 31)
    x = inputs(rng, 13, n, lo, hi, dt)
    root = root_for(q, n)
    got = gpu_run(gb, kind, n, q, root, x, flags=gb.FLAG_CANONICAL | gb.FLAG_NATURAL_ORDER)
    want = orc.ntt_exact(x, q, root)[:, orc.bitrev_perm(n)]
    assert np.array_equal(got.astype(np.int64), want)


@pytest.mark.parametrize("kind,n,q,dt", [(1, 1024, 12289, np.int16), (9, 4096, 12289, np.int16),
                                         (1, 16, 7681, np.int16), (5, 4096, 998244353, np.int32),
                                         (5, 32768, 469762049, np.int32)])
def test_canonical_natural_order_inverse_and_scale(gb, orc, kind, n, q, dt):
    rng = np.random.default_rng(SEED + 3500 + n + kind)
    x = inputs(rng, 9, n, 0, q, dt)
    root = root_for(q, n)
    br = orc.bitrev_perm(n)
    got = gpu_run(gb, kind, n, q, root, x, flags=gb.FLAG_CANONICAL | gb.FLAG_NATURAL_ORDER)
    assert np.array_equal(got.astype(np.int64), orc.ntt_exact(np.ascontiguousarray(x[:, br]), q, root, inverse=True))
    got = gpu_run(gb, kind, n, q, root, x, flags=gb.FLAG_CANONICAL | gb.FLAG_SCALE_NINV)
    want = orc.ntt_exact(x, q, root, inverse=True) * pow(n, -1, q) % q
    assert np.array_equal(got.astype(np.int64), want)


@pytest.mark.parametrize("fwd,inv,n,q,dt", [(0, 1, 1024, 12289, np.int16), (2, 9, 256, 7681, np.int16),
                                            (8, 1, 4096, 12289, np.int16), (4, 5, 8192, 167772161, np.int32)])
def test_canonical_round_trip(gb, fwd, inv, n, q, dt):
    """natural-order forward, then natural-order inverse with n^-1: the input mod q."""
    x = np.random.default_rng(SEED + 3600 + n).integers(-30000, 30000, (33, n)).astype(dt)
    root = root_for(q, n)
    y = gpu_run(gb, fwd, n, q, root, x, flags=gb.FLAG_CANONICAL | gb.FLAG_NATURAL_ORDER)
    z = gpu_run(gb, inv, n, q, root, y, flags=gb.FLAG_CANONICAL | gb.FLAG_NATURAL_ORDER | gb.FLAG_SCALE_NINV)
    assert np.array_equal(z.astype(np.int64), x.astype(np.int64) % q)


@pytest.mark.parametrize("kind,n,q,dt", [(0, 4096, 12289, np.int16), (1, 512, 10753, np.int16),
                                         (5, 8192, 998244353, np.int32)])
def test_canonical_in_place(gb, orc, kind, n, q, dt):
    rng = np.random.default_rng(SEED + 3700 + n)
    x = inputs(rng, 6, n, 0, q, dt)
    root = root_for(q, n)
    got = gpu_run(gb, kind, n, q, root, x, flags=gb.FLAG_CANONICAL, inplace=True)
    assert np.array_equal(got.astype(np.int64), orc.ntt_exact(x, q, root, inverse=kind in (1, 9, 5)))


def test_lane_exact_reproduces_the_reference_wrap(gb, orc):
    """Full-range int16 input to the radix-2 inverse: the reference's first
    layer wraps, so its residues differ from the exact transform's.
    LANE_EXACT returns the reference's; CANONICAL alone the exact ones."""
    q, n = 12289, 1024
    root = root_for(q, n)
    x = np.random.default_rng(SEED + 3800).integers(-32768, 32768, (16, n)).astype(np.int16)
    ref = orc.Plan(orc.R2_I16_INV, n, q, root)(x).astype(np.int64) % q
    exact = orc.ntt_exact(x, q, root, inverse=True)
    assert not np.array_equal(ref, exact)
    lane = gpu_run(gb, 1, n, q, root, x, flags=gb.FLAG_CANONICAL | gb.FLAG_LANE_EXACT)
    fast = gpu_run(gb, 1, n, q, root, x, flags=gb.FLAG_CANONICAL)
    assert np.array_equal(lane.astype(np.int64), ref)
    assert np.array_equal(fast.astype(np.int64), exact)


@pytest.mark.parametrize("L", [16, 17, 18, 19, 20, 21, 22])
@pytest.mark.parametrize("q", [998244353, 754974721])
def test_canonical_int32_four_step(gb, orc, q, L):
    """n = 2^16 .. 2^22: TMA-tiled column pass, twist, row pass; against the
    exact transform, both directions, out of place and in place, with the
    fused n^-1 on the inverse, and the round trip."""
    n = 1 << L
    rng = np.random.default_rng(SEED + 3900 + L)
    batch = 1 if L >= 21 else 3 if L >= 19 else 5
    root = root_for(q, n)
    x = inputs(rng, batch, n, -(1 << 31), 1 << 31, np.int32)
    y = gpu_run(gb, 4, n, q, root, x, flags=gb.FLAG_CANONICAL)
    assert np.array_equal(y.astype(np.int64), orc.ntt_exact(x, q, root))
    z = gpu_run(gb, 5, n, q, root, y, flags=gb.FLAG_CANONICAL, inplace=True)
    assert np.array_equal(z.astype(np.int64), (x.astype(np.int64) % q) * n % q)
    w = gpu_run(gb, 5, n, q, root, x, flags=gb.FLAG_CANONICAL | gb.FLAG_SCALE_NINV)
    assert np.array_equal(w.astype(np.int64), orc.ntt_exact(x, q, root, inverse=True) * pow(n, -1, q) % q)
    yi = gpu_run(gb, 4, n, q, root, x, flags=gb.FLAG_CANONICAL, inplace=True)
    assert np.array_equal(yi, y)


# the largest NTT primes below 2^30 (the canonical int32 family's bound: lanes
# below 2q, sums below 4q < 2^32) for a given 2-adic order: (q, generator, n)
Q30_EDGE = [(1073692673, 3, 4096), (1073692673, 3, 16384), (1073479681, 11, 1 << 16),
            (1073479681, 11, 1 << 18), (1053818881, 7, 1 << 20)]


@pytest.mark.parametrize("q,g,n", Q30_EDGE)
def test_canonical_int32_moduli_just_below_2_30(gb, orc, q, g, n):
    """Full-range int32 inputs at the largest moduli the canonical int32
    family takes, where its lazy bounds are tightest: per-plan (n = 4096, one
    CTA per polynomial at 2^14) and four-step (2^16 .. 2^20) forward, the
    inverse with the fused n^-1, and the persistent batch at n = 4096."""
    root = pow(g, (q - 1) // n, q)
    rng = np.random.default_rng(SEED + 4200 + n.bit_length())
    batch = 1 if n >= 1 << 18 else 3
    x = inputs(rng, batch, n, -(1 << 31), 1 << 31, np.int32)
    y = gpu_run(gb, 4, n, q, root, x, flags=gb.FLAG_CANONICAL)
    assert np.array_equal(y.astype(np.int64), orc.ntt_exact(x, q, root))
    w = gpu_run(gb, 5, n, q, root, y, flags=gb.FLAG_CANONICAL | gb.FLAG_SCALE_NINV)
    assert np.array_equal(w.astype(np.int64), x.astype(np.int64) % q)
    if n == 4096:
        xs = rng.integers(-(1 << 31), 1 << 31, (40, n)).astype(np.int32)
        d = torch.from_numpy(xs).cuda()
        out = torch.empty_like(d)
        b = gb.Batch([(gb.Plan(4, n, q, root, 0, gb.FLAG_CANONICAL), d, out)])
        assert b.launches == 1
        b.execute()
        torch.cuda.synchronize()
        b.status()
        assert np.array_equal(out.cpu().numpy().astype(np.int64), orc.ntt_exact(xs, q, root))


def test_canonical_four_step_status_and_many_chunks(gb, orc):
    """A batch spanning three L2 chunks (96 MiB, 24 polynomials of 2^20, each;
    programmatic dependent launches between the passes and the chunks) and the
    plan's status call."""
    q, n = 469762049, 1 << 20
    root = root_for(q, n)
    x = np.random.default_rng(SEED + 3990).integers(0, q, (50, n)).astype(np.int32)
    plan = gb.Plan(4, n, q, root, 0, gb.FLAG_CANONICAL)
    t = torch.from_numpy(x).cuda()
    y = plan(t)
    torch.cuda.synchronize()
    plan.status()
    got = y.cpu().numpy()
    for i in (0, 23, 24, 47, 48, 49):
        assert np.array_equal(got[i].astype(np.int64), orc.ntt_exact(x[i:i + 1], q, root)[0])


def test_four_step_chunk_size_setting(gb, tmp_path):
    """GBNTT_FOURSTEP_CHUNK_MB (read once per process): a child process with
    8 MiB chunks (two polynomials of 2^20 per chunk, so eleven chunks and 21
    dependent launches for 11 polynomials) gives the outputs of this process's
    default chunks, for the canonical four-step and the lane two-pass."""
    import os
    import subprocess
    import sys
    q, n, count = 998244353, 1 << 20, 11
    root = root_for(q, n)
    x = np.random.default_rng(SEED + 4100).integers(0, q, (count, n)).astype(np.int32)
    np.save(tmp_path / "x.npy", x)
    want = {}
    for name, kind, fl in (("canon_fwd", 4, gb.FLAG_CANONICAL), ("canon_inv", 5, gb.FLAG_CANONICAL),
                           ("lane_fwd", 4, 0), ("lane_inv", 5, 0)):
        want[name] = gb.Plan(kind, n, q, root, 0, fl)(torch.from_numpy(x).cuda()).cpu().numpy()
    root_dir = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    child = f"""
import numpy as np, torch, sys
sys.path.insert(0, {root_dir!r})
import ntts_on_amd_ai_engines_aie1_gb300 as gb
x = torch.from_numpy(np.load({str(tmp_path / "x.npy")!r})).cuda()
for name, kind, fl in (("canon_fwd", 4, gb.FLAG_CANONICAL), ("canon_inv", 5, gb.FLAG_CANONICAL),
                       ("lane_fwd", 4, 0), ("lane_inv", 5, 0)):
    p = gb.Plan(kind, {n}, {q}, {root}, 0, fl)
    y = p(x)
    torch.cuda.synchronize()
    p.status()
    np.save({str(tmp_path)!r} + "/" + name + ".npy", y.cpu().numpy())
"""
    env = dict(os.environ, GBNTT_FOURSTEP_CHUNK_MB="8")
    r = subprocess.run([sys.executable, "-c", child], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for name, w in want.items():
        assert np.array_equal(np.load(tmp_path / (name + ".npy")), w), name


def test_four_step_for_2_14_and_2_15_when_asked(gb, orc, tmp_path):
    """GBNTT_FOURSTEP_MIN_L=14 (read once per process) moves n = 2^14 and 2^15
    to the four-step (column pass of 4 and 8 rows): a child process checks
    forward, inverse with n^-1 and in-place runs against the exact transform."""
    import os
    import subprocess
    import sys
    q = 998244353
    rng = np.random.default_rng(SEED + 4300)
    cases = []
    for L in (14, 15):
        n = 1 << L
        x = rng.integers(-(1 << 31), 1 << 31, (3, n)).astype(np.int32)
        np.save(tmp_path / f"x{L}.npy", x)
        cases.append((L, x))
    root_dir = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    child = f"""
import numpy as np, torch, sys
sys.path.insert(0, {root_dir!r})
import ntts_on_amd_ai_engines_aie1_gb300 as gb
q = {q}
for L in (14, 15):
    n = 1 << L
    root = pow(3, (q - 1) >> L, q)
    x = torch.from_numpy(np.load({str(tmp_path)!r} + f"/x{{L}}.npy")).cuda()
    f = gb.Plan(4, n, q, root, 0, gb.FLAG_CANONICAL)
    i = gb.Plan(5, n, q, root, 0, gb.FLAG_CANONICAL | gb.FLAG_SCALE_NINV)
    y = f(x)
    z = i(y)
    w = x.clone()
    f.execute(w, w, w.shape[0])
    torch.cuda.synchronize()
    f.status(); i.status()
    np.save({str(tmp_path)!r} + f"/y{{L}}.npy", y.cpu().numpy())
    np.save({str(tmp_path)!r} + f"/z{{L}}.npy", z.cpu().numpy())
    np.save({str(tmp_path)!r} + f"/w{{L}}.npy", w.cpu().numpy())
"""
    env = dict(os.environ, GBNTT_FOURSTEP_MIN_L="14")
    r = subprocess.run([sys.executable, "-c", child], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for L, x in cases:
        root = pow(3, (q - 1) >> L, q)
        want = orc.ntt_exact(x, q, root)
        assert np.array_equal(np.load(tmp_path / f"y{L}.npy").astype(np.int64), want), L
        assert np.array_equal(np.load(tmp_path / f"w{L}.npy").astype(np.int64), want), L
        assert np.array_equal(np.load(tmp_path / f"z{L}.npy").astype(np.int64), x.astype(np.int64) % q), L
