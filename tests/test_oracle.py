"""Pins the CPU oracle: tables against the reference's own table code, kernel
loops against the O(n^2) modular DFT, and the AIE-specific rounding rules
against independent re-evaluations of the reference expressions."""
import hashlib
import json
import os
from fractions import Fraction

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_tables.json")

FAMILY = {  # reference family -> (oracle kind, which)
    "r2f16": 0, "r2i16": 1, "r4f16": 2, "r8f16": 3, "r2f32": 4, "r2g32": 5,
}


def _hash(values):
    return hashlib.sha256(" ".join(str(int(v)) for v in values).encode()).hexdigest()


def _golden():
    with open(GOLDEN) as f:
        return json.load(f)["tables"]


def _configs():
    cfgs = sorted({tuple(k.split()[:4]) for k in _golden()})
    return [(fam, int(n), int(q), int(r)) for fam, n, q, r in cfgs]


@pytest.mark.parametrize("fam,n,q,root", _configs())
def test_tables_match_reference(orc, fam, n, q, root):
    """Every per-layer table equals what src/twiddle.h builds (same values, same order)."""
    tables = _golden()
    kind = FAMILY[fam]
    plan = orc.Plan(kind, n, q, root)
    keys = [k for k in tables if tuple(k.split()[:4]) == (fam, str(n), str(q), str(root))]
    assert keys
    for key in keys:
        which, layer = int(key.split()[4]), int(key.split()[5])
        ref = tables[key]
        if which == 5:
            vals = ref["values"]
            if fam in ("r2f16", "r2f32"):
                assert vals[0] == pow(n, -1, q)            # ExtendedGCD<n, q>
                assert vals[1] == orc.lib().orc_log_root_order(q, root)
            elif fam == "r4f16":
                assert vals[0] == pow(root, n // 4, q)     # ROOT_4, ntt_r4.h:46
            continue
        mine = plan.table(which, layer)
        assert len(mine) == ref["len"], key
        assert _hash(mine) == ref["sha256"], key
        if "values" in ref:
            assert list(mine) == ref["values"], key


def test_trunc_half_rounding_quirk(orc):
    """round<T> of twiddle.h:28-31 truncates a+0.5 toward zero."""
    L = orc.lib()
    assert L.orc_round_trunc_half(-7887 * 12289 - 5284, 12289) == -7886   # -7887.43 -> -7886
    for num, den in [(65536, 12289), (1 << 32, 998244353), (-3 * 65536, 12289), (5 * 65536, 7681)]:
        exact = Fraction(num, den) + Fraction(1, 2)
        want = int(exact)  # int() truncates toward zero
        assert L.orc_round_trunc_half(num, den) == want


def _round_away(f):
    """C round(): nearest, halves away from zero (exact for float32 inputs)."""
    a = np.floor(abs(np.float64(f)) + 0.5)
    return int(a) if f >= 0 else -int(a)


def test_float_multipliers_match_ieee_single(orc):
    """twiddle.h:96 / :372 and full_reduction_kernels.cc:187 use float arithmetic."""
    L = orc.lib()
    rng = np.random.default_rng(7)
    for q in (12289, 7681, 10753):
        for tw in list(rng.integers(-(q - 1) // 2, (q - 1) // 2 + 1, 400)) + [-1168, 1, -1]:
            f = np.float32(np.float32(int(tw) * 65536) / np.float32(q))
            assert L.orc_kyber_wq(int(tw), q) == _round_away(f)
        for tw in rng.integers(0, q, 200):
            f = np.float32(np.float32(int(tw) << 31) / np.float32(q))
            assert L.orc_r8_wq_float(int(tw), q) == _round_away(f)
            assert abs(L.orc_r8_wq_exact(int(tw), q) - (int(tw) << 31) / q) <= 0.5
    assert L.orc_kyber_wq(-1168, 12289) == -6229      # C round(), half away from zero
    fs = 12286 - 12289
    f = np.float32(np.float32(fs * 65536) / np.float32(12289)) + np.float32(0.5)
    assert L.orc_fb_wq(fs, 12289) == _round_away(f)


def test_kernel_constants(orc):
    """Constants computed inside the kernels (.cc files), re-evaluated here."""
    for q in (12289, 7681, 10753):
        p = orc.Plan(orc.R2_I16_FWD, 16, q, pow({12289: 41, 7681: 17, 10753: 11}[q],
                                                 {12289: 256, 7681: 480, 10753: 672}[q], q))
        c16, c32, *_ = p.table(5)
        assert c16 == int(65536.0 / q + 0.5)             # ntt_r2_kernels.cc:388
    for q in (998244353, 469762049, 167772161, 754974721, 1073707009):
        assert int(Fraction(1 << 32, q) + Fraction(1, 2)) == orc.lib().orc_round_trunc_half(1 << 32, q)
    p = orc.Plan(orc.R4_I16_FWD, 4096, 12289, 41)
    _, _, fneg, wc, _, _ = p.table(5)
    r4 = pow(41, 1024, 12289)
    want_f = r4 if r4 <= 6144 else r4 - 12289
    assert fneg == want_f and wc == int(float(want_f * 65536) / 12289 + 0.5)   # ntt_r4_kernels.cc:112-113


RNG = np.random.default_rng(20261203)

R2_16 = [(16, 11567), (64, 3006), (256, 145), (1024, 11580), (4096, 41)]
R2_32 = [(998244353, 476477967, 256), (754974721, 704612943, 256), (1073707009, 196914830, 256),
         (998244353, 63912897, 4096), (469762049, 244412522, 4096), (167772161, 150794572, 4096),
         (754974721, 259521057, 4096), (1073707009, 992735929, 2048)]


def _fwd_equals_dft(orc, kind, n, q, root, x, **kw):
    p = orc.Plan(kind, n, q, root, **kw)
    y = p(x.astype(p.dtype)).astype(np.int64) % q
    X = orc.dft(x, q, root)
    return np.array_equal(y, X[orc.bitrev_perm(n)])


@pytest.mark.parametrize("n,root", R2_16)
def test_r2_i16_forward_is_dft_in_bitreversed_order(orc, n, root):
    x = RNG.integers(0, 12289, n)
    assert _fwd_equals_dft(orc, orc.R2_I16_FWD, n, 12289, root, x)


@pytest.mark.parametrize("n,root", [(16, 11567), (256, 145), (1024, 11580), (4096, 41)])
def test_r4_forward_is_dft_in_bitreversed_order(orc, n, root):
    x = RNG.integers(0, 12289, n)
    assert _fwd_equals_dft(orc, orc.R4_I16_FWD, n, 12289, root, x)


@pytest.mark.parametrize("q,root", [(7681, 2028), (10753, 4305)])
def test_r4_small_moduli(orc, q, root):
    x = RNG.integers(0, q, 256)
    assert _fwd_equals_dft(orc, orc.R4_I16_FWD, 256, q, root, x)


@pytest.mark.parametrize("n", [8, 64, 256, 512, 1024, 2048, 4096])
def test_r8_chained_exact_is_dft(orc, n):
    root = pow(41, 4096 // n, 12289)
    x = RNG.integers(-32768, 32768, n)
    assert _fwd_equals_dft(orc, orc.R8_I16_FWD, n, 12289, root, x, r8_exact=True)


@pytest.mark.parametrize("q,root,n", R2_32)
def test_r2_i32_forward_is_dft(orc, q, root, n):
    x = RNG.integers(0, q, n)
    assert _fwd_equals_dft(orc, orc.R2_I32_FWD, n, q, root, x)


@pytest.mark.parametrize("n,root", R2_16)
def test_r2_i16_inverse_roundtrip(orc, n, root):
    """Inverse maps BO -> NO and omits n^-1 (README.md:157-160)."""
    q = 12289
    x = RNG.integers(0, q, n)
    y = orc.Plan(orc.R2_I16_FWD, n, q, root)(x.astype(np.int16))
    z = orc.Plan(orc.R2_I16_INV, n, q, root)(y).astype(np.int64) % q
    assert np.array_equal(z, n * x % q)
    X = orc.dft(x, q, root)
    assert np.array_equal(orc.Plan(orc.R2_I16_INV, n, q, root)(X[orc.bitrev_perm(n)].astype(np.int16)).astype(np.int64) % q,
                          orc.dft(X, q, root, inverse=True))


@pytest.mark.parametrize("q,root,n", R2_32)
def test_r2_i32_inverse_roundtrip(orc, q, root, n):
    x = RNG.integers(0, q, n)
    y = orc.Plan(orc.R2_I32_FWD, n, q, root)(x.astype(np.int32))
    z = orc.Plan(orc.R2_I32_INV, n, q, root)(y).astype(np.int64) % q
    assert np.array_equal(z, n * x % q)


@pytest.mark.parametrize("n,root", [(16, 11567), (256, 145), (4096, 41)])
def test_r4_inverse_roundtrip(orc, n, root):
    q = 12289
    x = RNG.integers(0, q, n)
    y = orc.Plan(orc.R4_I16_FWD, n, q, root)(x.astype(np.int16))
    z = orc.Plan(orc.R4_I16_INV, n, q, root)(y).astype(np.int64) % q
    assert np.array_equal(z, n * x % q)


def test_r8_stage_reference_tables_defect(orc):
    """The reference's float K=31 multipliers (twiddle.h:372) are up to ~64 off,
    which breaks a few outputs of the radix-8 stage; exact multipliers do not."""
    n, q, root = 4096, 12289, 41
    ref = orc.Plan(orc.R8_I16_STAGE, n, q, root)
    exact = orc.Plan(orc.R8_I16_FWD, n, q, root, r8_exact=True)
    bad = 0
    for _ in range(20):
        x = RNG.integers(0, q, n).astype(np.int16)
        a = ref(x).astype(np.int64) % q
        b = exact.run_layer(0, x).astype(np.int64) % q
        bad += int((a != b).sum())
    assert bad < 100          # about 1e-4 of the outputs
    x = RNG.integers(0, 64, n).astype(np.int16)   # small inputs: no wrong outputs
    assert np.array_equal(ref(x).astype(np.int64) % q, exact.run_layer(0, x).astype(np.int64) % q)


def test_bitrev(orc):
    for n in (256, 512, 1024, 2048, 4096):
        x = RNG.integers(-32768, 32768, n).astype(np.int16)
        y = orc.Plan(orc.BITREV_I16, n)(x)
        assert np.array_equal(y[orc.bitrev_perm(n)], x)


def test_full_barrett(orc):
    q, n = 12289, 4096
    F = pow(n, -1, q)                       # project.cpp:154, ExtendedGCD<4096,12289> = 12286
    assert F == 12286
    x = RNG.integers(-32768, 32768, n)
    y = orc.Plan(orc.FULL_BARRETT_I16, n, q, 0, factor=F)(x.astype(np.int16)).astype(np.int64)
    assert np.array_equal(y % q, F * x % q)
    assert y.min() >= 0 and y.max() <= q


@pytest.mark.parametrize("q,g,n", [(12289, 11, 256), (7681, 17, 512), (998244353, 3, 128),
                                   (1073707009, 0, 64), (469762049, 3, 2),
                                   (1073692673, 3, 256), (1073479681, 11, 128), (1053818881, 7, 64)])
def test_exact_transform_is_the_dft(orc, q, g, n):
    """oracle.ntt_exact (the canonical families' checker) against the O(n^2)
    definition: forward in bit-reversed order, inverse from bit-reversed input,
    and the round trip returns n x."""
    root = pow(992735929, 2048 // n, q) if g == 0 else pow(g, (q - 1) // n, q)
    rng = np.random.default_rng(n + q % 101)
    x = rng.integers(-(1 << 31), 1 << 31, (3, n))
    br = orc.bitrev_perm(n)
    f = orc.ntt_exact(x, q, root)
    assert np.array_equal(f, np.stack([orc.dft(r, q, root) for r in x])[:, br])
    i = orc.ntt_exact(f, q, root, inverse=True)
    assert np.array_equal(i, np.stack([orc.dft(r[br], q, root, inverse=True) for r in f]))
    assert np.array_equal(i, (x % q) * n % q)


@pytest.mark.parametrize("kind,n,q,root,dt", [(2, 1024, 12289, 11580, np.int16), (5, 256, 998244353, 476477967, np.int32)])
def test_canonical_execution_reduces_in_threads(orc, kind, n, q, root, dt):
    """Plan(x, canonical=True): the reference's outputs reduced to [0, q) in
    the worker threads (the CPU arm of the canonical benchmark)."""
    x = np.random.default_rng(n).integers(-q, q, (37, n)).astype(dt)
    p = orc.Plan(kind, n, q, root)
    assert np.array_equal(p(x, threads=4, canonical=True).astype(np.int64), p(x).astype(np.int64) % q)
