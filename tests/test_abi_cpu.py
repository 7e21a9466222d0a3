"""C-ABI checks that need no GPU: the library loads, exports every function
include/gb300_ntt.h declares, validates parameters like the reference's
static_asserts, and builds tables identical to the reference's."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def gb():
    import ntts_on_amd_ai_engines_aie1_gb300 as gb
    from ntts_on_amd_ai_engines_aie1_gb300 import build
    build.build()
    return gb


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(gbntt_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(gb):
    names = _declared("gb300_ntt.h")
    assert "gbntt_plan_create" in names and "gbntt_execute" in names
    lib = gb.lib()
    for name in names:
        assert hasattr(lib, name), f"{name} missing from libgb300ntt.so"
    assert lib.gbntt_abi_version() == 1


def test_product_does_not_link_the_oracle(gb):
    """The product library must not depend on anything under oracle/."""
    data = open(gb.LIB_PATH, "rb").read()
    assert b"liboracle" not in data and b"orc_plan" not in data


ERR = [
    # (kind, n, q, root, factor, expected status)  -- reference static_asserts
    (0, 1000, 12289, 41, 0, 2),       # power of two (auxiliary.h:11)
    (0, 4096, 12288, 41, 0, 3),       # even modulus
    (0, 4096, 40961, 3, 0, 3),        # above 2^16/3 for int16 lanes
    (0, 4096, 12289, 2, 0, 4),        # ROOT is not correct (auxiliary.h:37,44)
    (0, 2048, 12289, 41, 0, 4),       # root of order 4096 used for n = 2048
    (2, 2048, 12289, 1681, 0, 5),     # radix-4 needs an even layer count (ntt_r4.h:62-63)
    (11, 16, 12289, 11567, 0, 6),     # unknown kind
    (7, 4096, 12289, 0, 12289, 1),    # factor outside [0, q)
    (3, 8, 12289, 4134, 0, 2),        # radix-8 stage needs n >= 16
]


@pytest.mark.parametrize("kind,n,q,root,factor,status", ERR)
def test_validation_errors(gb, kind, n, q, root, factor, status):
    ln = ctypes.c_int64(0)
    rc = gb.lib().gbntt_host_tables(kind, n, q, root, factor, 0, 0, None, 0, ctypes.byref(ln))
    assert rc == status
    assert gb.lib().gbntt_last_error()


def _pairs(tab):
    return tab.reshape(-1, 2)


CFG16 = [(16, 11567), (256, 145), (1024, 11580), (4096, 41)]
CFG32 = [(998244353, 63912897, 4096), (754974721, 259521057, 4096), (1073707009, 992735929, 2048)]


@pytest.mark.parametrize("n,root", CFG16)
def test_host_tables_r2_i16(gb, orc, n, root):
    q = 12289
    L = n.bit_length() - 1
    fwd = _pairs(gb.host_tables(gb.Kind.R2_I16_FWD, n, q, root))
    last = orc.Plan(orc.R2_I16_FWD, n, q, root).table(0, L - 1)       # layer L-1 holds the whole table
    assert np.array_equal(fwd[:, 0], last[: n // 2]) and np.array_equal(fwd[:, 1], last[n // 2:])
    inv = _pairs(gb.host_tables(gb.Kind.R2_I16_INV, n, q, root))
    op = orc.Plan(orc.R2_I16_INV, n, q, root)
    for i in range(1, L):
        rep = n >> (i + 1)
        tw, wq = op.table(0, i), op.table(1, i)
        for t in range(1 << i):
            g, e = divmod(t, 2)
            assert tuple(inv[(1 << i) + t]) == (tw[2 * g * rep + e], wq[2 * g * rep + e])


@pytest.mark.parametrize("q,root,n", CFG32)
def test_host_tables_r2_i32(gb, orc, q, root, n):
    fwd = _pairs(gb.host_tables(gb.Kind.R2_I32_FWD, n, q, root))
    L = n.bit_length() - 1
    last = orc.Plan(orc.R2_I32_FWD, n, q, root).table(0, L - 1)
    assert np.array_equal(fwd[:, 0], last[: n // 2]) and np.array_equal(fwd[:, 1], last[n // 2:])
    inv = _pairs(gb.host_tables(gb.Kind.R2_I32_INV, n, q, root))
    first = orc.Plan(orc.R2_I32_INV, n, q, root).table(0, 0)          # GS layer 0 = level L-1
    assert np.array_equal(inv[:, 0], first[: n // 2]) and np.array_equal(inv[:, 1], first[n // 2:])


@pytest.mark.parametrize("n,q,root", [(16, 12289, 11567), (256, 12289, 145), (1024, 12289, 11580),
                                      (4096, 12289, 41), (256, 7681, 2028), (256, 10753, 4305)])
def test_host_tables_r4(gb, orc, n, q, root):
    tab = _pairs(gb.host_tables(gb.Kind.R4_I16_FWD, n, q, root))
    op = orc.Plan(orc.R4_I16_FWD, n, q, root)
    off = 0
    for l in range((n.bit_length() - 1) // 2):
        f = op.table(0, l)
        for b in range(4 ** l):
            for d in range(4):
                assert tuple(tab[off + 4 * b + d]) == (f[d * n // 4 + b], f[n + d * n // 4 + b])
        off += 4 * 4 ** l
    consts = gb.host_tables(gb.Kind.R4_I16_FWD, n, q, root, which=1)
    _, _, fneg, wc, *_ = op.table(5)
    assert consts[1] == fneg and consts[2] == wc


@pytest.mark.parametrize("n,root", [(64, 3006), (512, 11121), (4096, 41)])
def test_host_tables_r8_stage(gb, orc, n, root):
    q = 12289
    tab = _pairs(gb.host_tables(gb.Kind.R8_I16_STAGE, n, q, root))
    op = orc.Plan(orc.R8_I16_STAGE, n, q, root)
    tw, wq = op.table(3), op.table(4)
    M = n // 8
    for i in range(M):
        for k in range(8):
            idx = 16 * (i // 2) + 2 * k + i % 2
            assert tuple(tab[k * M + i]) == (tw[idx], wq[idx])
    f8 = gb.host_tables(gb.Kind.R8_I16_STAGE, n, q, root, which=2).reshape(8, 8)
    ref = op.table(2)          # MAC-lane layout of twiddle.h:326-344
    for i in range(2):
        for j in range(2):
            for k in range(4):
                for l in range(4):
                    pos = 32 * i + 16 * j + 4 * k + [0, 2, 1, 3][l]
                    assert f8[4 * i + l, 4 * j + k] == ref[pos]


def test_full_barrett_constants(gb, orc):
    c = gb.host_tables(gb.Kind.FULL_BARRETT_I16, 4096, 12289, 0, 12286, which=1)
    o = orc.Plan(orc.FULL_BARRETT_I16, 4096, 12289, 0, factor=12286).table(5)
    assert c[3] == o[4] and c[4] == o[5]


def test_server_host_logic(gb):
    """Admission arena (first fit, coalescing, no over-admission) and percentiles."""
    assert gb.lib().gbntt_server_selftest() == 0, gb.lib().gbntt_last_error()
