"""ctypes binding of the C oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU baseline / reference legs.  The product library never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

R2_I16_FWD, R2_I16_INV, R4_I16_FWD, R8_I16_STAGE = 0, 1, 2, 3
R2_I32_FWD, R2_I32_INV, BITREV_I16, FULL_BARRETT_I16 = 4, 5, 6, 7
R8_I16_FWD, R4_I16_INV = 8, 9

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_plan_create.restype = ctypes.c_void_p
        L.orc_plan_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                      ctypes.c_int64, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.orc_plan_destroy.argtypes = [ctypes.c_void_p]
        L.orc_plan_layers.argtypes = [ctypes.c_void_p]
        L.orc_elem_bytes.argtypes = [ctypes.c_void_p]
        L.orc_plan_table.restype = ctypes.c_int64
        L.orc_plan_table.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.orc_run_layer.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_execute.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
        L.orc_execute_mt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                     ctypes.c_int]
        L.orc_execute_mt2.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                      ctypes.c_int, ctypes.c_int]
        L.orc_dft.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                              ctypes.c_void_p, ctypes.c_void_p]
        L.orc_ntt_exact.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p]
        for name, rt, at in [("orc_kyber_wq", ctypes.c_int16, [ctypes.c_int16, ctypes.c_int32]),
                             ("orc_r8_wq_float", ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
                             ("orc_r8_wq_exact", ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
                             ("orc_fb_wq", ctypes.c_int16, [ctypes.c_int32, ctypes.c_int32]),
                             ("orc_round_trunc_half", ctypes.c_int64, [ctypes.c_int64, ctypes.c_int64]),
                             ("orc_log_root_order", ctypes.c_int, [ctypes.c_int64, ctypes.c_int64]),
                             ("orc_bitrev", ctypes.c_uint32, [ctypes.c_uint32, ctypes.c_int])]:
            getattr(L, name).restype = rt
            getattr(L, name).argtypes = at
        _lib = L
    return _lib


def dtype_of(kind):
    return np.int32 if kind in (R2_I32_FWD, R2_I32_INV) else np.int16


class Plan:
    """One oracle pipeline (a restated graph of the reference)."""

    def __init__(self, kind, n, q=0, root=0, factor=0, r8_exact=False):
        err = ctypes.c_int(0)
        self.kind, self.n, self.q, self.root = kind, n, q, root
        self.h = lib().orc_plan_create(kind, n, q, root, factor, int(r8_exact), ctypes.byref(err))
        if not self.h:
            raise ValueError(f"oracle plan rejected (code {err.value}): kind={kind} n={n} q={q} root={root}")
        self.dtype = dtype_of(kind)
        self.layers = lib().orc_plan_layers(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_plan_destroy(self.h)
            self.h = None

    def table(self, which, layer=0):
        n = lib().orc_plan_table(self.h, which, layer, None)
        out = np.zeros(n, dtype=np.int64)
        lib().orc_plan_table(self.h, which, layer, out.ctypes.data)
        return out

    def run_layer(self, layer, x):
        x = np.ascontiguousarray(x, dtype=self.dtype)
        y = np.empty_like(x)
        rc = lib().orc_run_layer(self.h, layer, x.ctypes.data, y.ctypes.data)
        assert rc == 0
        return y

    def __call__(self, x, threads=1, canonical=False):
        """The pipeline on every polynomial of x; canonical: outputs reduced
        to [0, q) (inside the worker threads)."""
        x = np.ascontiguousarray(x, dtype=self.dtype)
        assert x.size % self.n == 0
        y = np.empty_like(x)
        batch = x.size // self.n
        if canonical:
            lib().orc_execute_mt2(self.h, x.ctypes.data, y.ctypes.data, batch, max(1, threads), 1)
        elif threads > 1:
            lib().orc_execute_mt(self.h, x.ctypes.data, y.ctypes.data, batch, threads)
        else:
            lib().orc_execute(self.h, x.ctypes.data, y.ctypes.data, batch)
        return y


def dft(x, q, root, inverse=False):
    x = np.ascontiguousarray(x, dtype=np.int64)
    y = np.empty_like(x)
    lib().orc_dft(x.size, q, root, int(inverse), x.ctypes.data, y.ctypes.data)
    return y


def ntt_exact(x, q, root, inverse=False):
    """The exact transform of every row of x (any integer dtype, taken mod q),
    canonical residues as int64, in the designs' orders: forward natural in /
    bit-reversed out, inverse bit-reversed in / natural out (no n^-1)."""
    x = np.ascontiguousarray(x, dtype=np.int64)
    n = x.shape[-1]
    flat = x.reshape(-1, n)
    out = np.empty_like(flat)
    for r in range(flat.shape[0]):
        lib().orc_ntt_exact(n, q, root, int(inverse), flat[r].ctypes.data, out[r].ctypes.data)
    return out.reshape(x.shape)


def bitrev_perm(n):
    L = n.bit_length() - 1
    return np.array([lib().orc_bitrev(i, L) for i in range(n)], dtype=np.int64)
