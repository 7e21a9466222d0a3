"""GB300 NTT library: Python host side over the C ABI of libgb300ntt.so.

The reference builds one ADF graph per design, constructed with compile-time
template parameters and run with ``graph.init(); graph.run(N); graph.end()``
(src/project.cpp:161-164).  This module mirrors those graph classes:

    NTT(LENGTH, MODULUS, ROOT, NTT_TYPE.TYPE_NTT_NO_to_BO)          src/ntt.h:43
    NTT_INT32(LENGTH, MODULUS, ROOT, NTT_INT32_TYPE.FORWARD_CT_NO_TO_BO)   src/ntt_int32.h:27
    NTT_R4(LENGTH, MODULUS, ROOT)                                    src/ntt_r4.h:30
    NTT_R8(MODULUS, LENGTH, ROOT)                                    src/ntt_r8.h:22
    BITREVERSE(LENGTH)                                               src/standalone_units.h:17
    FULL_BARRETT_MULTIPLICATION(LENGTH, MODULUS, FACTOR)             src/standalone_units.h:40

and ``dut_for_config(NTT_CONFIG)`` selects a design like src/project.cpp:139-157.
The in_data / out_data ports become device buffers (torch tensors or raw
pointers); ``run(iterations)`` transforms that many polynomials in one launch.
The compute path is the CUDA library only: importing this module fails loudly
when libgb300ntt.so is missing or cannot be loaded.
"""
import ctypes
import enum
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgb300ntt.so")


class Kind(enum.IntEnum):
    R2_I16_FWD = 0
    R2_I16_INV = 1
    R4_I16_FWD = 2
    R8_I16_STAGE = 3
    R2_I32_FWD = 4
    R2_I32_INV = 5
    BITREV_I16 = 6
    FULL_BARRETT_I16 = 7
    R8_I16_FWD = 8
    R4_I16_INV = 9


FLAG_CANONICAL = 0x1
FLAG_R8_EXACT = 0x2
FLAG_R8_FLOAT = 0x4
FLAG_NATURAL_ORDER = 0x8     # bit reversal fused: forward returns / inverse takes natural order
FLAG_SCALE_NINV = 0x10       # int16 inverse: full Barrett multiplication by n^-1 fused
FLAG_LANE_EXACT = 0x20       # with FLAG_CANONICAL: the reference's lane arithmetic, then reduced

STATUS = {0: "ok", 1: "invalid argument", 2: "unsupported length", 3: "invalid modulus",
          4: "root of unity has the wrong order", 5: "radix-4 needs an even number of layers",
          6: "unknown design kind", 7: "CUDA error", 8: "out of memory", 9: "timeout",
          10: "admission refused"}


class NTTError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Segment(ctypes.Structure):
    """gbntt_segment: plan, device input, device output, polynomial count."""
    _fields_ = [("plan", ctypes.c_void_p), ("d_in", ctypes.c_void_p), ("d_out", ctypes.c_void_p),
                ("count", ctypes.c_uint64)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_uint32), ("max_requests_per_batch", ctypes.c_uint32),
                ("device_bytes", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("refused", ctypes.c_uint64), ("polynomials", ctypes.c_uint64),
                ("microbatches", ctypes.c_uint64), ("launches", ctypes.c_uint64), ("p50_us", ctypes.c_double),
                ("p99_us", ctypes.c_double), ("max_us", ctypes.c_double), ("polys_per_s", ctypes.c_double),
                ("arena_bytes", ctypes.c_uint64), ("peak_arena_bytes", ctypes.c_uint64)]


_lib = None


def lib():
    """The loaded libgb300ntt.so (raises if it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with "
                              "`python -m ntts_on_amd_ai_engines_aie1_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, u64, i64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int
        L.gbntt_plan_create.argtypes = [ctypes.POINTER(vp), i32, u32, i64, i64, i64, u32]
        L.gbntt_plan_destroy.argtypes = [vp]
        L.gbntt_execute.argtypes = [vp, vp, vp, u64, vp]
        L.gbntt_execute_host.argtypes = [vp, vp, vp, u64, vp]
        L.gbntt_plan_query.argtypes = [vp, i32, ctypes.POINTER(i64)]
        L.gbntt_host_tables.argtypes = [i32, u32, i64, i64, i64, u32, i32, ctypes.POINTER(i64), i64,
                                        ctypes.POINTER(i64)]
        L.gbntt_batch_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Segment), u32, u32]
        L.gbntt_batch_execute.argtypes = [vp, vp]
        L.gbntt_batch_graph_launch.argtypes = [vp, vp]
        L.gbntt_batch_set_io.argtypes = [vp, u32, vp, vp]
        L.gbntt_batch_execute_host.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), vp]
        L.gbntt_batch_status.argtypes = [vp]
        L.gbntt_batch_query.argtypes = [vp, i32, ctypes.POINTER(i64)]
        L.gbntt_batch_destroy.argtypes = [vp]
        L.gbntt_server_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(vp), u32, ctypes.POINTER(ServerConfig)]
        L.gbntt_server_submit.argtypes = [vp, u32, vp, vp, u64, ctypes.POINTER(u64)]
        L.gbntt_server_wait.argtypes = [vp, u64, u32]
        L.gbntt_server_drain.argtypes = [vp, u32]
        L.gbntt_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats), i32]
        L.gbntt_server_destroy.argtypes = [vp]
        L.gbntt_server_submit_schedule.argtypes = [vp, u64, ctypes.POINTER(u32), ctypes.POINTER(vp),
                                                   ctypes.POINTER(vp), ctypes.POINTER(u64),
                                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(u64)]
        L.gbntt_plan_status.argtypes = [vp]
        L.gbntt_batch_execute_noalloc.argtypes = [ctypes.POINTER(Segment), u32, vp]
        L.gbntt_noalloc_status.argtypes = []
        L.gbntt_set_wait_limit.argtypes = [u32]
        L.gbntt_launch_count.restype = u64
        L.gbntt_last_error.restype = ctypes.c_char_p
        L.gbntt_status_string.restype = ctypes.c_char_p
        L.gbntt_status_string.argtypes = [i32]
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise NTTError(rc, lib().gbntt_last_error().decode())


def launch_count():
    """Kernels launched by the library so far in this process."""
    return int(lib().gbntt_launch_count())


WAIT_POLLS_DEFAULT = 1 << 22


def set_wait_limit(polls=WAIT_POLLS_DEFAULT):
    """Poll limit of the persistent kernel's bounded tile-load waits for
    launches enqueued from now on (default 2^22; 0: every wait gives up at
    once).  Small limits make the waits run out on purpose, to test the
    failure path."""
    _check(lib().gbntt_set_wait_limit(int(polls)))


def noalloc_status():
    """Raises NTTError (GBNTT_ERR_TIMEOUT) if a launch of the no-allocation
    batch entry point ran out of a bounded wait; clears the error."""
    _check(lib().gbntt_noalloc_status())


def host_tables(kind, n, q=0, root=0, factor=0, flags=0, which=0):
    """The plan's host-side table (no CUDA call): which=0 (tw, w') pairs, 1 constants, 2 F8."""
    import numpy as np
    ln = ctypes.c_int64(0)
    _check(lib().gbntt_host_tables(int(kind), n, q, root, factor, flags, which, None, 0, ctypes.byref(ln)))
    out = np.zeros(ln.value, dtype=np.int64)
    _check(lib().gbntt_host_tables(int(kind), n, q, root, factor, flags, which,
                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ln.value,
                                   ctypes.byref(ln)))
    return out


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _stream_ptr(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Plan:
    """One design instance: tables built once and kept on the device."""

    def __init__(self, kind, n, q=0, root=0, factor=0, flags=0):
        h = ctypes.c_void_p()
        _check(lib().gbntt_plan_create(ctypes.byref(h), int(kind), n, q, root, factor, flags))
        self._h = h
        self.kind, self.n, self.q, self.root, self.factor, self.flags = Kind(kind), n, q, root, factor, flags
        self.elem_bytes = self.query(2)
        self.stages = self.query(3)

    @property
    def handle(self):
        return self._h.value

    def query(self, what):
        v = ctypes.c_int64(0)
        _check(lib().gbntt_plan_query(self._h, what, ctypes.byref(v)))
        return v.value

    @property
    def dtype(self):
        import torch
        return torch.int32 if self.elem_bytes == 4 else torch.int16

    def execute(self, d_in, d_out, batch, stream=None):
        """Raw-pointer launch (device buffers)."""
        _check(lib().gbntt_execute(self._h, _ptr(d_in), _ptr(d_out), batch, _stream_ptr(stream)))

    def __call__(self, x, out=None, stream=None):
        """Transforms a (batch, n) or (n,) device tensor; returns the output tensor."""
        import torch
        if not x.is_cuda or x.dtype != self.dtype or not x.is_contiguous():
            raise NTTError(1, f"input must be a contiguous CUDA {self.dtype} tensor")
        if x.numel() % self.n:
            raise NTTError(1, "input size is not a multiple of n")
        if out is None:
            out = torch.empty_like(x)
        self.execute(x, out, x.numel() // self.n, stream)
        return out

    def status(self):
        """Raises NTTError (GBNTT_ERR_TIMEOUT) if a bounded wait in an earlier
        launch of this plan ran out; clears it."""
        _check(lib().gbntt_plan_status(self.handle))

    def execute_host(self, h_in, h_out, batch=None, stream=None):
        """Host buffers (numpy arrays or torch CPU tensors); synchronous."""
        def p(a):
            return a.ctypes.data if hasattr(a, "ctypes") else a.data_ptr()
        nb = batch if batch is not None else (h_in.size if hasattr(h_in, "size") and not callable(h_in.size)
                                              else h_in.numel()) // self.n
        _check(lib().gbntt_execute_host(self._h, p(h_in), p(h_out), nb, _stream_ptr(stream)))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().gbntt_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many polynomials of several designs in one persistent launch.

    segments: list of (plan, input tensor, output tensor); the tensors' first
    dimension (or numel / n) gives the polynomial count.  The batch keeps
    references to plans and tensors so they outlive it."""

    def __init__(self, segments, flags=0):
        self._keep = list(segments)
        arr = (Segment * len(segments))()
        for i, (plan, x, y) in enumerate(segments):
            arr[i].plan = plan.handle
            arr[i].d_in = _ptr(x)
            arr[i].d_out = _ptr(y)
            arr[i].count = (x.numel() // plan.n) if hasattr(x, "numel") else 0
        h = ctypes.c_void_p()
        _check(lib().gbntt_batch_create(ctypes.byref(h), arr, len(segments), flags))
        self._h = h

    def execute(self, stream=None):
        _check(lib().gbntt_batch_execute(self._h, _stream_ptr(stream)))

    def graph_launch(self, stream=None):
        _check(lib().gbntt_batch_graph_launch(self._h, _stream_ptr(stream)))

    def execute_host(self, h_in, h_out, stream=None):
        """Host arrays (one per segment, pinned for full bandwidth); synchronous."""
        def p(a):
            return a.ctypes.data if hasattr(a, "ctypes") else a.data_ptr()
        ins = (ctypes.c_void_p * len(h_in))(*[p(a) for a in h_in])
        outs = (ctypes.c_void_p * len(h_out))(*[p(a) for a in h_out])
        _check(lib().gbntt_batch_execute_host(self._h, ins, outs, _stream_ptr(stream)))

    def set_io(self, seg, x, y):
        plan = self._keep[seg][0]
        self._keep[seg] = (plan, x, y)
        _check(lib().gbntt_batch_set_io(self._h, seg, _ptr(x), _ptr(y)))

    def status(self):
        _check(lib().gbntt_batch_status(self._h))

    def query(self, what):
        v = ctypes.c_int64(0)
        _check(lib().gbntt_batch_query(self._h, what, ctypes.byref(v)))
        return v.value

    @property
    def launches(self):
        return self.query(0)

    @property
    def tiles(self):
        return self.query(1)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().gbntt_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _hptr(a):
    return a.ctypes.data if hasattr(a, "ctypes") else a.data_ptr()


class Server:
    """Continuous-batching request server over a fixed list of plans."""

    def __init__(self, plans, slots=8, device_bytes=0, max_requests_per_batch=0):
        self.plans = list(plans)
        arr = (ctypes.c_void_p * len(self.plans))(*[p.handle for p in self.plans])
        cfg = ServerConfig(slots, max_requests_per_batch, device_bytes)
        h = ctypes.c_void_p()
        _check(lib().gbntt_server_create(ctypes.byref(h), arr, len(self.plans), ctypes.byref(cfg)))
        self._h = h

    def submit(self, plan, h_in, h_out, count=None):
        t = ctypes.c_uint64(0)
        cnt = count if count is not None else (h_in.size if hasattr(h_in, "ctypes") else h_in.numel()) \
            // self.plans[plan].n
        _check(lib().gbntt_server_submit(self._h, plan, _hptr(h_in), _hptr(h_out), cnt, ctypes.byref(t)))
        return t.value

    def wait(self, ticket, timeout_ms=60000):
        """0 when done; raises NTTError (timeout, refused) otherwise."""
        _check(lib().gbntt_server_wait(self._h, ticket, timeout_ms))

    def try_wait(self, ticket, timeout_ms=60000):
        return lib().gbntt_server_wait(self._h, ticket, timeout_ms)

    def drain(self, timeout_ms=600000):
        _check(lib().gbntt_server_drain(self._h, timeout_ms))

    def submit_schedule(self, plan_idx, h_ins, h_outs, counts, arrival_us):
        n = len(plan_idx)
        P = (ctypes.c_uint32 * n)(*plan_idx)
        I = (ctypes.c_void_p * n)(*[_hptr(a) for a in h_ins])
        O = (ctypes.c_void_p * n)(*[_hptr(a) for a in h_outs])
        C = (ctypes.c_uint64 * n)(*counts)
        A = (ctypes.c_double * n)(*arrival_us)
        T = (ctypes.c_uint64 * n)()
        _check(lib().gbntt_server_submit_schedule(self._h, n, P, I, O, C, A, T))
        return list(T)

    def stats(self, reset=False):
        st = ServerStats()
        _check(lib().gbntt_server_get_stats(self._h, ctypes.byref(st), int(reset)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().gbntt_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# mirrors of the reference graph classes
# ---------------------------------------------------------------------------

class NTT_TYPE(enum.Enum):
    TYPE_NTT_NO_to_BO = 0     # forward, natural -> bit-reversed (src/ntt.h:31)
    TYPE_INTT_BO_to_NO = 1    # inverse, bit-reversed -> natural (src/ntt.h:32)


class NTT_INT32_TYPE(enum.Enum):
    FORWARD_CT_NO_TO_BO = 0   # src/ntt_int32.h:20
    INVERSE_GS_BO_TO_NO = 1   # src/ntt_int32.h:21


class NTT_R4_TYPE(enum.Enum):
    FORWARD_CT_NO_TO_BO = 0   # src/ntt_r4.h:24
    INVERSE_BO_TO_NO = 1      # src/ntt_r4.h:18-20 (bit-reversal + forward with inverse twiddles)


class _Graph:
    """graph.init(); graph.run(N); graph.end() over device in/out ports."""

    def __init__(self, kind, length, modulus=0, root=0, factor=0, flags=0):
        self._args = (kind, length, modulus, root, factor, flags)
        self.plan = None
        self.in_data = None
        self.out_data = None

    @property
    def NTT_LENGTH(self):
        return self._args[1]

    def init(self):
        if self.plan is None:
            self.plan = Plan(*self._args)
        return self

    def run(self, iterations=1, in_data=None, out_data=None, stream=None):
        self.init()
        src = in_data if in_data is not None else self.in_data
        dst = out_data if out_data is not None else self.out_data
        if dst is None:
            import torch
            dst = torch.empty_like(src)
            self.out_data = dst
        self.plan.execute(src, dst, iterations, stream)
        return dst

    def end(self):
        if self.plan is not None:
            self.plan.close()
            self.plan = None


class NTT(_Graph):
    """Radix-2 int16 pipeline (src/ntt.h:43), forward or inverse."""

    def __init__(self, LENGTH, MODULUS, ROOT, TYPE=NTT_TYPE.TYPE_NTT_NO_to_BO, flags=0):
        kind = Kind.R2_I16_FWD if TYPE == NTT_TYPE.TYPE_NTT_NO_to_BO else Kind.R2_I16_INV
        super().__init__(kind, LENGTH, MODULUS, ROOT, 0, flags)


class NTT_INT32(_Graph):
    """Radix-2 int32 pipeline (src/ntt_int32.h:27)."""

    def __init__(self, LENGTH, MODULUS, ROOT, TYPE=NTT_INT32_TYPE.FORWARD_CT_NO_TO_BO, flags=0):
        kind = Kind.R2_I32_FWD if TYPE == NTT_INT32_TYPE.FORWARD_CT_NO_TO_BO else Kind.R2_I32_INV
        super().__init__(kind, LENGTH, MODULUS, ROOT, 0, flags)


class NTT_R4(_Graph):
    """Radix-4 int16 pipeline (src/ntt_r4.h:30)."""

    def __init__(self, LENGTH, MODULUS, ROOT, TYPE=NTT_R4_TYPE.FORWARD_CT_NO_TO_BO, flags=0):
        kind = Kind.R4_I16_FWD if TYPE == NTT_R4_TYPE.FORWARD_CT_NO_TO_BO else Kind.R4_I16_INV
        super().__init__(kind, LENGTH, MODULUS, ROOT, 0, flags)


class NTT_R8(_Graph):
    """Radix-8 int16 (src/ntt_r8.h:22).  stages="one" is the reference graph
    (one stage, float multipliers); stages="all" chains every stage."""

    def __init__(self, MODULUS, LENGTH, ROOT, stages="one", flags=0):
        kind = Kind.R8_I16_STAGE if stages == "one" else Kind.R8_I16_FWD
        super().__init__(kind, LENGTH, MODULUS, ROOT, 0, flags)


class BITREVERSE(_Graph):
    """Bit-reversal unit (src/standalone_units.h:17; n in 256..4096 there)."""

    def __init__(self, LENGTH):
        super().__init__(Kind.BITREV_I16, LENGTH)


class FULL_BARRETT_MULTIPLICATION(_Graph):
    """out = FACTOR * in mod q in [0, q] (src/standalone_units.h:40)."""

    def __init__(self, LENGTH, MODULUS, FACTOR):
        super().__init__(Kind.FULL_BARRETT_I16, LENGTH, MODULUS, 0, FACTOR)


# parameters of src/project.cpp:47-51
Q_INT16, ROOT_INT16 = 12289, 41
Q_INT32, ROOT_INT32 = 1073707009, 992735929
BITREV_N = 4096


def dut_for_config(NTT_CONFIG, BITREV_N=BITREV_N):
    """The design under test of src/project.cpp:139-157 for NTT_CONFIG 0..7."""
    if NTT_CONFIG == 0:
        return NTT(4096, Q_INT16, ROOT_INT16, NTT_TYPE.TYPE_NTT_NO_to_BO)
    if NTT_CONFIG == 1:
        return NTT(4096, Q_INT16, ROOT_INT16, NTT_TYPE.TYPE_INTT_BO_to_NO)
    if NTT_CONFIG == 2:
        return NTT_R4(4096, Q_INT16, ROOT_INT16)
    if NTT_CONFIG == 3:
        return NTT_R8(Q_INT16, 4096, ROOT_INT16)
    if NTT_CONFIG == 4:
        return NTT_INT32(2048, Q_INT32, ROOT_INT32, NTT_INT32_TYPE.FORWARD_CT_NO_TO_BO)
    if NTT_CONFIG == 5:
        return NTT_INT32(2048, Q_INT32, ROOT_INT32, NTT_INT32_TYPE.INVERSE_GS_BO_TO_NO)
    if NTT_CONFIG == 6:
        return BITREVERSE(BITREV_N)
    if NTT_CONFIG == 7:
        return FULL_BARRETT_MULTIPLICATION(4096, Q_INT16, pow(4096, -1, Q_INT16))
    raise ValueError("Unknown NTT_CONFIG, see the table at the top of src/project.cpp")
