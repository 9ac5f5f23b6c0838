"""ctypes view of the C ABI in include/ffgpu.h (libffgpu.so).

This is the boundary a non-Python caller binds (ctypes here; cgo, JNI and
other FFIs bind the same symbols); tests and bench.py use it to drive the
kernels with device pointers (e.g. torch tensors' data_ptr()) and CUDA
streams.
"""

import ctypes
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libffgpu.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "ffgpu.h")

OK = 0
EINVAL = -1
ECUDA = -2
ENOMEM = -3
EASSERT = -4
ETIMEOUT = -5
ECANCELLED = -6
STATUS_ASSERT = 0xFF


class FFGPUError(RuntimeError):
    def __init__(self, rc, msg):
        super().__init__(f"ffgpu error {rc}: {msg}")
        self.rc = rc


_lib = None


def declared_symbols():
    """Function names declared in include/ffgpu.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(ffgpu_\w+)\s*\(", text, re.M)))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libffgpu.so is not built")
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


_P = ctypes.c_void_p
_SZ = ctypes.c_size_t
_I = ctypes.c_int
_U32 = ctypes.c_uint32
_PP = ctypes.POINTER(ctypes.c_void_p)


def _declare(L):
    sig = {
        "ffgpu_last_error": (ctypes.c_char_p, []),
        "ffgpu_version": (ctypes.c_char_p, []),
        "ffgpu_init": (_I, [_I]),
        "ffgpu_kernel_launches": (ctypes.c_uint64, []),
        "ffgpu_default_stream": (_P, []),
        "ffgpu_synchronize": (_I, [_P]),
        "ffgpu_timing_enable": (_I, [_I]),
        "ffgpu_set_host_chunk_blocks": (_I, [_SZ]),
        "ffgpu_timing_collect": (_I, [ctypes.c_char_p, _SZ, ctypes.POINTER(_SZ)]),
        "ffgpu_host_alloc": (_I, [_SZ, _PP]),
        "ffgpu_host_free": (_I, [_P]),
        "ffgpu_rs256_create": (_I, [_I, _I, _I, _PP]),
        "ffgpu_rs256_destroy": (_I, [_P]),
        "ffgpu_rs256_generator": (_I, [_P, _P, _P]),
        "ffgpu_rs256_encode": (_I, [_P, _P, _SZ, _SZ, _P, _P]),
        "ffgpu_rs256_decode": (_I, [_P, _P, _P, _SZ, _SZ, _P, _P]),
        "ffgpu_rs256_synds": (_I, [_P, _P, _P, _SZ, _SZ, _P, _P]),
        "ffgpu_rs256_encode_host": (_I, [_P, _P, _SZ, _SZ, _P]),
        "ffgpu_rs256_decode_host": (_I, [_P, _P, _P, _SZ, _SZ, _P]),
        "ffgpu_rs256_synds_host": (_I, [_P, _P, _P, _SZ, _SZ, _P]),
        "ffgpu_rs256_set_table_only": (_I, [_P, _I]),
        "ffgpu_rs256_decode_noalloc": (_I, [_P, _P, _P, _SZ, _SZ, _P, _P]),
        "ffgpu_rsi16_create": (_I, [_SZ, _SZ, _U32, _PP]),
        "ffgpu_rsi16_destroy": (_I, [_P]),
        "ffgpu_rsi16_repair_counters": (_I, [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64), _I]),
        "ffgpu_rsi16_info": (_I, [_P, ctypes.POINTER(_U32), ctypes.POINTER(_SZ)]),
        "ffgpu_rsi16_encode": (_I, [_P, _P, _SZ, _P, _P]),
        "ffgpu_rsi16_encode_interleaved": (_I, [_P, _P, _SZ, _SZ, _P, _P]),
        "ffgpu_rsi16_repair": (_I, [_P, _P, _P, _SZ, _P, _P]),
        "ffgpu_rsi16_repair_interleaved": (_I, [_P, _P, _P, _SZ, _P, _SZ, _P, _P]),
        "ffgpu_rsi16_repair_known": (_I, [_P, _P, _P, _SZ, _P, _SZ, _P, _P]),
        "ffgpu_rsi16_synd": (_I, [_P, _P, _P, _SZ, _P, _P]),
        "ffgpu_rsi16_sugiyama": (_I, [_P, _P, _SZ, _P, _P, _P, _P]),
        "ffgpu_rsi16_roots": (_I, [_P, _P, _P, _P]),
        "ffgpu_rsi16_encode_host": (_I, [_P, _P, _SZ, _SZ, _P]),
        "ffgpu_rsi16_repair_host": (_I, [_P, _P, _P, _SZ, _SZ, _P, ctypes.c_long, _P]),
        "ffgpu_circ16_create": (_I, [_SZ, _SZ, _SZ, _SZ, _SZ, _U32, _PP]),
        "ffgpu_circ16_destroy": (_I, [_P]),
        "ffgpu_circ16_info": (_I, [_P, ctypes.POINTER(_SZ), ctypes.POINTER(_SZ)]),
        "ffgpu_circ16_encode": (_I, [_P, _P, _SZ, _P, _P]),
        "ffgpu_circ16_repair": (_I, [_P, _P, _P, _SZ, _P, _P]),
        "ffgpu_circ16_find_outer_error_locations": (_I, [_P, _P, _P, _SZ, _P, _P]),
        "ffgpu_circ16_encode_host": (_I, [_P, _P, _SZ, _P]),
        "ffgpu_circ16_repair_host": (_I, [_P, _P, _P, _SZ, _P]),
        "ffgpu_server_create": (_I, [_SZ, _I, _I, _PP]),
        "ffgpu_server_destroy": (_I, [_P]),
        "ffgpu_server_submit_rs256": (_I, [_P, _P, _I, _P, _P, _SZ, _SZ, _P, ctypes.POINTER(ctypes.c_uint64)]),
        "ffgpu_server_submit_rsi16": (_I, [_P, _P, _I, _P, _P, _SZ, _P, ctypes.POINTER(ctypes.c_uint64)]),
        "ffgpu_server_submit_circ16": (_I, [_P, _P, _I, _P, _P, _SZ, _P, ctypes.POINTER(ctypes.c_uint64)]),
        "ffgpu_server_poll": (_I, [_P, ctypes.c_uint64, ctypes.POINTER(_I)] + [ctypes.POINTER(ctypes.c_double)] * 3),
        "ffgpu_server_wait": (_I, [_P, ctypes.c_uint64, ctypes.c_double]),
        "ffgpu_server_release": (_I, [_P, ctypes.c_uint64]),
        "ffgpu_server_cancel": (_I, [_P, ctypes.c_uint64]),
        "ffgpu_server_debug_fail_allocs": (_I, [_I]),
        "ffgpu_batch_create": (_I, [_PP]),
        "ffgpu_batch_destroy": (_I, [_P]),
        "ffgpu_batch_clear": (_I, [_P]),
        "ffgpu_batch_add_rs256": (_I, [_P, _P, _I, _P, _P, _SZ, _SZ, _P]),
        "ffgpu_batch_add_rsi16": (_I, [_P, _P, _I, _P, _P, _SZ, _P]),
        "ffgpu_batch_add_circ16": (_I, [_P, _P, _I, _P, _P, _SZ, _P]),
        "ffgpu_batch_plan": (_I, [_P, _I, _P]),
        "ffgpu_batch_capture": (_I, [_P, _P]),
        "ffgpu_batch_launch": (_I, [_P, _P]),
        "ffgpu_batch_info": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                                  ctypes.POINTER(_SZ), ctypes.POINTER(ctypes.c_uint)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args


def check(rc):
    if rc != OK:
        raise FFGPUError(rc, lib().ffgpu_last_error().decode())
    return rc


def call(name, *args):
    return check(getattr(lib(), name)(*args))


class RS256Code:
    """Device-resident RS256 code handle (ffgpu_rs256)."""

    def __init__(self, ecc_len, primitive=2, polynomial=0x11D):
        h = ctypes.c_void_p()
        call("ffgpu_rs256_create", ecc_len, primitive, polynomial, ctypes.byref(h))
        self.h = h
        self.ecc_len = ecc_len

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ffgpu_rs256_destroy(self.h)
            self.h = None

    def encode(self, data_ptr, nblocks, message_len, parity_ptr, stream=None):
        call("ffgpu_rs256_encode", self.h, data_ptr, nblocks, message_len, parity_ptr, stream)

    def decode(self, data_ptr, parity_ptr, nblocks, message_len, status_ptr, stream=None):
        call("ffgpu_rs256_decode", self.h, data_ptr, parity_ptr, nblocks, message_len, status_ptr, stream)

    def synds(self, data_ptr, parity_ptr, nblocks, message_len, synds_ptr, stream=None):
        call("ffgpu_rs256_synds", self.h, data_ptr, parity_ptr, nblocks, message_len, synds_ptr, stream)

    def set_table_only(self, on=True):
        """Use the byte-table kernels only (cross-check of the bitsliced ones)."""
        call("ffgpu_rs256_set_table_only", self.h, 1 if on else 0)


class RSi16Code:
    """Device-resident RSi16 code handle (ffgpu_rsi16)."""

    def __init__(self, block_len, ecc_len, primitive=3):
        h = ctypes.c_void_p()
        call("ffgpu_rsi16_create", block_len, ecc_len, primitive, ctypes.byref(h))
        self.h = h
        self.block_len = block_len
        self.ecc_len = ecc_len
        self.message_len = block_len - ecc_len

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ffgpu_rsi16_destroy(self.h)
            self.h = None

    def encode(self, msg_ptr, nblocks, parity_ptr, stream=None):
        call("ffgpu_rsi16_encode", self.h, msg_ptr, nblocks, parity_ptr, stream)

    def repair(self, msg_ptr, parity_ptr, nblocks, status_ptr, stream=None):
        call("ffgpu_rsi16_repair", self.h, msg_ptr, parity_ptr, nblocks, status_ptr, stream)

    def synd(self, msg_ptr, parity_ptr, nblocks, synds_ptr, stream=None):
        """ecc_len uint32 syndromes per block (NTT::pntt over the whole block)."""
        call("ffgpu_rsi16_synd", self.h, msg_ptr, parity_ptr, nblocks, synds_ptr, stream)


class CIRC16Code:
    """Device-resident CIRC16 code handle (ffgpu_circ16)."""

    def __init__(self, ib, ie, ob, oe, interleave=1, primitive=3):
        h = ctypes.c_void_p()
        call("ffgpu_circ16_create", ib, ie, ob, oe, interleave, primitive, ctypes.byref(h))
        self.h = h
        ml, el = _SZ(), _SZ()
        call("ffgpu_circ16_info", h, ctypes.byref(ml), ctypes.byref(el))
        self.message_len, self.ecc_len = ml.value, el.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ffgpu_circ16_destroy(self.h)
            self.h = None

    def encode(self, msg_ptr, nblocks, ecc_ptr, stream=None):
        call("ffgpu_circ16_encode", self.h, msg_ptr, nblocks, ecc_ptr, stream)

    def repair(self, msg_ptr, ecc_ptr, nblocks, status_ptr, stream=None):
        call("ffgpu_circ16_repair", self.h, msg_ptr, ecc_ptr, nblocks, status_ptr, stream)


ENCODE, DECODE = 0, 1


class Batch:
    """Requests of mixed codes served by one persistent launch (ffgpu_batch).

    Buffers are device pointers and must outlive the batch's use."""

    def __init__(self):
        h = ctypes.c_void_p()
        call("ffgpu_batch_create", ctypes.byref(h))
        self.h = h
        self._keep = []

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ffgpu_batch_destroy(self.h)
            self.h = None

    def add_rs256(self, code, op, data_ptr, parity_ptr, nblocks, message_len, status_ptr=None):
        self._keep.append(code)
        call("ffgpu_batch_add_rs256", self.h, code.h, op, data_ptr, parity_ptr, nblocks, message_len, status_ptr)

    def add_rsi16(self, code, op, msg_ptr, parity_ptr, nblocks, status_ptr=None):
        self._keep.append(code)
        call("ffgpu_batch_add_rsi16", self.h, code.h, op, msg_ptr, parity_ptr, nblocks, status_ptr)

    def add_circ16(self, code, msg_ptr, ecc_ptr, nblocks, op=ENCODE, status_ptr=None):
        self._keep.append(code)
        call("ffgpu_batch_add_circ16", self.h, code.h, op, msg_ptr, ecc_ptr, nblocks, status_ptr)

    def plan(self, autotune=False, stream=None):
        call("ffgpu_batch_plan", self.h, 1 if autotune else 0, stream)

    def capture(self, stream=None):
        call("ffgpu_batch_capture", self.h, stream)

    def launch(self, stream=None):
        call("ffgpu_batch_launch", self.h, stream)

    def info(self):
        a, b, c = _I(), _I(), _I()
        n, g = _SZ(), ctypes.c_uint()
        call("ffgpu_batch_info", self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(n),
             ctypes.byref(g))
        return {"tile_rs256": a.value, "tile_rsi16": b.value, "ctas_per_sm": c.value, "items": n.value,
                "grid": g.value}


class Server:
    """Asynchronous serving of host-buffer requests (ffgpu_server)."""

    def __init__(self, hbm_budget=0, slots=4, max_batch=64):
        h = ctypes.c_void_p()
        call("ffgpu_server_create", hbm_budget, slots, max_batch, ctypes.byref(h))
        self.h = h
        self._keep = {}

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.ffgpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _t(self, keep, fn, *args):
        t = ctypes.c_uint64()
        call(fn, self.h, *args, ctypes.byref(t))
        self._keep[t.value] = keep
        return t.value

    def submit_rs256(self, code, op, data_ptr, parity_ptr, nblocks, message_len, status_ptr=None, keep=None):
        return self._t((code, keep), "ffgpu_server_submit_rs256", code.h, op, data_ptr, parity_ptr, nblocks,
                       message_len, status_ptr)

    def submit_rsi16(self, code, op, msg_ptr, parity_ptr, nblocks, status_ptr=None, keep=None):
        return self._t((code, keep), "ffgpu_server_submit_rsi16", code.h, op, msg_ptr, parity_ptr, nblocks,
                       status_ptr)

    def submit_circ16(self, code, msg_ptr, ecc_ptr, nblocks, op=ENCODE, status_ptr=None, keep=None):
        return self._t((code, keep), "ffgpu_server_submit_circ16", code.h, op, msg_ptr, ecc_ptr, nblocks, status_ptr)

    def wait(self, ticket, timeout=-1.0):
        call("ffgpu_server_wait", self.h, ticket, timeout)

    def poll(self, ticket):
        st = _I()
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        call("ffgpu_server_poll", self.h, ticket, ctypes.byref(st), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return {"state": st.value, "submit": a.value, "start": b.value, "done": c.value}

    def release(self, ticket):
        call("ffgpu_server_release", self.h, ticket)
        self._keep.pop(ticket, None)

    def cancel(self, ticket):
        """withdraw a request that is still queued (FFGPUError if admitted)"""
        call("ffgpu_server_cancel", self.h, ticket)


def rsi16_repair_counters(reset=False):
    """(blocks served by the bounded-distance path, blocks served by the mirror)"""
    f, m = ctypes.c_uint64(), ctypes.c_uint64()
    call("ffgpu_rsi16_repair_counters", ctypes.byref(f), ctypes.byref(m), 1 if reset else 0)
    return f.value, m.value


def timing_enable(on=True):
    call("ffgpu_timing_enable", 1 if on else 0)


def timing_collect():
    """{kernel name: (total ms, launches)} of the launches timed since the last call."""
    n = _SZ(0)
    buf = ctypes.create_string_buffer(1 << 16)
    call("ffgpu_timing_collect", buf, 1 << 16, ctypes.byref(n))
    out = {}
    for line in buf.value.decode().splitlines():
        name, ms, cnt = line.rsplit(" ", 2)
        out[name] = (float(ms), int(cnt))
    return out


def kernel_launches():
    return int(lib().ffgpu_kernel_launches())
