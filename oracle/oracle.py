"""ctypes view of the C restatement in ffrs_oracle.c.

TEST INFRASTRUCTURE ONLY: the checker for libffrs_gb300.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
It never runs on the product path.
"""

import ctypes
import os
import platform
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build", platform.machine())
_LIB_PATH = os.path.join(_BUILD, "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile ffrs_oracle.c into oracle/_build/liboracle.so."""
    src = os.path.join(_HERE, "ffrs_oracle.c")
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(_HERE, "ffrs_oracle.h"))
    ):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-o", tmp, src, "-lpthread"])
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = ctypes.CDLL(build())
            _declare(_lib)
        return _lib


_P = ctypes.c_void_p
_SZ = ctypes.c_size_t
_U32 = ctypes.c_uint32
_I = ctypes.c_int


def _declare(L):
    sig = {
        "orc_rs256_new": (_P, [_I, _I, _I]),
        "orc_rs256_free": (None, [_P]),
        "orc_rs256_generator": (None, [_P, _P, _P]),
        "orc_rs256_tables": (None, [_P, _P, _P]),
        "orc_rs256_encode": (None, [_P, _P, _SZ, _P]),
        "orc_rs256_encode_buffer": (_SZ, [_P, _P, _SZ, _SZ, _P, _I]),
        "orc_rs256_synds": (None, [_P, _P, _SZ, _P, _P]),
        "orc_rs256_decode": (_I, [_P, _P, _SZ, _P]),
        "orc_rs256_decode_blocks": (None, [_P, _P, _P, _SZ, _SZ, _P, _I]),
        "orc_rsi16_new": (_P, [_SZ, _SZ, _U32, ctypes.c_char_p, _SZ]),
        "orc_rsi16_free": (None, [_P]),
        "orc_rsi16_ntt_len": (_SZ, [_P]),
        "orc_rsi16_root": (_U32, [_P]),
        "orc_rsi16_rbo": (_U32, [_P, _U32]),
        "orc_rsi16_table": (_P, [_P, _I, ctypes.POINTER(_SZ)]),
        "orc_rsi16_encode_u32": (None, [_P, _P, _P]),
        "orc_rsi16_encode_blocks": (None, [_P, _P, _SZ, _P, _I]),
        "orc_rsi16_encode_interleaved_u32": (None, [_P, _P, _SZ, _P]),
        "orc_rsi16_synd": (None, [_P, _P, _P]),
        "orc_rsi16_temp_len": (_SZ, [_P]),
        "orc_rsi16_repair": (_I, [_P, _P, _P]),
        "orc_rsi16_repair_known": (_I, [_P, _P, _P, _SZ, _P]),
        "orc_rsi16_repair_blocks": (None, [_P, _P, _P, _SZ, _P, _I]),
        "orc_rsi16_repair_interleaved_u32": (_I, [_P, _P, _P, _SZ, _SZ, _SZ, _P, ctypes.c_long]),
        "orc_rsi16_sugiyama": (_I, [_P, _P, _P, _P, _P]),
        "orc_rsi16_pintt_ecc": (None, [_P, _P]),
        "orc_rsi16_mix_ecc": (None, [_P, _P]),
        "orc_circ16_new": (_P, [_SZ, _SZ, _SZ, _SZ, _SZ, _U32, ctypes.c_char_p, _SZ]),
        "orc_circ16_free": (None, [_P]),
        "orc_circ16_message_len": (_SZ, [_P]),
        "orc_circ16_ecc_len": (_SZ, [_P]),
        "orc_circ16_encode": (None, [_P, _P, _P]),
        "orc_circ16_encode_blocks": (None, [_P, _P, _SZ, _P, _I]),
        "orc_circ16_repair": (_I, [_P, _P, _P]),
        "orc_circ16_find_outer_error_locations": (ctypes.c_long, [_P, _P, _P, _SZ, _P, _SZ]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _u8(buf):
    return np.frombuffer(bytes(buf), dtype=np.uint8).copy() if not isinstance(buf, np.ndarray) else buf


class RS256:
    """Oracle for ffrs.RS256 (libffrs/pyrs256.hpp)."""

    def __init__(self, ecc_len, primitive=2, polynomial=0x11D, block_len=255):
        self._h = lib().orc_rs256_new(ecc_len, primitive, polynomial)
        if not self._h:
            raise ValueError("invalid RS256 parameters")
        self.ecc_len = ecc_len
        self.block_len = block_len
        self.message_len = block_len - ecc_len

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_rs256_free(self._h)
            self._h = None

    @property
    def generator(self):
        g = np.zeros(self.ecc_len + 1, np.uint8)
        r = np.zeros(self.ecc_len, np.uint8)
        lib().orc_rs256_generator(self._h, _ptr(g), _ptr(r))
        return bytes(g)

    @property
    def generator_roots(self):
        g = np.zeros(self.ecc_len + 1, np.uint8)
        r = np.zeros(self.ecc_len, np.uint8)
        lib().orc_rs256_generator(self._h, _ptr(g), _ptr(r))
        return bytes(r)

    def encode(self, buf, threads=1):
        a = np.ascontiguousarray(np.frombuffer(bytes(buf), np.uint8))
        n = a.size
        if n == 0:
            return bytearray()
        nb = -(-n // self.message_len)
        out = np.zeros(nb * self.ecc_len, np.uint8)
        lib().orc_rs256_encode_buffer(self._h, _ptr(a), n, self.message_len, _ptr(out), threads)
        return bytearray(out.tobytes())

    def encode_blocks(self, data, threads=1):
        """data: uint8 [nblocks, message_len] -> parity [nblocks, ecc_len]"""
        data = np.ascontiguousarray(data, np.uint8)
        nb, ml = data.shape
        out = np.zeros((nb, self.ecc_len), np.uint8)
        lib().orc_rs256_encode_buffer(self._h, _ptr(data), data.size, ml, _ptr(out), threads)
        return out

    def synds(self, buf):
        a = np.frombuffer(bytes(buf), np.uint8).copy()
        s = np.zeros(max(self.ecc_len, 1), np.uint8)
        lib().orc_rs256_synds(self._h, _ptr(a), self.message_len, _ptr(a[self.message_len :]), _ptr(s))
        return bytes(s[: self.ecc_len])

    def repair(self, buf, ecc):
        """Mirrors RS256.repair: returns bool, mutates buf and ecc in place."""
        d = np.frombuffer(bytes(buf), np.uint8).copy()
        p = np.frombuffer(bytes(ecc), np.uint8).copy()
        ok = lib().orc_rs256_decode(self._h, _ptr(d), self.message_len, _ptr(p))
        buf[: d.size] = d.tobytes()
        ecc[: p.size] = p.tobytes()
        return bool(ok)

    def decode_blocks(self, data, parity, threads=1):
        """In place over uint8 [nb, message_len] / [nb, ecc_len]; returns uint8 status."""
        assert data.flags.c_contiguous and parity.flags.c_contiguous
        nb = data.shape[0]
        st = np.zeros(nb, np.uint8)
        lib().orc_rs256_decode_blocks(self._h, _ptr(data), _ptr(parity), nb, data.shape[1], _ptr(st), threads)
        return st


class RSi16:
    """Oracle for ffrs.RSi16 with W = 1 semantics (libffrs/pyrsi16.hpp)."""

    def __init__(self, block_len, ecc_len, primitive=3):
        err = ctypes.create_string_buffer(256)
        self._h = lib().orc_rsi16_new(block_len, ecc_len, primitive, err, 256)
        if not self._h:
            raise RuntimeError(err.value.decode())
        self.block_len = block_len
        self.ecc_len = ecc_len
        self.message_len = block_len - ecc_len
        self.ntt_len = lib().orc_rsi16_ntt_len(self._h)
        self.root = lib().orc_rsi16_root(self._h)
        self.temp_len = lib().orc_rsi16_temp_len(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_rsi16_free(self._h)
            self._h = None

    def rbo(self, i):
        return lib().orc_rsi16_rbo(self._h, i)

    def table(self, which):
        n = _SZ()
        p = lib().orc_rsi16_table(self._h, which, ctypes.byref(n))
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint32)), shape=(n.value,)).copy()

    def encode_u32(self, msg):
        m = np.ascontiguousarray(msg, np.uint32)
        p = np.zeros(self.ecc_len, np.uint32)
        lib().orc_rsi16_encode_u32(self._h, _ptr(m), _ptr(p))
        return p

    def encode_blocks(self, msg, threads=1):
        """uint16 [nb, message_len] -> uint16 [nb, ecc_len]"""
        m = np.ascontiguousarray(msg, np.uint16)
        nb = m.shape[0]
        out = np.zeros((nb, self.ecc_len), np.uint16)
        lib().orc_rsi16_encode_blocks(self._h, _ptr(m), nb, _ptr(out), threads)
        return out

    def encode_interleaved(self, msg_u32, interleave):
        m = np.ascontiguousarray(msg_u32, np.uint32)
        out = np.zeros(self.ecc_len * interleave, np.uint32)
        lib().orc_rsi16_encode_interleaved_u32(self._h, _ptr(m), interleave, _ptr(out))
        return out

    def synd(self, block_u32):
        b = np.ascontiguousarray(block_u32, np.uint32)
        s = np.zeros(self.ecc_len, np.uint32)
        lib().orc_rsi16_synd(self._h, _ptr(b), _ptr(s))
        return s

    def repair_block(self, block_u32, error_pos=None):
        """One W=1 repair of a uint32 block in place; returns the status (negative = RuntimeError)."""
        b = block_u32
        t = np.zeros(self.temp_len + 1, np.uint32)
        if error_pos is None:
            return lib().orc_rsi16_repair(self._h, _ptr(b), _ptr(t))
        pr = np.array([self.rbo(p) for p in error_pos] + [0], np.uint32)
        return lib().orc_rsi16_repair_known(self._h, _ptr(b), _ptr(pr), len(error_pos), _ptr(t))

    def repair(self, message, ecc, error_pos=None):
        """Mirrors RSi16.repair for interleave == 1 on uint16 numpy arrays (in place)."""
        if error_pos is not None and len(error_pos) == 0:
            return 0
        b = np.concatenate([message.astype(np.uint32), ecc.astype(np.uint32)])
        st = self.repair_block(b, error_pos)
        if st < 0:
            raise RuntimeError("reference assertion")
        message[:] = (b[: self.message_len] & 0xFFFF).astype(np.uint16)
        ecc[:] = (b[self.message_len :] & 0xFFFF).astype(np.uint16)
        return st

    def repair_blocks(self, msg, parity, threads=1):
        assert msg.flags.c_contiguous and parity.flags.c_contiguous
        nb = msg.shape[0]
        st = np.zeros(nb, np.int8)
        lib().orc_rsi16_repair_blocks(self._h, _ptr(msg), _ptr(parity), nb, _ptr(st), threads)
        return st

    def repair_interleaved(self, msg_u32, ecc_u32, interleave, col_start, col_count, error_pos=None):
        pos = np.array(list(error_pos or []) + [0], np.uint32)
        cnt = -1 if error_pos is None else len(error_pos)
        return lib().orc_rsi16_repair_interleaved_u32(
            self._h, _ptr(msg_u32), _ptr(ecc_u32), interleave, col_start, col_count, _ptr(pos), cnt
        )

    def sugiyama(self, synd):
        r1 = np.ascontiguousarray(synd, np.uint32).copy()
        a1 = np.zeros(self.ecc_len, np.uint32)
        t4 = np.zeros(4 * self.ecc_len, np.uint32)
        n = _U32()
        st = lib().orc_rsi16_sugiyama(self._h, _ptr(a1), _ptr(r1), _ptr(t4), ctypes.byref(n))
        if st < 0:
            raise RuntimeError("reference assertion")
        return a1, r1, n.value

    def roots(self, poly):
        t = np.zeros(self.ntt_len, np.uint32)
        t[: self.ecc_len] = poly
        lib().orc_rsi16_pintt_ecc(self._h, _ptr(t))
        return [i for i in range(self.block_len) if t[i] == 0]

    def mix_ecc(self, ecc):
        e = np.ascontiguousarray(ecc, np.uint32).copy()
        lib().orc_rsi16_mix_ecc(self._h, _ptr(e))
        return e


class CIRC16:
    """Oracle for ffrs.CIRC16 with W = 1 semantics (libffrs/pycirc16.hpp)."""

    def __init__(self, inner_block_len, inner_ecc_len, outer_block_len, outer_ecc_len, interleave=1, primitive=3):
        err = ctypes.create_string_buffer(256)
        self._h = lib().orc_circ16_new(
            inner_block_len, inner_ecc_len, outer_block_len, outer_ecc_len, interleave, primitive, err, 256
        )
        if not self._h:
            raise RuntimeError(err.value.decode())
        self.message_len = lib().orc_circ16_message_len(self._h)
        self.ecc_len = lib().orc_circ16_ecc_len(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_circ16_free(self._h)
            self._h = None

    def encode(self, msg_u16, threads=1):
        m = np.ascontiguousarray(msg_u16, np.uint16)
        assert m.size % self.message_len == 0
        nb = m.size // self.message_len
        out = np.zeros(nb * self.ecc_len, np.uint16)
        lib().orc_circ16_encode_blocks(self._h, _ptr(m), nb, _ptr(out), threads)
        return out

    def repair(self, msg_u16, ecc_u16):
        """In place on uint16 arrays; returns 0 or a negative RuntimeError code."""
        assert msg_u16.size == self.message_len and ecc_u16.size == self.ecc_len
        return lib().orc_circ16_repair(self._h, _ptr(msg_u16), _ptr(ecc_u16))

    def find_outer_error_locations(self, msg_u16, ecc_u16, k):
        out = np.zeros(1 << 17, np.uintp)
        n = lib().orc_circ16_find_outer_error_locations(self._h, _ptr(msg_u16), _ptr(ecc_u16), k, _ptr(out), out.size)
        return [int(x) for x in out[:n]]
