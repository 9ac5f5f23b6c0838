"""Expected outputs of the serving and batch requests that bench.py builds,
computed by the oracle from each request's pristine inputs (test helper)."""

import numpy as np

from oracle import oracle as O

_codes = {}


def _code(kind, *key):
    k = (kind,) + key
    if k not in _codes:
        _codes[k] = {"rs256": O.RS256, "rsi16": O.RSi16, "circ16": O.CIRC16}[kind](*key)
    return _codes[k]


def serving(r, threads=8):
    """(a, b, status or None) for one request of bench.make_serving_requests"""
    a0, b0 = r["a0"], r["b0"]
    nb, dec = r["nb"], r["op"] == "dec"
    if r["kind"] in ("rs8", "rs32"):
        ecc, ml = r["ecc"], r["ml"]
        o = _code("rs256", ecc, 2, 0x11D, ml + ecc)
        d = a0.reshape(nb, ml).copy()
        if not dec:
            return a0.copy(), o.encode_blocks(d, threads=threads).reshape(-1), None
        p = b0.reshape(nb, ecc).copy()
        st = o.decode_blocks(d, p, threads=threads)
        return d.reshape(-1), p.reshape(-1), st
    if r["kind"] == "rsi":
        o = _code("rsi16", 1024, 64)
        m = a0.reshape(nb, 960).copy()
        if not dec:
            return a0.copy(), o.encode_blocks(m, threads=threads).reshape(-1), None
        p = b0.reshape(nb, 64).copy()
        st = o.repair_blocks(m, p, threads=threads)
        return m.reshape(-1), p.reshape(-1), np.where(st < 0, 255, st).astype(np.uint8)
    c = r["code"]
    o = _code("circ16", 128, 8, 128, 8, 4)
    ml, el = c.message_len, c.ecc_len
    if not dec:
        return a0.copy(), o.encode(a0, threads=threads), None
    m = a0.reshape(nb, ml).copy()
    e = b0.reshape(nb, el).copy()
    st = np.zeros(nb, np.uint8)
    for i in range(nb):
        mi, ei = m[i].copy(), e[i].copy()
        rc = o.repair(mi, ei)
        m[i] = mi
        if rc < 0:
            st[i] = 255  # a raising codeword keeps its ecc
        else:
            e[i] = ei
    return m.reshape(-1), e.reshape(-1), st
