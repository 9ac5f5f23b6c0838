"""The reference's own pure-Python package ``ffrs`` -- unmodified, imported from
a reference checkout -- running on top of this module: ``ffrs/__init__.py``
does ``from libffrs import *`` and subclasses RSi16 and CIRC16, and the
``ffrs.par`` CLI calls ``ffrs.CIRC16(...)``, ``serialize`` / ``deserialize``,
``create_buffer``, ``encode``, ``repair`` and ``set_logger``.  Every result is
compared with the oracle.

The checkout is found through $FFRS_REFERENCE, else a "reference" directory
beside the repository; the test is skipped where neither holds ffrs/."""

import logging
import os
import sys

import numpy as np
import pytest

from conftest import REPO
from oracle import oracle as O

REF = os.environ.get("FFRS_REFERENCE") or os.path.join(os.path.dirname(REPO), "reference")

pytestmark = [
    pytest.mark.gpu,
    pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "ffrs", "__init__.py")),
                       reason="no reference checkout with the ffrs package"),
]


@pytest.fixture(scope="module")
def ffrs(built):
    import libffrs_gb300  # registers this module as the top-level ``libffrs``

    sys.path.insert(0, os.path.abspath(REF))
    try:
        import ffrs as pkg
    finally:
        sys.path.pop(0)
    assert pkg.libffrs is libffrs_gb300.libffrs
    return pkg


def test_package_classes_subclass_this_module(ffrs):
    import libffrs_gb300

    assert issubclass(ffrs.RSi16, libffrs_gb300.libffrs.RSi16)
    assert issubclass(ffrs.CIRC16, libffrs_gb300.libffrs.CIRC16)
    assert ffrs.RS256 is libffrs_gb300.libffrs.RS256
    assert repr(ffrs.RSi16(1024, 64)) == "RSi16(block_len=1024, ecc_len=64)"
    assert repr(ffrs.RSi16(256, 32, interleave=3)) == "RSi16(block_len=256, ecc_len=32, interleave=3)"
    ffrs.set_logger(logging.getLogger("ffrs-dropin"))


def test_circ16_serialize_encode_repair(ffrs):
    c = ffrs.CIRC16(128, 8, 128, 8, 4)
    assert repr(c) == "CIRC(128, 8, 128, 8, 4)"
    s = c.serialize()
    c2 = ffrs.CIRC16.deserialize(s)
    assert c2.serialize() == s and repr(c2) == repr(c)
    oc = O.CIRC16(128, 8, 128, 8, 4)
    rng = np.random.Generator(np.random.PCG64(31))
    buf = ffrs.create_buffer(c.message_len * 2)
    msg = np.frombuffer(buf, np.uint16)
    msg[:] = rng.integers(0, 65536, c.message_len, dtype=np.uint16)
    ecc = bytearray(c.encode(buf))
    want = oc.encode(msg.copy())
    np.testing.assert_array_equal(np.frombuffer(bytes(ecc), np.uint16), want)
    # a burst of changed message words, repaired in place by the package's object
    msg[100:140] += 1
    mo, eo = msg.copy(), want.copy()
    oc.repair(mo, eo)
    assert c.repair(buf, ecc) is False  # CircRepair always returns False
    np.testing.assert_array_equal(msg, mo)
    np.testing.assert_array_equal(np.frombuffer(bytes(ecc), np.uint16), eo)


def test_rs256_and_rsi16_through_the_package(ffrs):
    rng = np.random.Generator(np.random.PCG64(32))
    rs = ffrs.RS256(ecc_len=32)
    data = rng.integers(0, 256, 223, dtype=np.uint8)
    par = bytearray(rs.encode(data.tobytes()))
    assert bytes(par) == bytes(O.RS256(32).encode(data.tobytes()))
    d = bytearray(data.tobytes())
    d[5] ^= 0x11
    d[200] ^= 0x80
    assert rs.repair(d, par) is True and bytes(d) == data.tobytes()
    ri = ffrs.RSi16(1024, 64)
    msg = rng.integers(0, 65536, 960, dtype=np.uint16)
    e = bytearray(ri.encode(msg.tobytes()))
    np.testing.assert_array_equal(np.frombuffer(bytes(e), np.uint16), O.RSi16(1024, 64).encode_blocks(msg[None])[0])
    m = bytearray(msg.tobytes())
    m[10] ^= 0x5A
    assert int(ri.repair(m, e)) == int(ffrs.RepairStatus.RepairOk) and bytes(m) == msg.tobytes()
