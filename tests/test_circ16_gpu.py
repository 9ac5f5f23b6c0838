"""CIRC16 on the GPU against the reference's golden outputs and the oracle."""

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gold():
    return load_golden("circ16.npz")


def test_circ16_golden_api(ffrs_gpu, gold):
    for g in range(int(gold["ngeoms"][0])):
        p = f"g{g}_"
        geom = tuple(int(x) for x in gold[p + "geom"])
        c = ffrs_gpu.CIRC16(*geom)
        assert bytes(c.encode(gold[p + "msg"].tobytes())) == gold[p + "ecc"].tobytes(), geom
        for t in range(gold[p + "recv_msg"].shape[0]):
            m = bytearray(gold[p + "recv_msg"][t].tobytes())
            e = bytearray(gold[p + "recv_ecc"][t].tobytes())
            if int(gold[p + "rc"][t]) < 0:
                with pytest.raises(RuntimeError):
                    c.repair(m, e)
                continue
            assert c.repair(m, e) is False
            assert bytes(m) == gold[p + "rep_msg"][t].tobytes(), (geom, t)
            assert bytes(e) == gold[p + "rep_ecc"][t].tobytes(), (geom, t)


def test_circ16_properties(ffrs_gpu):
    rs = ffrs_gpu.CIRC16(128, 8, 128, 8, 4)
    assert rs.ecc_len == rs.inner_block_len * rs.outer_block_len * rs.interleave - rs.message_len
    assert rs.block_len == rs.message_len + rs.ecc_len
    assert rs.outer_interleave == rs.inner_message_len * rs.interleave
    assert rs.rso.interleave == rs.outer_interleave and rs.rsi.interleave == 1


@pytest.mark.parametrize("geom", [(16, 4, 16, 4, 1), (64, 4, 32, 8, 4), (52, 2, 192, 64, 3)])
def test_circ16_vs_oracle_random(ffrs_gpu, geom):
    rng = np.random.Generator(np.random.PCG64(sum(geom)))
    c = ffrs_gpu.CIRC16(*geom)
    o = O.CIRC16(*geom)
    for trial in range(4):
        msg = rng.integers(0, 65536, size=c.message_len, dtype=np.uint16)
        ecc = np.frombuffer(bytes(c.encode(msg.tobytes())), np.uint16).copy()
        np.testing.assert_array_equal(ecc, o.encode(msg))
        m, e = msg.copy(), ecc.copy()
        nrows = int(rng.integers(1, c.outer_ecc_len + 3))
        for row in rng.choice(c.outer_block_len, size=min(nrows, c.outer_block_len), replace=False):
            k = int(rng.integers(0, c.interleave))
            if row < c.outer_message_len:
                for col in range(c.inner_message_len):
                    m[c.message_offset(k, int(row), col)] ^= int(rng.integers(1, 65536))
            else:
                for col in range(c.inner_message_len):
                    e[c.rso_ecc_offset(k, int(row) - c.outer_message_len, col)] ^= int(rng.integers(1, 65536))
        if trial % 2:
            e[rng.choice(e.size, size=min(20, e.size), replace=False)] = 0
            m[rng.choice(m.size, size=5, replace=False)] = 0
        for k in range(c.interleave):
            assert c._find_outer_error_locations(m.tobytes(), e.tobytes(), k) == o.find_outer_error_locations(
                m.copy(), e.copy(), k
            )
        mo, eo = m.copy(), e.copy()
        rc = o.repair(mo, eo)
        mb, eb = bytearray(m.tobytes()), bytearray(e.tobytes())
        if rc < 0:
            with pytest.raises(RuntimeError):
                c.repair(mb, eb)
            continue
        c.repair(mb, eb)
        np.testing.assert_array_equal(np.frombuffer(bytes(mb), np.uint16), mo)
        np.testing.assert_array_equal(np.frombuffer(bytes(eb), np.uint16), eo)


@pytest.mark.parametrize("geom", [(16, 4, 16, 4, 1), (64, 4, 32, 8, 4)])
def test_circ16_repair_blocks_vs_oracle(ffrs_gpu, geom):
    """Several codewords in one call (one fused launch): every codeword's
    message equals the oracle's, its ecc too where the reference returns, and
    its status is 255 exactly where the reference raises."""
    rng = np.random.Generator(np.random.PCG64(7 * sum(geom)))
    c = ffrs_gpu.CIRC16(*geom)
    o = O.CIRC16(*geom)
    nb = 12
    ms, es, want_m, want_e, rcs = [], [], [], [], []
    for i in range(nb):
        msg = rng.integers(0, 65536, size=c.message_len, dtype=np.uint16)
        ecc = np.frombuffer(bytes(c.encode(msg.tobytes())), np.uint16).copy()
        m, e = msg.copy(), ecc.copy()
        nrows = int(rng.integers(0, c.outer_ecc_len + 4))
        for row in rng.choice(c.outer_block_len, size=min(nrows, c.outer_block_len), replace=False):
            k = int(rng.integers(0, c.interleave))
            if row < c.outer_message_len:
                for col in range(c.inner_message_len):
                    m[c.message_offset(k, int(row), col)] ^= int(rng.integers(1, 65536))
            else:
                for col in range(c.inner_message_len):
                    e[c.rso_ecc_offset(k, int(row) - c.outer_message_len, col)] ^= int(rng.integers(1, 65536))
        if i % 3 == 2:
            e[rng.choice(e.size, size=min(20, e.size), replace=False)] = 0
        mo, eo = m.copy(), e.copy()
        rcs.append(o.repair(mo, eo))
        ms.append(m)
        es.append(e)
        want_m.append(mo)
        want_e.append(eo)
    mb = bytearray(np.concatenate(ms).tobytes())
    eb = bytearray(np.concatenate(es).tobytes())
    st = np.frombuffer(bytes(c.repair_blocks(mb, eb)), np.uint8)
    got_m = np.frombuffer(bytes(mb), np.uint16).reshape(nb, c.message_len)
    got_e = np.frombuffer(bytes(eb), np.uint16).reshape(nb, c.ecc_len)
    for i in range(nb):
        assert st[i] == (255 if rcs[i] < 0 else 0), i
        np.testing.assert_array_equal(got_m[i], want_m[i])
        if rcs[i] >= 0:
            np.testing.assert_array_equal(got_e[i], want_e[i])
        else:
            np.testing.assert_array_equal(got_e[i], es[i])  # a raising codeword keeps its ecc


def test_circ16_repair_blocks_golden(ffrs_gpu, gold):
    """The reference's golden codewords of every geometry repaired in one
    multi-codeword call: statuses, messages and ecc as the reference's.  (A
    raising codeword, which none of the fixtures holds, must come back with
    status 255, the message as the pinned oracle leaves it and its ecc
    untouched.)"""
    for g in range(int(gold["ngeoms"][0])):
        p = f"g{g}_"
        geom = tuple(int(x) for x in gold[p + "geom"])
        c = ffrs_gpu.CIRC16(*geom)
        o = O.CIRC16(*geom)
        rm, re_ = gold[p + "recv_msg"], gold[p + "recv_ecc"]
        nt = rm.shape[0]
        if nt < 2:
            continue
        mb, eb = bytearray(rm.tobytes()), bytearray(re_.tobytes())
        st = np.frombuffer(bytes(c.repair_blocks(mb, eb)), np.uint8)
        got_m = np.frombuffer(bytes(mb), np.uint16).reshape(rm.shape)
        got_e = np.frombuffer(bytes(eb), np.uint16).reshape(re_.shape)
        for t in range(nt):
            if int(gold[p + "rc"][t]) < 0:
                assert st[t] == 255, (geom, t)
                mo, eo = rm[t].copy(), re_[t].copy()
                assert o.repair(mo, eo) < 0
                np.testing.assert_array_equal(got_m[t], mo)
                np.testing.assert_array_equal(got_e[t], re_[t])
            else:
                assert st[t] == 0, (geom, t)
                np.testing.assert_array_equal(got_m[t], gold[p + "rep_msg"][t])
                np.testing.assert_array_equal(got_e[t], gold[p + "rep_ecc"][t])
