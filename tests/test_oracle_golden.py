"""The CPU oracle (oracle/ffrs_oracle.c) reproduces the reference's own outputs
stored in tests/golden/ (made by tests/golden/make_golden.py from the reference
extension).  Runs without a GPU."""

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O


@pytest.fixture(scope="module")
def rs():
    return load_golden("rs256.npz")


@pytest.fixture(scope="module")
def ri():
    return load_golden("rsi16.npz")


@pytest.fixture(scope="module")
def ci():
    return load_golden("circ16.npz")


def test_rs256_golden(rs):
    for c in range(int(rs["ncases"][0])):
        p = f"c{c}_"
        ecc, bl = map(int, rs[p + "geom"])
        o = O.RS256(ecc, block_len=bl)
        assert o.generator == bytes(rs[p + "generator"])
        assert bytes(o.encode(rs[p + "buffer"].tobytes())) == rs[p + "encoded"].tobytes()
        data = rs[p + "received_data"].copy()
        par = rs[p + "received_parity"].copy()
        for i in range(data.shape[0]):
            assert o.synds(data[i].tobytes() + par[i].tobytes()) == rs[p + "synds"][i].tobytes()
        st = o.decode_blocks(data, par)
        np.testing.assert_array_equal(st, rs[p + "status"], err_msg=f"ecc={ecc} bl={bl}")
        np.testing.assert_array_equal(data, rs[p + "repaired_data"])
        np.testing.assert_array_equal(par, rs[p + "repaired_parity"])


def test_rsi16_golden(ri):
    for g in range(int(ri["ngeoms"][0])):
        p = f"g{g}_"
        bl, ecc, root, ntt_len = map(int, ri[p + "geom"])
        o = O.RSi16(bl, ecc)
        assert (o.root, o.ntt_len) == (root, ntt_len)
        np.testing.assert_array_equal(o.encode_blocks(ri[p + "msgs"]), ri[p + "parity"])
        recv = ri[p + "received"]
        ml = bl - ecc
        for i in range(recv.shape[0]):
            blk = recv[i].astype(np.uint32)
            np.testing.assert_array_equal(o.synd(blk), ri[p + "synd"][i])
            if ri[p + "locator"][i][0] != 0xFFFFFFFF or ecc == 1:
                a1, r1, _ = o.sugiyama(ri[p + "synd"][i])
                np.testing.assert_array_equal(a1, ri[p + "locator"][i])
                np.testing.assert_array_equal(r1, ri[p + "evaluator"][i])
            m, e = recv[i, :ml].copy(), recv[i, ml:].copy()
            want = int(ri[p + "status"][i])
            if want < 0:
                with pytest.raises(RuntimeError):
                    o.repair(m, e)
                continue
            assert o.repair(m, e) == want
            np.testing.assert_array_equal(m, ri[p + "repaired_data"][i])
            np.testing.assert_array_equal(e, ri[p + "repaired_parity"][i])
        krecv = ri[p + "known_received"]
        for i in range(krecv.shape[0]):
            pos = [int(x) for x in ri[p + "known_pos"][i] if x >= 0]
            m, e = krecv[i, :ml].copy(), krecv[i, ml:].copy()
            assert o.repair(m, e, pos) == int(ri[p + "known_status"][i])
            np.testing.assert_array_equal(m, ri[p + "known_data"][i])
            np.testing.assert_array_equal(e, ri[p + "known_parity"][i])


def test_circ16_golden(ci):
    for g in range(int(ci["ngeoms"][0])):
        p = f"g{g}_"
        geom = tuple(int(x) for x in ci[p + "geom"])
        o = O.CIRC16(*geom)
        np.testing.assert_array_equal(o.encode(ci[p + "msg"]), ci[p + "ecc"])
        for t in range(ci[p + "recv_msg"].shape[0]):
            m = ci[p + "recv_msg"][t].copy()
            e = ci[p + "recv_ecc"][t].copy()
            rc = o.repair(m, e)
            assert rc == int(ci[p + "rc"][t])
            if rc == 0:
                np.testing.assert_array_equal(m, ci[p + "rep_msg"][t])
                np.testing.assert_array_equal(e, ci[p + "rep_ecc"][t])


def test_oracle_threads_agree():
    """The multi-threaded batch drivers give the same bytes as one thread."""
    rng = np.random.Generator(np.random.PCG64(7))
    o = O.RS256(32)
    data = rng.integers(0, 256, size=(500, 223), dtype=np.uint8)
    par = o.encode_blocks(data, threads=1)
    np.testing.assert_array_equal(par, o.encode_blocks(data, threads=4))
    d1, p1 = data.copy(), par.copy()
    d1[:, :5] ^= 1
    d2, p2 = d1.copy(), p1.copy()
    s1 = o.decode_blocks(d1, p1, threads=1)
    s2 = o.decode_blocks(d2, p2, threads=3)
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(d1, data)
    np.testing.assert_array_equal(d2, data)
