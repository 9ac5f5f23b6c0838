"""RSi16 on the GPU against the reference's golden outputs and the oracle."""

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gold():
    return load_golden("rsi16.npz")


def test_rsi16_golden_api(ffrs_gpu, gold):
    for g in range(int(gold["ngeoms"][0])):
        p = f"g{g}_"
        bl, ecc, root, ntt_len = map(int, gold[p + "geom"])
        rs = ffrs_gpu.RSi16(bl, ecc)
        assert (rs.root, rs.ntt_len) == (root, ntt_len)
        assert bytes(rs.encode(gold[p + "msgs"].tobytes())) == gold[p + "parity"].tobytes(), (bl, ecc)
        recv = gold[p + "received"]
        ml = bl - ecc
        for i in range(recv.shape[0]):
            m = bytearray(recv[i, :ml].tobytes())
            e = bytearray(recv[i, ml:].tobytes())
            assert rs._synd(m, e) == list(map(int, gold[p + "synd"][i]))
            if gold[p + "locator"][i][0] != 0xFFFFFFFF:
                loc, ev = rs._sugiyama(list(map(int, gold[p + "synd"][i])))
                assert loc == list(map(int, gold[p + "locator"][i])), (bl, ecc, i)
                assert ev == list(map(int, gold[p + "evaluator"][i])), (bl, ecc, i)
            want = int(gold[p + "status"][i])
            if want < 0:
                with pytest.raises(RuntimeError):
                    rs.repair(m, e)
                continue
            assert int(rs.repair(m, e)) == want, (bl, ecc, i)
            assert bytes(m) == gold[p + "repaired_data"][i].tobytes(), (bl, ecc, i)
            assert bytes(e) == gold[p + "repaired_parity"][i].tobytes(), (bl, ecc, i)
        krecv = gold[p + "known_received"]
        for i in range(krecv.shape[0]):
            pos = [int(x) for x in gold[p + "known_pos"][i] if x >= 0]
            m = bytearray(krecv[i, :ml].tobytes())
            e = bytearray(krecv[i, ml:].tobytes())
            assert int(rs.repair(m, e, pos)) == int(gold[p + "known_status"][i]), (bl, ecc, i)
            assert bytes(m) == gold[p + "known_data"][i].tobytes(), (bl, ecc, i)
            assert bytes(e) == gold[p + "known_parity"][i].tobytes(), (bl, ecc, i)


def _corrupt_words(rng, cw, k):
    pos = rng.choice(cw.size, size=k, replace=False)
    for q in pos:
        while True:
            d = int(rng.integers(1, 65537))
            v = (int(cw[q]) + d) % 65537
            if v != 65536:
                break
        cw[q] = v


@pytest.mark.parametrize("bl,ecc", [(1024, 64), (256, 32), (96, 16), (4096, 128), (128, 64), (512, 2), (128, 8),
                                    (60, 4), (130, 2), (48, 16)])
def test_rsi16_batched_vs_oracle(ffrs_gpu, bl, ecc):
    rng = np.random.Generator(np.random.PCG64(bl * 7 + ecc))
    rs = ffrs_gpu.RSi16(bl, ecc)
    o = O.RSi16(bl, ecc)
    nb = 600 if bl <= 1024 else 120
    ml = bl - ecc
    msg = rng.integers(0, 65536, size=(nb, ml), dtype=np.uint16)
    par = np.frombuffer(bytes(rs.encode(msg.tobytes())), np.uint16).reshape(nb, ecc).copy()
    np.testing.assert_array_equal(par, o.encode_blocks(msg, threads=8))
    cw = np.concatenate([msg, par], axis=1)
    for i in range(nb):
        _corrupt_words(rng, cw[i], int(rng.integers(0, ecc // 2 + 3)))
    m = np.ascontiguousarray(cw[:, :ml])
    e = np.ascontiguousarray(cw[:, ml:])
    mb, eb = bytearray(m.tobytes()), bytearray(e.tobytes())
    st = np.frombuffer(bytes(rs.repair_blocks(mb, eb)), np.uint8)
    mo, eo = m.copy(), e.copy()
    so = o.repair_blocks(mo, eo, threads=8)
    np.testing.assert_array_equal(st.astype(np.int16), np.where(so < 0, 255, so.astype(np.int16)))
    np.testing.assert_array_equal(np.frombuffer(bytes(mb), np.uint16).reshape(nb, ml), mo)
    np.testing.assert_array_equal(np.frombuffer(bytes(eb), np.uint16).reshape(nb, ecc), eo)


def test_rsi16_bounded_distance_path(ffrs_gpu):
    """Blocks with at most ecc/2 errors are all served by the Berlekamp-Massey
    path; blocks beyond it fall back to the mirror; both agree with the oracle."""
    from libffrs_gb300 import capi

    bl, ecc = 1024, 64
    rng = np.random.Generator(np.random.PCG64(99))
    rs = ffrs_gpu.RSi16(bl, ecc)
    o = O.RSi16(bl, ecc)
    ml = bl - ecc
    for lo, hi, want_mirror in ((1, ecc // 2 + 1, False), (ecc // 2 + 8, ecc // 2 + 12, True)):
        nb = 200
        msg = rng.integers(0, 65536, size=(nb, ml), dtype=np.uint16)
        par = o.encode_blocks(msg, threads=8)
        cw = np.concatenate([msg, par], axis=1)
        for i in range(nb):
            _corrupt_words(rng, cw[i], int(rng.integers(lo, hi)))
        m, e = np.ascontiguousarray(cw[:, :ml]), np.ascontiguousarray(cw[:, ml:])
        mb, eb = bytearray(m.tobytes()), bytearray(e.tobytes())
        capi.rsi16_repair_counters(reset=True)
        st = np.frombuffer(bytes(rs.repair_blocks(mb, eb)), np.uint8)
        fast, mirror = capi.rsi16_repair_counters()
        assert fast + mirror == nb
        if want_mirror:
            assert mirror > 0
        else:
            assert mirror == 0 and (st == 2).all()
        mo, eo = m.copy(), e.copy()
        so = o.repair_blocks(mo, eo, threads=8)
        np.testing.assert_array_equal(st.astype(np.int16), np.where(so < 0, 255, so.astype(np.int16)))
        np.testing.assert_array_equal(np.frombuffer(bytes(mb), np.uint16).reshape(nb, ml), mo)
        np.testing.assert_array_equal(np.frombuffer(bytes(eb), np.uint16).reshape(nb, ecc), eo)


@pytest.mark.parametrize("interleave", [2, 3, 16, 33])
def test_rsi16_interleaved_vs_oracle(ffrs_gpu, interleave):
    bl, ecc = 256, 32
    rng = np.random.Generator(np.random.PCG64(interleave))
    rs = ffrs_gpu.RSi16(bl, ecc, interleave=interleave)
    o = O.RSi16(bl, ecc)
    ml = bl - ecc
    msg = rng.integers(0, 65536, size=ml * interleave, dtype=np.uint16)
    par = np.frombuffer(bytes(rs.encode(msg.tobytes())), np.uint16).copy()
    want = o.encode_interleaved(msg.astype(np.uint32), interleave).astype(np.uint16)
    np.testing.assert_array_equal(par, want)
    for known in (False, True):
        m, e = msg.copy(), par.copy()
        rows = sorted(rng.choice(bl, size=ecc // 2 - 1 if not known else ecc - 2, replace=False).tolist())
        for r in rows:
            for col in range(interleave):
                if r < ml:
                    m[r * interleave + col] ^= int(rng.integers(1, 65536))
                else:
                    e[(r - ml) * interleave + col] ^= int(rng.integers(1, 65536))
        mo, eo = m.astype(np.uint32), e.astype(np.uint32)
        so = o.repair_interleaved(mo, eo, interleave, 0, interleave, rows if known else None)
        mb, eb = bytearray(m.tobytes()), bytearray(e.tobytes())
        s = rs.repair(mb, eb, rows) if known else rs.repair(mb, eb)
        assert int(s) == so
        np.testing.assert_array_equal(np.frombuffer(bytes(mb), np.uint16), (mo & 0xFFFF).astype(np.uint16))
        np.testing.assert_array_equal(np.frombuffer(bytes(eb), np.uint16), (eo & 0xFFFF).astype(np.uint16))


def test_rsi16_errors(ffrs_gpu):
    with pytest.raises(RuntimeError):
        ffrs_gpu.RSi16(100, 3)
    with pytest.raises(RuntimeError):
        ffrs_gpu.RSi16(100, 8)
    rs = ffrs_gpu.RSi16(16, 4)
    assert bytes(rs.encode(b"")) == b""
    with pytest.raises(RuntimeError):
        rs.encode(bytearray(6))
    m, e = bytearray(24), bytearray(8)
    assert rs.repair(m, e, []) == ffrs_gpu.RepairStatus.NoErrors
    assert rs.repair(m, e) == ffrs_gpu.RepairStatus.NoErrors


@pytest.mark.parametrize("bl,ecc", [(130, 2), (60, 4), (128, 8), (96, 16), (256, 32), (1024, 64), (4096, 128),
                                    (2048, 256)])
def test_rsi16_synd_blocks_vs_oracle(bl, ecc):
    """Batched syndromes (every ecc: the sub-warp, register and shared-memory
    transforms) against the oracle's NTT::pntt, block by block."""
    import torch

    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(bl + 31 * ecc))
    nb = 333
    ml = bl - ecc
    o = O.RSi16(bl, ecc)
    msg = rng.integers(0, 65536, size=(nb, ml), dtype=np.uint16)
    par = rng.integers(0, 65536, size=(nb, ecc), dtype=np.uint16)
    code = capi.RSi16Code(bl, ecc)
    dm = torch.from_numpy(msg.view(np.int16)).cuda()
    dp = torch.from_numpy(par.view(np.int16)).cuda()
    ds = torch.zeros((nb, ecc), dtype=torch.int32, device="cuda")
    code.synd(dm.data_ptr(), dp.data_ptr(), nb, ds.data_ptr(), torch.cuda.current_stream().cuda_stream)
    got = ds.cpu().numpy().view(np.uint32)
    for i in range(nb):
        blk = np.concatenate([msg[i], par[i]]).astype(np.uint32)
        np.testing.assert_array_equal(got[i], o.synd(blk), err_msg=f"block {i}")
