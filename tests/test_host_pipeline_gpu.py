"""The host-buffer entry points split a call into chunks of blocks over
several streams (copy in, code, copy out of different chunks overlap).  With
small chunks forced, ragged last chunks and tails, and both pageable and
page-locked outputs, their results still equal the oracle's."""

import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture
def chunk(built):
    from libffrs_gb300 import capi

    yield lambda n: capi.call("ffgpu_set_host_chunk_blocks", n)
    capi.call("ffgpu_set_host_chunk_blocks", 0)


def _flip(rng, cw, k):
    for q in rng.choice(cw.shape[0], size=k, replace=False):
        cw[q] ^= rng.integers(1, 256, dtype=np.uint8)


@pytest.mark.parametrize("forced", [0, 97, 1000])
def test_rs256_host_chunks(ffrs_gpu, chunk, forced):
    chunk(forced)
    rng = np.random.Generator(np.random.PCG64(500 + forced))
    ecc, ml, nb = 32, 223, 2500
    o = O.RS256(ecc, block_len=ml + ecc)
    rs = ffrs_gpu.RS256(ecc_len=ecc)
    # encode of full blocks and a ragged tail, output into a new (pageable) buffer
    buf = rng.integers(0, 256, size=nb * ml + 77, dtype=np.uint8)
    got = np.frombuffer(bytes(rs.encode(buf.tobytes())), np.uint8)
    want = np.concatenate([o.encode_blocks(buf[:nb * ml].reshape(nb, ml), threads=8).ravel(),
                           O.RS256(ecc, block_len=77 + ecc).encode_blocks(buf[nb * ml:].reshape(1, 77)).ravel()])
    np.testing.assert_array_equal(got, want)
    # repair of corrupted blocks: pageable (bytearray) and page-locked buffers
    data = buf[:nb * ml].reshape(nb, ml).copy()
    par = o.encode_blocks(data, threads=8)
    cw = np.concatenate([data, par], axis=1)
    for i in range(nb):
        _flip(rng, cw[i], int(rng.integers(0, ecc // 2 + 3)))
    d0, p0 = np.ascontiguousarray(cw[:, :ml]), np.ascontiguousarray(cw[:, ml:])
    dw, pw = d0.copy(), p0.copy()
    sw = o.decode_blocks(dw, pw, threads=8)
    db, pb = bytearray(d0.tobytes()), bytearray(p0.tobytes())
    st = np.frombuffer(bytes(rs.repair_blocks(db, pb)), np.uint8)
    np.testing.assert_array_equal(st, sw)
    assert bytes(db) == dw.tobytes() and bytes(pb) == pw.tobytes()
    hd, hp = ffrs_gpu.create_buffer(nb * ml), ffrs_gpu.create_buffer(nb * ecc)
    hd[:] = d0.tobytes()
    hp[:] = p0.tobytes()
    st = np.frombuffer(bytes(rs.repair_blocks(hd, hp)), np.uint8)
    np.testing.assert_array_equal(st, sw)
    assert bytes(hd) == dw.tobytes() and bytes(hp) == pw.tobytes()


@pytest.mark.parametrize("forced", [0, 61, 700])
def test_rs256_host_decode_pinned_status(built, chunk, forced):
    """C-ABI host decode with every buffer page-locked (no staging copy)."""
    import torch

    from libffrs_gb300 import capi

    chunk(forced)
    rng = np.random.Generator(np.random.PCG64(900 + forced))
    ecc, ml, nb = 16, 180, 1500
    o = O.RS256(ecc, block_len=ml + ecc)
    data = rng.integers(0, 256, size=(nb, ml), dtype=np.uint8)
    cw = np.concatenate([data, o.encode_blocks(data, threads=8)], axis=1)
    for i in range(nb):
        _flip(rng, cw[i], int(rng.integers(0, ecc // 2 + 3)))
    d0, p0 = np.ascontiguousarray(cw[:, :ml]), np.ascontiguousarray(cw[:, ml:])
    hd = torch.from_numpy(d0.copy()).pin_memory()
    hp = torch.from_numpy(p0.copy()).pin_memory()
    hs = torch.zeros(nb, dtype=torch.uint8).pin_memory()
    code = capi.RS256Code(ecc)
    capi.call("ffgpu_rs256_decode_host", code.h, ctypes.c_void_p(hd.data_ptr()), ctypes.c_void_p(hp.data_ptr()),
              nb, ml, ctypes.c_void_p(hs.data_ptr()))
    dw, pw = d0.copy(), p0.copy()
    sw = o.decode_blocks(dw, pw, threads=8)
    np.testing.assert_array_equal(hs.numpy(), sw)
    np.testing.assert_array_equal(hd.numpy(), dw)
    np.testing.assert_array_equal(hp.numpy(), pw)


@pytest.mark.parametrize("forced", [0, 53, 400])
@pytest.mark.parametrize("bl,ecc", [(1024, 64), (256, 16)])
def test_rsi16_host_chunks(ffrs_gpu, chunk, forced, bl, ecc):
    chunk(forced)
    rng = np.random.Generator(np.random.PCG64(forced * 31 + bl + ecc))
    rs = ffrs_gpu.RSi16(bl, ecc)
    o = O.RSi16(bl, ecc)
    nb, ml = 450, bl - ecc
    msg = rng.integers(0, 65536, size=(nb, ml), dtype=np.uint16)
    par = np.frombuffer(bytes(rs.encode(msg.tobytes())), np.uint16).reshape(nb, ecc)
    want = o.encode_blocks(msg, threads=8)
    np.testing.assert_array_equal(par, want)
    cw = np.concatenate([msg, want], axis=1)
    for i in range(nb):
        k = int(rng.integers(0, ecc // 2 + 3))
        for q in rng.choice(bl, size=k, replace=False):
            cw[i, q] = (int(cw[i, q]) + int(rng.integers(1, 65536))) & 0xFFFF
    m, e = np.ascontiguousarray(cw[:, :ml]), np.ascontiguousarray(cw[:, ml:])
    mo, eo = m.copy(), e.copy()
    so = o.repair_blocks(mo, eo, threads=8)
    mb, eb = bytearray(m.tobytes()), bytearray(e.tobytes())
    st = np.frombuffer(bytes(rs.repair_blocks(mb, eb)), np.uint8)
    np.testing.assert_array_equal(st.astype(np.int16), np.where(so < 0, 255, so.astype(np.int16)))
    np.testing.assert_array_equal(np.frombuffer(bytes(mb), np.uint16).reshape(nb, ml), mo)
    np.testing.assert_array_equal(np.frombuffer(bytes(eb), np.uint16).reshape(nb, ecc), eo)


def test_rs256_host_encode_split_upload(ffrs_gpu):
    """An encode of 32,768 blocks or more in one chunk uploads in four pieces,
    each encoded once its copy is in; with a ragged tail, from a pageable and
    from a page-locked buffer, against the oracle."""
    rng = np.random.Generator(np.random.PCG64(4242))
    ecc, ml, nb, tail = 32, 223, 40003, 150
    o = O.RS256(ecc, block_len=ml + ecc)
    rs = ffrs_gpu.RS256(ecc_len=ecc)
    buf = rng.integers(0, 256, size=nb * ml + tail, dtype=np.uint8)
    want = np.concatenate([o.encode_blocks(buf[:nb * ml].reshape(nb, ml), threads=8).ravel(),
                           O.RS256(ecc, block_len=tail + ecc).encode_blocks(buf[nb * ml:].reshape(1, tail)).ravel()])
    np.testing.assert_array_equal(np.frombuffer(bytes(rs.encode(buf.tobytes())), np.uint8), want)
    pinned = ffrs_gpu.create_buffer(buf.size)
    np.frombuffer(pinned, np.uint8)[:] = buf
    np.testing.assert_array_equal(np.frombuffer(bytes(rs.encode(pinned)), np.uint8), want)
