"""Bitsliced RS256 kernels (ecc_len 16 / 32, primitive 2) against the oracle
and against the byte-table kernels, over ragged block counts (tiles are 2048
blocks, plane words 32 blocks), odd message lengths (unaligned block starts)
and unaligned buffers (which take the table kernels)."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _corrupt(rng, data, par, ks):
    ml = data.shape[1]
    n = ml + par.shape[1]
    for i, k in enumerate(ks):
        pos = rng.choice(n, size=int(k), replace=False)
        vals = rng.integers(1, 256, size=int(k), dtype=np.uint8)
        for q, v in zip(pos, vals):
            if q < ml:
                data[i, q] ^= v
            else:
                par[i, q - ml] ^= v


def _run(code, data, par, ml, ecc, offset=0):
    """encode, synds, decode through the C ABI; returns numpy results."""
    import torch

    nb = data.shape[0]
    stream = torch.cuda.current_stream().cuda_stream
    raw_d = torch.zeros(nb * ml + offset + 8, dtype=torch.uint8, device="cuda")
    raw_p = torch.zeros(nb * ecc + offset + 8, dtype=torch.uint8, device="cuda")
    d = raw_d[offset : offset + nb * ml]
    p = raw_p[offset : offset + nb * ecc]
    d.copy_(torch.from_numpy(data.reshape(-1)).cuda())
    code.encode(d.data_ptr(), nb, ml, p.data_ptr(), stream)
    torch.cuda.synchronize()
    enc = p.cpu().numpy().reshape(nb, ecc).copy()
    p.copy_(torch.from_numpy(par.reshape(-1)).cuda())
    s = torch.zeros(nb * ecc, dtype=torch.uint8, device="cuda")
    code.synds(d.data_ptr(), p.data_ptr(), nb, ml, s.data_ptr(), stream)
    st = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    code.decode(d.data_ptr(), p.data_ptr(), nb, ml, st.data_ptr(), stream)
    torch.cuda.synchronize()
    return (
        enc,
        s.cpu().numpy().reshape(nb, ecc),
        st.cpu().numpy(),
        d.cpu().numpy().reshape(nb, ml),
        p.cpu().numpy().reshape(nb, ecc),
    )


CASES = [
    (32, 223, 1),
    (32, 223, 31),
    (32, 223, 33),
    (32, 223, 2049),
    (32, 223, 2048 * 3 + 7),
    (32, 1, 100),
    (32, 3, 257),
    (32, 17, 4100),
    (32, 100, 999),
    (16, 239, 2049),
    (16, 5, 77),
    (16, 128, 4096),
]


@pytest.mark.parametrize("ecc,ml,nb", CASES)
def test_bitsliced_vs_oracle(built, ecc, ml, nb):
    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(ecc * 100000 + ml * 100 + nb))
    o = O.RS256(ecc, block_len=ml + ecc)
    data = rng.integers(0, 256, size=(nb, ml), dtype=np.uint8)
    par = o.encode_blocks(data, threads=8)
    ks = rng.integers(0, ecc // 2 + 3, size=nb)
    cd, cp = data.copy(), par.copy()
    _corrupt(rng, cd, cp, ks)
    fast = capi.RS256Code(ecc)
    table = capi.RS256Code(ecc)
    table.set_table_only(True)
    # encode/decode on the corrupted blocks (both kernel families), then on the clean ones
    enc_f, syn_f, st_f, d_f, p_f = _run(fast, cd.copy(), cp.copy(), ml, ecc)
    enc_t, syn_t, st_t, d_t, p_t = _run(table, cd.copy(), cp.copy(), ml, ecc)
    clean_f = _run(fast, data.copy(), par.copy(), ml, ecc)
    np.testing.assert_array_equal(clean_f[0], par)
    assert not clean_f[1].any()
    assert clean_f[2].all()
    np.testing.assert_array_equal(syn_f, syn_t)
    sample = rng.choice(nb, size=min(nb, 64), replace=False)
    for i in sample:
        want = np.frombuffer(o.synds(bytes(cd[i]) + bytes(cp[i])), np.uint8)
        np.testing.assert_array_equal(syn_f[i], want)
    od, op = cd.copy(), cp.copy()
    so = o.decode_blocks(od, op, threads=8)
    for st, d, p in ((st_f, d_f, p_f), (st_t, d_t, p_t)):
        np.testing.assert_array_equal(st, so)
        np.testing.assert_array_equal(d, od)
        np.testing.assert_array_equal(p, op)


@pytest.mark.parametrize("offset", [1, 2, 3, 4, 8, 12])
def test_bitsliced_unaligned_buffers(built, offset):
    """Buffers off a 4-byte boundary (table kernels) and off a 16-byte one
    (offsets 4, 8, 12: the nibble-table encoder's first chunk starts before
    the buffer and its parity goes out in 4-byte words) give the oracle's
    results."""
    from libffrs_gb300 import capi

    ecc, ml, nb = 32, 223, 300
    rng = np.random.Generator(np.random.PCG64(offset))
    o = O.RS256(ecc)
    data = rng.integers(0, 256, size=(nb, ml), dtype=np.uint8)
    par = o.encode_blocks(data)
    cd, cp = data.copy(), par.copy()
    _corrupt(rng, cd, cp, rng.integers(0, 18, size=nb))
    code = capi.RS256Code(ecc)
    enc, syn, st, d, p = _run(code, cd.copy(), cp.copy(), ml, ecc, offset=offset)
    np.testing.assert_array_equal(enc, o.encode_blocks(cd))
    od, op = cd.copy(), cp.copy()
    so = o.decode_blocks(od, op)
    np.testing.assert_array_equal(st, so)
    np.testing.assert_array_equal(d, od)
    np.testing.assert_array_equal(p, op)


@pytest.mark.parametrize("ml,nb", [(223, 180000 + 3), (223, 2 * 152 * 1024 + 1000), (100, 2 * 160 * 1024 + 5)])
def test_encode_large_batches(built, ml, nb):
    """Batches on either side of the switch from the nibble-table encoder
    (each warp four blocks at a time) to the bitsliced LFSR (2048-block
    tiles), at about 1,365 blocks per SM."""
    import torch
    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(ml * 7 + nb))
    data = rng.integers(0, 256, size=(nb, ml), dtype=np.uint8)
    data[:64] = 255
    o = O.RS256(32, block_len=ml + 32)
    want = o.encode_blocks(data, threads=16)
    code = capi.RS256Code(32)
    stream = torch.cuda.current_stream().cuda_stream
    d = torch.from_numpy(data.reshape(-1)).cuda()
    p = torch.zeros(nb * 32, dtype=torch.uint8, device="cuda")
    code.encode(d.data_ptr(), nb, ml, p.data_ptr(), stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(p.cpu().numpy().reshape(nb, 32), want)
