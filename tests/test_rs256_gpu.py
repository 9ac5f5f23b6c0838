"""RS256 on the GPU: the reference-facing API against the reference's golden
outputs, the C ABI against the oracle, and full-size properties."""

import ctypes

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gold():
    return load_golden("rs256.npz")


def test_rs256_golden_api(ffrs_gpu, gold):
    for c in range(int(gold["ncases"][0])):
        p = f"c{c}_"
        ecc, bl = map(int, gold[p + "geom"])
        rs = ffrs_gpu.RS256(bl, ecc_len=ecc)
        assert rs.generator == gold[p + "generator"].tobytes()
        assert bytes(rs.encode(gold[p + "buffer"].tobytes())) == gold[p + "encoded"].tobytes(), (ecc, bl)
        data = gold[p + "received_data"]
        par = gold[p + "received_parity"]
        for i in range(data.shape[0]):
            assert bytes(rs._synds(data[i].tobytes() + par[i].tobytes())) == gold[p + "synds"][i].tobytes()
        # one block per call, as the reference API
        for i in range(data.shape[0]):
            m, e = bytearray(data[i].tobytes()), bytearray(par[i].tobytes())
            ok = rs.repair(m, e)
            assert ok == bool(gold[p + "status"][i]), (ecc, bl, i)
            assert bytes(m) == gold[p + "repaired_data"][i].tobytes()
            assert bytes(e) == gold[p + "repaired_parity"][i].tobytes()
        # batched over the contiguous buffers
        m, e = bytearray(data.tobytes()), bytearray(par.tobytes())
        st = np.frombuffer(bytes(rs.repair_blocks(m, e)), np.uint8)
        np.testing.assert_array_equal(st, gold[p + "status"])
        assert bytes(m) == gold[p + "repaired_data"].tobytes()
        assert bytes(e) == gold[p + "repaired_parity"].tobytes()


def test_rs256_constructor_errors(ffrs_gpu):
    with pytest.raises(ValueError):
        ffrs_gpu.RS256(message_len=223)
    with pytest.raises(ValueError):
        ffrs_gpu.RS256(255, 223, ecc_len=33)
    with pytest.raises(ValueError):
        ffrs_gpu.RS256(254, 255)
    with pytest.raises(ValueError):
        ffrs_gpu.RS256(block_len=8, ecc_len=8)
    with pytest.raises(ValueError):
        ffrs_gpu.RS256()
    rs = ffrs_gpu.RS256(ecc_len=32)
    assert rs.block_len == 255 and rs.message_len == 223
    rs.block_len = 48
    assert rs.message_len == 16
    with pytest.raises(ValueError):
        rs.block_len = 32
    assert ffrs_gpu.RS256(254, 222).ecc_len == 32
    assert ffrs_gpu.RS256(message_len=8, ecc_len=9).block_len == 17
    assert bytes(rs.encode(b"")) == b""


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


@pytest.mark.parametrize("ecc,ml", [(32, 223), (2, 200), (4, 120), (8, 247), (16, 239), (64, 191), (17, 90), (5, 7)])
def test_rs256_capi_vs_oracle(built, ecc, ml):
    import torch

    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(ecc * 1000 + ml))
    nb = 3000
    o = O.RS256(ecc, block_len=ml + ecc)
    code = capi.RS256Code(ecc)
    data = rng.integers(0, 256, size=(nb, ml), dtype=np.uint8)
    d_data = torch.from_numpy(data).cuda()
    d_par = torch.zeros((nb, ecc), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    code.encode(d_data.data_ptr(), nb, ml, d_par.data_ptr(), stream)
    torch.cuda.synchronize()
    par = o.encode_blocks(data, threads=8)
    np.testing.assert_array_equal(d_par.cpu().numpy(), par)
    ks = rng.integers(0, ecc // 2 + 4, size=nb)
    _corrupt(rng, data, par, ks)
    d_data = torch.from_numpy(data).cuda()
    d_par = torch.from_numpy(par).cuda()
    d_st = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    code.decode(d_data.data_ptr(), d_par.data_ptr(), nb, ml, d_st.data_ptr(), stream)
    torch.cuda.synchronize()
    st = o.decode_blocks(data, par, threads=8)
    np.testing.assert_array_equal(d_st.cpu().numpy(), st)
    np.testing.assert_array_equal(d_data.cpu().numpy(), data)
    np.testing.assert_array_equal(d_par.cpu().numpy(), par)


def test_rs256_full_size_roundtrip(built):
    """1,048,576 blocks of 223 + 32 bytes, 0-16 errors (1% with 17-20): every
    block within capacity is restored with status 1; the others match the
    oracle's status and bytes."""
    import torch

    from libffrs_gb300 import capi

    nb, ml, ecc = 1 << 20, 223, 32
    g = torch.Generator(device="cuda")
    g.manual_seed(99)
    data = torch.randint(0, 256, (nb, ml), dtype=torch.uint8, device="cuda", generator=g)
    par = torch.zeros((nb, ecc), dtype=torch.uint8, device="cuda")
    code = capi.RS256Code(ecc)
    stream = torch.cuda.current_stream().cuda_stream
    code.encode(data.data_ptr(), nb, ml, par.data_ptr(), stream)
    orig_d, orig_p = data.clone(), par.clone()
    rng = np.random.Generator(np.random.PCG64(5))
    ks = rng.integers(0, 17, size=nb)
    heavy = rng.random(nb) < 0.01
    ks[heavy] = rng.integers(17, 21, size=int(heavy.sum()))
    # vectorised corruption on the device: up to 20 distinct positions per block
    pos = torch.rand((nb, 255), device="cuda", generator=g).argsort(dim=1)[:, :20]
    mask = torch.arange(20, device="cuda")[None, :] < torch.from_numpy(ks).cuda()[:, None]
    vals = torch.randint(1, 256, (nb, 20), dtype=torch.uint8, device="cuda", generator=g) * mask.to(torch.uint8)
    cw = torch.cat([data, par], dim=1)
    rows = torch.arange(nb, device="cuda")[:, None].expand(nb, 20)
    cw[rows, pos] ^= vals
    data = cw[:, :ml].contiguous()
    par = cw[:, ml:].contiguous()
    st = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    code.decode(data.data_ptr(), par.data_ptr(), nb, ml, st.data_ptr(), stream)
    torch.cuda.synchronize()
    stn = st.cpu().numpy()
    ok = ~heavy
    assert stn[ok].all()
    assert torch.equal(data[torch.from_numpy(ok).cuda()], orig_d[torch.from_numpy(ok).cuda()])
    assert torch.equal(par[torch.from_numpy(ok).cuda()], orig_p[torch.from_numpy(ok).cuda()])
    # beyond capacity: compare with the oracle on those blocks
    hi = np.nonzero(heavy)[0]
    o = O.RS256(32)
    hd = cw[torch.from_numpy(hi).cuda(), :ml].cpu().numpy().copy()
    hp = cw[torch.from_numpy(hi).cuda(), ml:].cpu().numpy().copy()
    so = o.decode_blocks(hd, hp, threads=8)
    np.testing.assert_array_equal(stn[hi], so)
    np.testing.assert_array_equal(data[torch.from_numpy(hi).cuda()].cpu().numpy(), hd)
    np.testing.assert_array_equal(par[torch.from_numpy(hi).cuda()].cpu().numpy(), hp)
