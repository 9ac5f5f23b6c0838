"""Edge cases on the GPU: zero-block calls of every entry point, an empty
batch, batches of a single kind (CIRC16 alone runs the staged chain with no
item launch), the narrowest and widest RS256 codes, RSi16 codes whose
message is empty (block_len == ecc_len), and single-block calls; every
output against the oracle or the plain per-request path."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


def test_zero_blocks(built):
    import torch

    from libffrs_gb300 import capi

    sp = _stream()
    buf = torch.zeros(64, dtype=torch.uint8, device="cuda")
    p = buf.data_ptr()
    rs = capi.RS256Code(32)
    rs.encode(p, 0, 223, p, sp)
    rs.decode(p, p, 0, 223, p, sp)
    ri = capi.RSi16Code(1024, 64)
    ri.encode(p, 0, p, sp)
    ri.repair(p, p, 0, p, sp)
    ri.synd(p, p, 0, p, sp)
    c = capi.CIRC16Code(128, 8, 128, 8, 4)
    c.encode(p, 0, p, sp)
    c.repair(p, p, 0, p, sp)
    torch.cuda.synchronize()
    assert int(buf.sum()) == 0


def test_empty_batch(built):
    import torch

    from libffrs_gb300 import capi

    sp = _stream()
    b = capi.Batch()
    b.plan(autotune=True, stream=sp)
    b.capture(sp)
    b.launch(sp)
    b.launch(sp)
    torch.cuda.synchronize()
    assert b.info()["items"] == 0


def _circ_requests(torch, c, rng, sizes, decode):
    reqs = []
    for nb in sizes:
        msg = torch.from_numpy(rng.integers(-32768, 32768, size=(nb, c.message_len), dtype=np.int16)).cuda()
        ecc = torch.zeros((nb, c.ecc_len), dtype=torch.int16, device="cuda")
        c.encode(msg.data_ptr(), nb, ecc.data_ptr(), _stream())
        if decode:
            for i in range(nb):
                n = int(rng.integers(1, 65))
                s0 = int(rng.integers(0, c.message_len - n))
                msg[i, s0:s0 + n] += 1
        st = torch.zeros(nb, dtype=torch.uint8, device="cuda")
        reqs.append((nb, msg, ecc, st, msg.clone(), ecc.clone()))
    torch.cuda.synchronize()
    return reqs


@pytest.mark.parametrize("decode", [False, True])
@pytest.mark.parametrize("geom", [(128, 8, 128, 8, 4), (64, 4, 32, 8, 4)])
def test_batch_circ16_only(built, geom, decode):
    """A batch of CIRC16 requests only, with two codes: the gathered chain
    per code and direction, scattered back, against one plain call per
    request."""
    import torch

    from libffrs_gb300 import capi

    sp = _stream()
    rng = np.random.Generator(np.random.PCG64(sum(geom) + decode))
    codes = [capi.CIRC16Code(*geom), capi.CIRC16Code(32, 4, 64, 8, 2)]
    reqs = [(c, r) for c in codes for r in _circ_requests(torch, c, rng, (1, 3, 2), decode)]
    # plain path
    for c, (nb, msg, ecc, st, m0, e0) in reqs:
        if decode:
            c.repair(msg.data_ptr(), ecc.data_ptr(), nb, st.data_ptr(), sp)
        else:
            c.encode(msg.data_ptr(), nb, ecc.data_ptr(), sp)
    torch.cuda.synchronize()
    want = [(msg.clone(), ecc.clone(), st.clone()) for _, (nb, msg, ecc, st, m0, e0) in reqs]
    for _, (nb, msg, ecc, st, m0, e0) in reqs:
        msg.copy_(m0)
        ecc.copy_(e0 if decode else torch.zeros_like(e0))
        st.zero_()
    b = capi.Batch()
    op = capi.DECODE if decode else capi.ENCODE
    for c, (nb, msg, ecc, st, m0, e0) in reqs:
        b.add_circ16(c, msg.data_ptr(), ecc.data_ptr(), nb, op, st.data_ptr() if decode else None)
    b.plan(autotune=False, stream=sp)
    b.capture(sp)
    b.launch(sp)
    torch.cuda.synchronize()
    assert b.info()["items"] == 0
    for (_, (nb, msg, ecc, st, m0, e0)), (wm, we, ws) in zip(reqs, want):
        assert torch.equal(msg, wm) and torch.equal(ecc, we)
        if decode:
            assert torch.equal(st, ws)


@pytest.mark.parametrize("ecc,ml", [(1, 254), (254, 1), (128, 127), (100, 50), (3, 1)])
def test_rs256_extreme_codes_vs_oracle(built, ecc, ml):
    import torch

    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(ecc * 7 + ml))
    nb = 700
    o = O.RS256(ecc, block_len=ml + ecc)
    code = capi.RS256Code(ecc)
    data = rng.integers(0, 256, size=(nb, ml), dtype=np.uint8)
    par = o.encode_blocks(data, threads=8)
    d_data = torch.from_numpy(data).cuda()
    d_par = torch.zeros((nb, ecc), dtype=torch.uint8, device="cuda")
    code.encode(d_data.data_ptr(), nb, ml, d_par.data_ptr(), _stream())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_par.cpu().numpy(), par)
    n = ml + ecc
    for i in range(nb):
        for _ in range(int(rng.integers(0, ecc // 2 + 3))):
            q = int(rng.integers(0, n))
            v = np.uint8(rng.integers(1, 256))
            if q < ml:
                data[i, q] ^= v
            else:
                par[i, q - ml] ^= v
    d_data = torch.from_numpy(data).cuda()
    d_par = torch.from_numpy(par).cuda()
    d_st = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    code.decode(d_data.data_ptr(), d_par.data_ptr(), nb, ml, d_st.data_ptr(), _stream())
    torch.cuda.synchronize()
    st = o.decode_blocks(data, par, threads=8)
    np.testing.assert_array_equal(d_st.cpu().numpy(), st)
    np.testing.assert_array_equal(d_data.cpu().numpy(), data)
    np.testing.assert_array_equal(d_par.cpu().numpy(), par)


@pytest.mark.parametrize("ecc", [16, 32, 64])
def test_rsi16_empty_message(built, ecc):
    """block_len == ecc_len: every word is parity; encode gives zeros, and
    repairs of corrupted all-parity blocks match the oracle."""
    import torch

    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(ecc))
    nb = 200
    o = O.RSi16(ecc, ecc)
    code = capi.RSi16Code(ecc, ecc)
    msg = torch.zeros((nb, 1), dtype=torch.int16, device="cuda")  # no message words are read
    par = torch.full((nb, ecc), 7, dtype=torch.int16, device="cuda")
    code.encode(msg.data_ptr(), nb, par.data_ptr(), _stream())
    torch.cuda.synchronize()
    assert int(par.abs().sum()) == 0
    cw = np.zeros((nb, ecc), np.uint16)
    for i in range(nb):
        for q in rng.choice(ecc, size=int(rng.integers(0, ecc // 2 + 2)), replace=False):
            cw[i, q] = int(rng.integers(1, 65536))
    d_par = torch.from_numpy(cw.view(np.int16).copy()).cuda()
    st = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    code.repair(msg.data_ptr(), d_par.data_ptr(), nb, st.data_ptr(), _stream())
    torch.cuda.synchronize()
    mo = np.zeros((nb, 0), np.uint16)
    eo = cw.copy()
    so = o.repair_blocks(mo, eo, threads=8)
    np.testing.assert_array_equal(st.cpu().numpy().astype(np.int16), np.where(so < 0, 255, so.astype(np.int16)))
    np.testing.assert_array_equal(d_par.cpu().numpy().view(np.uint16), eo)


def test_single_block_calls(built):
    """One block through every device entry point, against the oracle."""
    import torch

    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(1))
    sp = _stream()
    for ecc, ml in ((32, 223), (8, 40)):
        o = O.RS256(ecc, block_len=ml + ecc)
        data = rng.integers(0, 256, size=(1, ml), dtype=np.uint8)
        par = o.encode_blocks(data, threads=1)
        data[0, 3] ^= 0x5A
        d_d, d_p = torch.from_numpy(data).cuda(), torch.from_numpy(par).cuda()
        st = torch.zeros(1, dtype=torch.uint8, device="cuda")
        capi.RS256Code(ecc).decode(d_d.data_ptr(), d_p.data_ptr(), 1, ml, st.data_ptr(), sp)
        torch.cuda.synchronize()
        so = o.decode_blocks(data, par, threads=1)
        assert int(st[0]) == int(so[0]) == 1
        np.testing.assert_array_equal(d_d.cpu().numpy(), data)
    o = O.RSi16(1024, 64)
    msg = rng.integers(0, 65536, size=(1, 960), dtype=np.uint16)
    par = o.encode_blocks(msg, threads=1)
    code = capi.RSi16Code(1024, 64)
    d_m = torch.from_numpy(msg.view(np.int16).copy()).cuda()
    d_p = torch.zeros((1, 64), dtype=torch.int16, device="cuda")
    code.encode(d_m.data_ptr(), 1, d_p.data_ptr(), sp)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_p.cpu().numpy().view(np.uint16), par)
