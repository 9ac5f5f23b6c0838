"""Parity at the benchmark configurations' full sizes, on the benchmark's own
seeded inputs (bench.py's generators), every block against the oracle:

* RS256 encode, ecc_len 32: 65,536 blocks of 223 bytes;
* RSi16(1024, 64) encode and decode with 0-32 symbol errors per block:
  262,144 blocks;
* the mixed batch (RS256 / RSi16 / CIRC16, encodes and decodes, uneven
  lengths): 64 MiB, every request.

The RS256 decode configuration (1,048,576 blocks) is covered at full size in
test_rs256_gpu.py."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

THREADS = 16


def test_rs256_encode_65536_blocks(built):
    import torch

    import bench
    from libffrs_gb300 import capi

    nb = 65536
    data = bench.rs256_encode_chunk(2000, 0, nb)
    d = torch.from_numpy(data).cuda()
    p = torch.zeros((nb, 32), dtype=torch.uint8, device="cuda")
    capi.RS256Code(32).encode(d.data_ptr(), nb, 223, p.data_ptr(), torch.cuda.current_stream().cuda_stream)
    np.testing.assert_array_equal(p.cpu().numpy(), O.RS256(32).encode_blocks(data, threads=THREADS))


def _rsi16_gpu(torch, capi, msg, pos=None, d=None):
    nb = msg.shape[0]
    code = capi.RSi16Code(1024, 64)
    sp = torch.cuda.current_stream().cuda_stream
    m = torch.from_numpy(msg.view(np.int16)).cuda()
    p = torch.zeros((nb, 64), dtype=torch.int16, device="cuda")
    code.encode(m.data_ptr(), nb, p.data_ptr(), sp)
    clean = p.cpu().numpy().view(np.uint16).copy()
    if pos is None:
        return clean, None
    import bench

    cw = torch.cat([m, p], dim=1)
    bench.torch_rsi16_apply_errors(torch, cw, pos, d)
    m2, p2 = cw[:, :960].contiguous(), cw[:, 960:].contiguous()
    s = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    code.repair(m2.data_ptr(), p2.data_ptr(), nb, s.data_ptr(), sp)
    torch.cuda.synchronize()
    return clean, (m2.cpu().numpy().view(np.uint16), p2.cpu().numpy().view(np.uint16), s.cpu().numpy())


def test_rsi16_encode_262144_blocks(built):
    import torch

    import bench
    from libffrs_gb300 import capi

    msg = bench.chunks(bench.rsi16_chunk, 3000, 262144, bench.RSI_CHUNK, corrupt=False)[0]
    par, _ = _rsi16_gpu(torch, capi, msg)
    np.testing.assert_array_equal(par, O.RSi16(1024, 64).encode_blocks(msg, threads=THREADS))


def test_rsi16_decode_262144_blocks(built):
    """Every block's RepairStatus and repaired words, 0-32 errors per block."""
    import torch

    import bench
    from libffrs_gb300 import capi

    nb = 262144
    msg, pos, d = bench.chunks(bench.rsi16_chunk, 3100, nb, bench.RSI_CHUNK, corrupt=True)
    par, (gm, gp, gs) = _rsi16_gpu(torch, capi, msg, pos, d)
    o = O.RSi16(1024, 64)
    np.testing.assert_array_equal(par, o.encode_blocks(msg, threads=THREADS))
    cw = np.concatenate([msg, par], axis=1).astype(np.int64)
    bench.rsi16_apply_errors(cw, pos, d)
    m = np.ascontiguousarray(cw[:, :960].astype(np.uint16))
    p = np.ascontiguousarray(cw[:, 960:].astype(np.uint16))
    st = o.repair_blocks(m, p, threads=THREADS)
    np.testing.assert_array_equal(gs, np.where(st < 0, 255, st.astype(np.int16)).astype(np.uint8))
    np.testing.assert_array_equal(gm, m)
    np.testing.assert_array_equal(gp, p)
    assert (st == 2).mean() > 0.9  # most blocks are repaired, not trivially clean


def test_mixed_batch_64mib_every_request(built):
    """The batched launch (autotuned plan, graph replay) on a 64 MiB mix: every
    request's outputs equal the oracle's."""
    import torch

    import bench

    reqs, _ = bench.make_mixed(torch, 64 << 20, 4321)
    host0 = [(bench._host_u(r["data0"]), bench._host_u(r["par0"])) for r in reqs]
    sp = torch.cuda.current_stream().cuda_stream
    b = bench.mixed_batch(reqs)
    bench.mixed_restore(reqs)
    b.plan(autotune=True, stream=sp)
    b.capture(sp)
    for _ in range(2):  # the second replay starts from the first one's outputs restored
        bench.mixed_restore(reqs)
        b.launch(sp)
    torch.cuda.synchronize()
    codes = {}
    kinds = set()
    for r, (a0, b0) in zip(reqs, host0):
        wa, wb, ws = bench.mixed_expect(r, a0, b0, codes, THREADS)
        kinds.add((r["kind"], r["op"]))
        np.testing.assert_array_equal(bench._host_u(r["par"]), wb)
        if r["op"] == "dec":
            np.testing.assert_array_equal(bench._host_u(r["data"]), wa)
            np.testing.assert_array_equal(r["status"].cpu().numpy(), ws)
    assert len(kinds) == 6, kinds
