"""The fused batch path (one persistent launch over mixed requests) gives the
same bytes and statuses as the plain per-request entry points, planned by hand,
autotuned, and replayed from a captured CUDA graph; and a sample of its RS256 /
RSi16 results matches the oracle."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _outputs(torch, reqs):
    return [(r["data"].clone(), r["par"].clone(), None if r["status"] is None else r["status"].clone())
            for r in reqs]


def _same(torch, a, b):
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            if (u is None) != (v is None):
                return False
            if u is not None and not torch.equal(u, v):
                return False
    return True


@pytest.fixture(scope="module")
def mixed(built):
    import torch

    import bench

    reqs, codes = bench.make_mixed(torch, 6 << 20, 1234)
    return torch, bench, reqs, codes


def test_batch_equals_plain(mixed):
    from libffrs_gb300 import capi

    torch, bench, reqs, _ = mixed
    sp = torch.cuda.current_stream().cuda_stream
    kinds = {(r["kind"], r["op"]) for r in reqs}
    assert {("rs256", "enc"), ("rs256", "dec"), ("rsi16", "enc"), ("rsi16", "dec"), ("circ16", "enc"),
            ("circ16", "dec")} <= kinds
    bench.mixed_restore(reqs)
    bench.mixed_plain(reqs, sp)
    torch.cuda.synchronize()
    ref = _outputs(torch, reqs)
    b = bench.mixed_batch(reqs)
    # hand-set plan (defaults), then the autotuned plan, then graph replays
    bench.mixed_restore(reqs)
    b.plan(autotune=False, stream=sp)
    n0 = capi.kernel_launches()
    b.launch(sp)
    torch.cuda.synchronize()
    # the persistent kernel, plus the CIRC16 chain: gather, the repair
    # stages over all codewords, scatter
    n_direct = capi.kernel_launches() - n0
    assert n_direct > 1
    assert _same(torch, ref, _outputs(torch, reqs))
    bench.mixed_restore(reqs)
    b.plan(autotune=True, stream=sp)
    info = b.info()
    assert info["items"] > 0 and info["grid"] > 0
    # autotuning restores the decode inputs: they still equal the pristine ones
    for r in reqs:
        if r["op"] == "dec":
            assert torch.equal(r["data"], r["data0"]) and torch.equal(r["par"], r["par0"])
    b.capture(sp)
    for _ in range(2):
        bench.mixed_restore(reqs)
        n0 = capi.kernel_launches()
        b.launch(sp)
        torch.cuda.synchronize()
        # one graph replay runs the same kernels as the direct launch
        assert capi.kernel_launches() - n0 == n_direct
        assert _same(torch, ref, _outputs(torch, reqs))


def test_batch_sample_vs_oracle(mixed):
    torch, bench, reqs, _ = mixed
    sp = torch.cuda.current_stream().cuda_stream
    bench.mixed_restore(reqs)
    b = bench.mixed_batch(reqs)
    b.plan(autotune=False, stream=sp)
    b.launch(sp)
    torch.cuda.synchronize()
    checked = 0
    for r in reqs:
        if checked >= 6:
            break
        if r["kind"] == "rs256":
            o = O.RS256(r["ecc"], block_len=r["ml"] + r["ecc"])
            if r["op"] == "enc":
                want = o.encode_blocks(r["data"].cpu().numpy())
                np.testing.assert_array_equal(r["par"].cpu().numpy(), want)
            else:
                d, p = r["data0"].cpu().numpy().copy(), r["par0"].cpu().numpy().copy()
                st = o.decode_blocks(d, p)
                np.testing.assert_array_equal(r["status"].cpu().numpy(), st)
                np.testing.assert_array_equal(r["data"].cpu().numpy(), d)
                np.testing.assert_array_equal(r["par"].cpu().numpy(), p)
            checked += 1
        elif r["kind"] == "rsi16" and r["nb"] <= 8:
            o = O.RSi16(r["ml"] + r["ecc"], r["ecc"])
            if r["op"] == "enc":
                want = o.encode_blocks(r["data"].cpu().numpy().view(np.uint16))
                np.testing.assert_array_equal(r["par"].cpu().numpy().view(np.uint16), want)
            else:
                m = r["data0"].cpu().numpy().view(np.uint16).copy()
                p = r["par0"].cpu().numpy().view(np.uint16).copy()
                st = o.repair_blocks(m, p)
                np.testing.assert_array_equal(r["status"].cpu().numpy(), st.astype(np.uint8))
                np.testing.assert_array_equal(r["data"].cpu().numpy().view(np.uint16), m)
                np.testing.assert_array_equal(r["par"].cpu().numpy().view(np.uint16), p)
            checked += 1
    assert checked >= 4
    # a CIRC16 repair request, codeword by codeword against the oracle
    r = next(r for r in reqs if r["kind"] == "circ16" and r["op"] == "dec")
    c = r["code"]
    o = O.CIRC16(128, 8, 128, 8, 4)
    m0 = r["data0"].cpu().numpy().view(np.uint16)
    e0 = r["par0"].cpu().numpy().view(np.uint16)
    got_m = r["data"].cpu().numpy().view(np.uint16)
    got_e = r["par"].cpu().numpy().view(np.uint16)
    got_s = r["status"].cpu().numpy()
    for i in range(min(r["nb"], 3)):
        m, e = m0[i].copy(), e0[i].copy()
        rc = o.repair(m, e)
        assert (got_s[i] == 0) == (rc == 0)
        np.testing.assert_array_equal(got_m[i], m)
        if rc == 0:
            np.testing.assert_array_equal(got_e[i], e)


def test_batch_rejects_bad_requests(built):
    from libffrs_gb300 import capi

    b = capi.Batch()
    c = capi.RS256Code(32)
    with pytest.raises(capi.FFGPUError):
        b.add_rs256(c, 7, None, None, 1, 223, None)
    with pytest.raises(capi.FFGPUError):
        b.add_rs256(c, capi.DECODE, None, None, 1, 223, None)  # decode needs a status array
    with pytest.raises(capi.FFGPUError):
        b.add_rs256(c, capi.ENCODE, None, None, 1, 224, None)  # 224 + 32 > 255
