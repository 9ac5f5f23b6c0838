"""The one-block-per-thread RSi16 kernels (ecc 32 and 64 on contiguous,
16-byte aligned uint16 blocks) against the oracle: ragged block counts around the
32-block warp tile, the shortest and longest block lengths, extreme words
(the lazy reduction's largest magnitudes), and the fallback taken when the
buffers are not 16-byte aligned."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _encode(torch, capi, bl, ecc, msg, offset_words=0):
    """parity of msg [nb, bl - ecc] through the C ABI; the message buffer
    starts offset_words uint16 words past a 16-byte boundary"""
    nb, ml = msg.shape
    flat = torch.zeros(nb * ml + 8, dtype=torch.int16, device="cuda")
    m = flat[offset_words:offset_words + nb * ml]
    m.copy_(torch.from_numpy(msg.reshape(-1).view(np.int16)).cuda())
    p = torch.zeros(nb * ecc, dtype=torch.int16, device="cuda")
    capi.RSi16Code(bl, ecc).encode(m.data_ptr(), nb, p.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return p.cpu().numpy().view(np.uint16).reshape(nb, ecc)


@pytest.mark.parametrize("ecc", [32, 64])
@pytest.mark.parametrize("bl,nb", [(128, 1), (128, 33), (1024, 31), (1024, 32), (1024, 33), (1024, 1000),
                                   (4096, 70), (65536, 3)])
def test_bt_encode_vs_oracle(built, bl, nb, ecc):
    import torch

    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(bl * 3 + nb + ecc))
    msg = rng.integers(0, 65536, size=(nb, bl - ecc), dtype=np.uint16)
    np.testing.assert_array_equal(_encode(torch, capi, bl, ecc, msg), O.RSi16(bl, ecc).encode_blocks(msg))


@pytest.mark.parametrize("ecc", [32, 64])
def test_bt_encode_extreme_words(built, ecc):
    import torch

    from libffrs_gb300 import capi

    bl = 1024
    rng = np.random.Generator(np.random.PCG64(77))
    msg = np.empty((96, bl - ecc), dtype=np.uint16)
    msg[:32] = 65535
    msg[32:64] = 0
    msg[64:] = rng.choice(np.array([0, 1, 32768, 65535], dtype=np.uint16), size=(32, bl - ecc))
    np.testing.assert_array_equal(_encode(torch, capi, bl, ecc, msg), O.RSi16(bl, ecc).encode_blocks(msg))


@pytest.mark.parametrize("ecc", [32, 64])
def test_bt_unaligned_falls_back(built, ecc):
    import torch

    from libffrs_gb300 import capi

    bl, nb = 1024, 45
    rng = np.random.Generator(np.random.PCG64(78))
    msg = rng.integers(0, 65536, size=(nb, bl - ecc), dtype=np.uint16)
    want = O.RSi16(bl, ecc).encode_blocks(msg)
    np.testing.assert_array_equal(_encode(torch, capi, bl, ecc, msg, offset_words=1), want)
    np.testing.assert_array_equal(_encode(torch, capi, bl, ecc, msg, offset_words=8), want)


def _corrupt(rng, cw, k):
    """k changed words at distinct positions, each by a nonzero delta mod
    65537 whose result still fits a uint16 word"""
    for q in rng.choice(cw.size, size=k, replace=False):
        while True:
            v = (int(cw[q]) + int(rng.integers(1, 65537))) % 65537
            if v != 65536:
                break
        cw[q] = v


@pytest.mark.parametrize("ecc", [32, 64])
@pytest.mark.parametrize("bl,nb", [(128, 33), (1024, 1), (1024, 95), (4096, 40), (65536, 3)])
def test_bt_repair_vs_oracle(built, bl, nb, ecc):
    """Statuses and repaired words of every block, 0 to ecc/2 + 4 errors (the
    ones past ecc/2 go to the mirror), and the path counters."""
    import torch

    from libffrs_gb300 import capi

    ml = bl - ecc
    rng = np.random.Generator(np.random.PCG64(bl * 5 + nb + ecc))
    o = O.RSi16(bl, ecc)
    msg = rng.integers(0, 65536, size=(nb, ml), dtype=np.uint16)
    cw = np.concatenate([msg, o.encode_blocks(msg)], axis=1)
    for i in range(nb):
        _corrupt(rng, cw[i], int(rng.integers(0, ecc // 2 + 5)) if i % 7 else 0)
    m, p = np.ascontiguousarray(cw[:, :ml]), np.ascontiguousarray(cw[:, ml:])
    dm = torch.from_numpy(m.view(np.int16)).cuda()
    dp = torch.from_numpy(p.view(np.int16)).cuda()
    ds = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    capi.rsi16_repair_counters(reset=True)
    capi.RSi16Code(bl, ecc).repair(dm.data_ptr(), dp.data_ptr(), nb, ds.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    fast, mirror = capi.rsi16_repair_counters()
    assert fast + mirror == nb
    mo, po = m.copy(), p.copy()
    so = o.repair_blocks(mo, po)
    np.testing.assert_array_equal(ds.cpu().numpy(), np.where(so < 0, 255, so.astype(np.int16)).astype(np.uint8))
    np.testing.assert_array_equal(dm.cpu().numpy().view(np.uint16), mo)
    np.testing.assert_array_equal(dp.cpu().numpy().view(np.uint16), po)


@pytest.mark.parametrize("nb,k", [(1, 16), (40, 16), (1000, 48), (300, 64)])
def test_known_location_repair_many_blocks(built, nb, k):
    """ffgpu_rsi16_repair_known: nblocks blocks sharing one list of k known
    error positions (device memory), every block against the oracle."""
    import torch

    from libffrs_gb300 import capi

    bl, ecc = 1024, 64
    rng = np.random.Generator(np.random.PCG64(nb * 11 + k))
    o = O.RSi16(bl, ecc)
    msg = rng.integers(0, 65536, size=(nb, bl - ecc), dtype=np.uint16)
    cw = np.concatenate([msg, o.encode_blocks(msg)], axis=1)
    pos = np.sort(rng.choice(bl, size=k, replace=False)).astype(np.uint32)
    for i in range(nb):
        for q in pos:
            while True:
                v = (int(cw[i, q]) + int(rng.integers(1, 65537))) % 65537
                if v != 65536:
                    break
            cw[i, q] = v
    m, p = np.ascontiguousarray(cw[:, :bl - ecc]), np.ascontiguousarray(cw[:, bl - ecc:])
    dm = torch.from_numpy(m.view(np.int16)).cuda()
    dp = torch.from_numpy(p.view(np.int16)).cuda()
    ds = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    dpos = torch.from_numpy(pos.view(np.int32)).cuda()
    code = capi.RSi16Code(bl, ecc)  # held: its handle is freed with the object
    capi.call("ffgpu_rsi16_repair_known", code.h, dm.data_ptr(), dp.data_ptr(), nb, dpos.data_ptr(), k,
              ds.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    want_m, want_p, want_s = m.copy(), p.copy(), []
    for i in range(nb):
        mi, pi = want_m[i].copy(), want_p[i].copy()
        want_s.append(int(o.repair(mi, pi, [int(x) for x in pos])))
        want_m[i], want_p[i] = mi, pi
    np.testing.assert_array_equal(ds.cpu().numpy(), np.array(want_s, dtype=np.uint8))
    np.testing.assert_array_equal(dm.cpu().numpy().view(np.uint16), want_m)
    np.testing.assert_array_equal(dp.cpu().numpy().view(np.uint16), want_p)
