"""ffgpu_rs256_decode_noalloc (decode on the library's fixed scratch array)
against ffgpu_rs256_decode on the same corrupted blocks, twice in a row
(the second call reuses the scratch the first one left behind), plus its
limits.  Collected last so that it also runs after every other GPU test."""

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _blocks(rng, nb, ml, ecc):
    o = O.RS256(ecc, block_len=ml + ecc)
    data = rng.integers(0, 256, size=(nb, ml), dtype=np.uint8)
    par = o.encode_blocks(data, threads=8)
    cw = np.concatenate([data, par], axis=1)
    for i in range(nb):
        k = int(rng.integers(0, ecc // 2 + 3))
        pos = rng.choice(ml + ecc, size=k, replace=False)
        cw[i, pos] ^= rng.integers(1, 256, size=k, dtype=np.uint8)
    return np.ascontiguousarray(cw[:, :ml]), np.ascontiguousarray(cw[:, ml:])


def _decode(torch, code, fn, data, par):
    from libffrs_gb300 import capi

    nb, ml = data.shape
    d = torch.from_numpy(data).cuda()
    p = torch.from_numpy(par).cuda()
    s = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    capi.call(fn, code.h, d.data_ptr(), p.data_ptr(), nb, ml, s.data_ptr(), stream)
    torch.cuda.synchronize()
    return d.cpu().numpy(), p.cpu().numpy(), s.cpu().numpy()


@pytest.mark.parametrize("ecc,ml,nb", [(32, 223, 5000), (16, 239, 3001)])
def test_noalloc_matches_decode_twice(built, ecc, ml, nb):
    import torch

    from libffrs_gb300 import capi

    code = capi.RS256Code(ecc)
    rng = np.random.Generator(np.random.PCG64(ecc * 7 + nb))
    for _ in range(2):
        data, par = _blocks(rng, nb, ml, ecc)
        want = _decode(torch, code, "ffgpu_rs256_decode", data, par)
        got = _decode(torch, code, "ffgpu_rs256_decode_noalloc", data, par)
        for w, g in zip(want, got):
            np.testing.assert_array_equal(g, w)
        od, op = data.copy(), par.copy()
        st = O.RS256(ecc, block_len=ml + ecc).decode_blocks(od, op)
        np.testing.assert_array_equal(got[2], st)
        np.testing.assert_array_equal(got[0], od)


def _pool_used_high():
    """High-water mark of the device's default stream-ordered pool (the pool
    ffgpu_rs256_decode allocates its scratch from), read through the driver
    API; None where the query is not available."""
    import ctypes

    try:
        cu = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return None
    dev = ctypes.c_int()
    pool = ctypes.c_void_p()
    val = ctypes.c_uint64()
    if cu.cuCtxGetDevice(ctypes.byref(dev)) or cu.cuDeviceGetDefaultMemPool(ctypes.byref(pool), dev):
        return None
    CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8
    if cu.cuMemPoolGetAttribute(pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, ctypes.byref(val)):
        return None
    return pool, cu, val.value


def test_noalloc_allocates_nothing(built):
    """After the high-water mark of the stream-ordered pool is reset, a
    decode through the no-allocation entry point leaves it at zero, while the
    allocating entry point raises it."""
    import ctypes

    import torch

    from libffrs_gb300 import capi

    torch.zeros(1, device="cuda")
    q = _pool_used_high()
    if q is None:
        pytest.skip("the driver's pool attribute query is not available")
    pool, cu, _ = q
    code = capi.RS256Code(32)
    rng = np.random.Generator(np.random.PCG64(3))
    data, par = _blocks(rng, 4096, 223, 32)
    _decode(torch, code, "ffgpu_rs256_decode_noalloc", data, par)  # first call: scratch address set-up
    zero = ctypes.c_uint64(0)
    CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8
    assert cu.cuMemPoolSetAttribute(pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, ctypes.byref(zero)) == 0
    _decode(torch, code, "ffgpu_rs256_decode_noalloc", data, par)
    assert _pool_used_high()[2] == 0
    _decode(torch, code, "ffgpu_rs256_decode", data, par)
    assert _pool_used_high()[2] > 0


def test_noalloc_limits(built):
    import torch

    from libffrs_gb300 import capi

    code = capi.RS256Code(32)
    d = torch.zeros(8, dtype=torch.uint8, device="cuda")
    with pytest.raises(capi.FFGPUError, match="scratch"):
        # 524,289 blocks exceed the fixed scratch; rejected before any access
        capi.call("ffgpu_rs256_decode_noalloc", code.h, d.data_ptr(), d.data_ptr(), 524289, 223, d.data_ptr(), None)
    with pytest.raises(capi.FFGPUError, match="ecc_len 16 and 32"):
        other = capi.RS256Code(8)
        capi.call("ffgpu_rs256_decode_noalloc", other.h, d.data_ptr(), d.data_ptr(), 1, 200, d.data_ptr(), None)
    with pytest.raises(capi.FFGPUError, match="aligned"):
        capi.call("ffgpu_rs256_decode_noalloc", code.h, d.data_ptr() + 1, d.data_ptr(), 1, 223, d.data_ptr(), None)
    with pytest.raises(capi.FFGPUError, match="table decoder"):
        tab = capi.RS256Code(32)
        tab.set_table_only(True)
        capi.call("ffgpu_rs256_decode_noalloc", tab.h, d.data_ptr(), d.data_ptr(), 1, 223, d.data_ptr(), None)
