"""The C ABI library builds, loads and exports every symbol include/ffgpu.h
declares; error paths that need no GPU behave.  Runs without a GPU."""

import ctypes
import os

import pytest

from conftest import REPO


def test_header_declares_entry_points():
    from libffrs_gb300 import capi

    syms = capi.declared_symbols()
    for must in ("ffgpu_rs256_encode", "ffgpu_rs256_decode", "ffgpu_rsi16_encode", "ffgpu_rsi16_repair",
                 "ffgpu_circ16_encode", "ffgpu_circ16_repair", "ffgpu_last_error"):
        assert must in syms


def test_library_exports_all_declared_symbols(built):
    from libffrs_gb300 import capi

    lib = ctypes.CDLL(capi.LIB_PATH)
    missing = [s for s in capi.declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_extension_module_loads(built):
    import libffrs_gb300

    lf = libffrs_gb300.libffrs
    for name in ("RS256", "RSi16", "CIRC16", "RepairStatus", "GF256", "GFi16", "create_buffer", "set_logger"):
        assert hasattr(lf, name), name
    assert int(lf.RepairStatus.RepairOk) == 2 and int(lf.RepairStatus.ErrorLocationFail) == 4


def test_argument_errors_without_gpu(built):
    """Geometry errors are raised before any device work."""
    import libffrs_gb300

    lf = libffrs_gb300.libffrs
    with pytest.raises(ValueError):
        lf.RS256()
    with pytest.raises(ValueError):
        lf.RS256(message_len=223)
    with pytest.raises(ValueError):
        lf.RS256(255, 223, ecc_len=33)


def test_gf_helpers_match_oracle(built):
    import numpy as np

    import libffrs_gb300
    from oracle import oracle as O

    lf = libffrs_gb300.libffrs
    gf = lf.GF256()
    o = O.RS256(16)
    gen = o.generator
    msg = bytes(range(1, 40))
    # the reference's own encode property (tests/test_lib_rs256.py:84-90)
    assert bytes(gf.poly_mod_x_n(msg, gen[1:])) == bytes(o.encode(msg))
    # field identities
    for a in range(1, 256, 7):
        assert gf.mul(a, gf.inv(a)) == 1
        assert gf.div(gf.mul(a, 9), 9) == a
    g16 = lf.GFi16()
    for a in (1, 2, 3, 65535, 65536):
        assert g16.mul(a, g16.inv(a)) == 1
    assert g16.add(65536, 1) == 0 and g16.sub(0, 1) == 65536
    assert np.uint32(g16.mul(65537 % 65537 + 65536, 2)) == g16.mul(65536, 2)
