"""The `.ffrs` backup / repair pipeline (libffrs_gb300.par) against what the
reference's own tools write for the same files (tests/golden/ffrs_par.json,
from tests/golden/make_ffrs_golden.py): the parity files byte for byte, and
the repaired files."""

import hashlib
import json
import os

import pytest

from conftest import GOLDEN

CASES = json.load(open(os.path.join(GOLDEN, "ffrs_par.json")))["cases"]


def _input(case):
    import numpy as np

    return np.random.Generator(np.random.PCG64(case["seed"])).integers(0, 256, case["size"], dtype=np.uint8).tobytes()


def _write(path, data, mtime_ns):
    with open(path, "wb") as f:
        f.write(data)
    os.utime(path, ns=(mtime_ns, mtime_ns))


def test_file_entry_lines_match_the_reference(built):
    """The file entry (size, modification time, BLAKE2b, quoted name) of every
    case, without a GPU."""
    import base64

    from libffrs_gb300 import par

    for case in CASES:
        digest = hashlib.blake2b(_input(case), digest_size=20).digest()
        line = "f s:%s m:%s h:b2:%s p:%s" % (par.b64hex(case["size"]), par.b64hex(case["mtime_ns"]),
                                            base64.urlsafe_b64encode(digest).strip(b"=").decode(),
                                            par._quote(case["name"]))
        assert line == case["ffrs_header"][2]
        assert par.b64hex_dec(par.b64hex(case["mtime_ns"])) == case["mtime_ns"]


@pytest.mark.gpu
def test_backup_is_byte_identical_to_the_reference(built, tmp_path):
    from libffrs_gb300 import par

    names = []
    for case in CASES:
        _write(tmp_path / case["name"], _input(case), case["mtime_ns"])
        names.append(case["name"])
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        codecs = {c["name"]: par.deserialize(c["ffrs_header"][1].encode()) for c in CASES}
        # several files through one pipeline run, each with the codec the
        # reference chose for its size
        sizes = {c["size"]: codecs[c["name"]] for c in CASES}
        out = par.backup(names, lambda size: sizes[size])
    finally:
        os.chdir(cwd)
    assert out == [n + ".ffrs" for n in names]
    for case in CASES:
        got = open(tmp_path / (case["name"] + ".ffrs"), "rb").read()
        assert got.split(b"\n", 4)[:4] == [ln.encode("latin-1") for ln in case["ffrs_header"]]
        assert len(got) == case["ffrs_len"]
        assert hashlib.sha256(got).hexdigest() == case["ffrs_sha256"], case["name"]


@pytest.mark.gpu
def test_repair_restores_like_the_reference(built, tmp_path):
    from libffrs_gb300 import par

    for case in CASES:
        data = _input(case)
        path = tmp_path / case["name"]
        _write(path, data, case["mtime_ns"])
        par.backup([str(path)], par.deserialize(case["ffrs_header"][1].encode()))
        bad = bytearray(data)
        for a, b in case["damage"]:
            bad[a:b] = bytes(b - a)
        _write(path, bytes(bad), case["mtime_ns"])
        assert par.repair(str(path) + ".ffrs") == str(path)
        got = open(path, "rb").read()
        assert hashlib.sha256(got).hexdigest() == case["repaired_sha256"], case["name"]
        assert got == data
        assert os.stat(path).st_mtime_ns == case["mtime_ns"]


@pytest.mark.gpu
def test_parity_file_round_trip(built, tmp_path):
    from libffrs_gb300 import par

    case = CASES[0]
    path = tmp_path / "sub dir" / "x.bin"
    path.parent.mkdir()
    _write(path, _input(case), case["mtime_ns"])
    codec = par.deserialize(case["ffrs_header"][1].encode())
    par.backup([str(path)], codec)
    c2, files, ecc = par.read_parity_file(str(path) + ".ffrs")
    assert par.serialize(c2) == par.serialize(codec)
    assert files[0][0] == case["size"] and files[0][1] == case["mtime_ns"] and files[0][3] == str(path)
    assert len(ecc) == codec.ecc_size
    with pytest.raises(FileExistsError):
        par.backup([str(path)], codec)
