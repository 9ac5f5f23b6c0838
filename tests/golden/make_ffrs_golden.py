"""Generates tests/golden/ffrs_par.json: what the reference's own `.ffrs`
tools (`python -m ffrs.par backup` / `repair`, running on the reference's
extension built by oracle/build_ref.sh) write for seeded input files.

    oracle/build_ref.sh /root/reference
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_ffrs_golden.py /root/reference

For every case: a file of `size` seeded bytes (numpy PCG64, `seed`) named
`name`, modification time `mtime_ns`, backed up in its own directory; the
fixture keeps the parity file's header lines (signature, codec, file entry,
data entry), its length and SHA-256, and, after `damage` (byte ranges
overwritten with zeros) and the reference's repair, the SHA-256 of the
repaired file.  tests/test_par_gpu.py rebuilds the same inputs and checks
libffrs_gb300.par against these records byte for byte.
"""

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

CASES = [
    {"name": "sample.bin", "size": 300000, "seed": 7, "mtime_ns": 1735787045123456789,
     "damage": [[1000, 1400], [150000, 150100]]},
    {"name": "archive part.dat", "size": 4 << 20, "seed": 8, "mtime_ns": 1700000000000000000,
     "damage": [[12345, 20000]]},
    {"name": "tiny.txt", "size": 1000, "seed": 9, "mtime_ns": 1600000000000000001, "damage": [[10, 30]]},
]


def input_bytes(case):
    return np.random.Generator(np.random.PCG64(case["seed"])).integers(0, 256, case["size"], dtype=np.uint8).tobytes()


def damaged(data, case):
    d = bytearray(data)
    for a, b in case["damage"]:
        d[a:b] = bytes(b - a)
    return bytes(d)


def main(ref):
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1",
               PYTHONPATH=os.pathsep.join([os.path.join(REPO, "oracle", "_ref"), ref]))
    out = []
    for case in CASES:
        with tempfile.TemporaryDirectory() as tmp:
            path = os.path.join(tmp, case["name"])
            data = input_bytes(case)
            with open(path, "wb") as f:
                f.write(data)
            os.utime(path, ns=(case["mtime_ns"], case["mtime_ns"]))
            subprocess.run([sys.executable, "-m", "ffrs.par", "backup", case["name"]], cwd=tmp, env=env, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            par = open(path + ".ffrs", "rb").read()
            lines = par.split(b"\n", 4)[:4]
            with open(path, "wb") as f:
                f.write(damaged(data, case))
            os.utime(path, ns=(case["mtime_ns"], case["mtime_ns"]))
            subprocess.run([sys.executable, "-m", "ffrs.par", "repair", case["name"] + ".ffrs"], cwd=tmp, env=env,
                           check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            repaired = open(path, "rb").read()
            rec = dict(case, ffrs_len=len(par), ffrs_sha256=hashlib.sha256(par).hexdigest(),
                       ffrs_header=[ln.decode("latin-1") for ln in lines],
                       repaired_sha256=hashlib.sha256(repaired).hexdigest(),
                       repaired_equals_input=repaired == data)
            out.append(rec)
            print(case["name"], lines[1].decode(), rec["repaired_equals_input"])
    with open(os.path.join(HERE, "ffrs_par.json"), "w") as f:
        json.dump({"generated_by": "tests/golden/make_ffrs_golden.py (the reference's ffrs.par backup / repair)",
                   "cases": out}, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
