"""Calibration of the oracle port against the reference's own build (test and
measurement infrastructure, never on the product path).

The CPU baseline on the GPU machine times the oracle (a C restatement of the
reference path) because the reference's sources do not travel there.  This
script measures, on the machine where oracle/_ref was built from the
reference's sources (oracle/build_ref.sh), how fast the reference's own
extension runs each path against the port, on the same inputs and one pinned
core, and writes oracle/calibration.json.  bench.py reports the ratios next
to its CPU figures, so that a reader knows how far the port over- or
understates the reference.

    python oracle/calibrate.py            # writes oracle/calibration.json

Paths (the reference's own API in each case):
  rs256-encode  RS256(ecc_len=32).encode over 65,536 x 223 bytes
  rs256-decode  RS256.repair, one call per block, 0-16 errors (1% 17-20)
  rsi16-encode  RSi16(1024, 64).encode, default SIMD dispatch and W = 1
  rsi16-decode  RSi16.repair, one call per block (W = 1), 0-32 errors
"""

import json
import os
import platform
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
# run as a script, this directory would shadow the oracle package
sys.path = [p for p in sys.path if os.path.abspath(p or ".") != HERE]


def _inputs(which):
    rng = np.random.Generator(np.random.PCG64(20261204))
    if which == "rs256-encode":
        return {"data": rng.integers(0, 256, size=(65536, 223), dtype=np.uint8)}
    if which == "rs256-decode":
        nb = 8192
        return {"data": rng.integers(0, 256, size=(nb, 223), dtype=np.uint8),
                "k": np.where(rng.random(nb) < 0.01, rng.integers(17, 21, nb), rng.integers(0, 17, nb)),
                "keys": rng.random((nb, 255), dtype=np.float32),
                "vals": rng.integers(1, 256, size=(nb, 20), dtype=np.uint8)}
    if which == "rsi16-encode":
        return {"msg": rng.integers(0, 65536, size=(8192, 960), dtype=np.uint16)}
    nb = 512
    return {"msg": rng.integers(0, 65536, size=(nb, 960), dtype=np.uint16), "k": rng.integers(0, 33, nb),
            "keys": rng.random((nb, 1024), dtype=np.float32), "d": rng.integers(1, 65537, size=(nb, 32))}


def _corrupt_rs256(inp, par):
    cw = np.concatenate([inp["data"], par], axis=1)
    pos = np.argsort(inp["keys"], axis=1)[:, :20]
    vals = inp["vals"] * (np.arange(20)[None, :] < inp["k"][:, None])
    rows = np.repeat(np.arange(cw.shape[0])[:, None], 20, axis=1)
    cw[rows, pos] ^= vals.astype(np.uint8)
    return cw


def _corrupt_rsi16(inp, par):
    cw = np.concatenate([inp["msg"], par], axis=1).astype(np.int64)
    pos = np.argsort(inp["keys"], axis=1)[:, :32]
    rows = np.repeat(np.arange(cw.shape[0])[:, None], 32, axis=1)
    v = cw[rows, pos]
    d = inp["d"]
    nv = (v + d) % 65537
    nv = np.where(nv == 65536, np.where(d > 1, (v + d - 1) % 65537, (v + 2) % 65537), nv)
    cw[rows, pos] = np.where(np.arange(32)[None, :] < inp["k"][:, None], nv, v)
    return cw


def _best(fn, reps=3):
    best = 1e30
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def _run_port(which):
    sys.path.insert(0, REPO)
    from oracle import oracle as O

    inp = _inputs(which)
    if which == "rs256-encode":
        o = O.RS256(32)
        d = inp["data"]
        return d.shape[0] * 255, _best(lambda: o.encode_blocks(d, threads=1))
    if which == "rs256-decode":
        o = O.RS256(32)
        cw = _corrupt_rs256(inp, o.encode_blocks(inp["data"], threads=8))

        def run():
            o.decode_blocks(np.ascontiguousarray(cw[:, :223]), np.ascontiguousarray(cw[:, 223:]), threads=1)
        return cw.shape[0] * 256, _best(run)
    if which == "rsi16-encode":
        o = O.RSi16(1024, 64)
        m = inp["msg"]
        return m.shape[0] * 2048, _best(lambda: o.encode_blocks(m, threads=1))
    o = O.RSi16(1024, 64)
    cw = _corrupt_rsi16(inp, o.encode_blocks(inp["msg"], threads=8))

    def run():
        o.repair_blocks(np.ascontiguousarray(cw[:, :960].astype(np.uint16)),
                        np.ascontiguousarray(cw[:, 960:].astype(np.uint16)), threads=1)
    return cw.shape[0] * 2052, _best(run, 2)


def _run_ref(which, simd):
    sys.path.insert(0, os.path.join(HERE, "_ref"))
    import libffrs as R  # the reference's own extension, built from its sources

    inp = _inputs(which)
    if which == "rs256-encode":
        rs = R.RS256(ecc_len=32)
        buf = inp["data"].tobytes()
        return len(buf) // 223 * 255, _best(lambda: rs.encode(buf))
    if which == "rs256-decode":
        rs = R.RS256(ecc_len=32)
        par = np.frombuffer(bytes(rs.encode(inp["data"].tobytes())), np.uint8).reshape(-1, 32)
        cw = _corrupt_rs256(inp, par.copy())
        blocks = [(bytearray(cw[i, :223].tobytes()), bytearray(cw[i, 223:].tobytes())) for i in range(cw.shape[0])]

        def run():
            for d, p in blocks:
                rs.repair(bytearray(d), bytearray(p))
        return cw.shape[0] * 256, _best(run)
    kw = {} if simd else {"simd_x4": False, "simd_x8": False, "simd_x16": False}
    rs = R.RSi16(1024, 64, **kw)
    if which == "rsi16-encode":
        buf = inp["msg"].tobytes()
        return inp["msg"].shape[0] * 2048, _best(lambda: rs.encode(buf))
    par = np.frombuffer(bytes(R.RSi16(1024, 64).encode(inp["msg"].tobytes())), np.uint16).reshape(-1, 64)
    cw = _corrupt_rsi16(inp, par.copy())
    blocks = [(cw[i, :960].astype(np.uint16).tobytes(), cw[i, 960:].astype(np.uint16).tobytes())
              for i in range(cw.shape[0])]

    def run():
        for m, e in blocks:
            rs.repair(bytearray(m), bytearray(e))
    return cw.shape[0] * 2052, _best(run, 2)


def _child(args):
    os.sched_setaffinity(0, {0})
    kind, which = args[0], args[1]
    if kind == "port":
        nbytes, sec = _run_port(which)
    else:
        nbytes, sec = _run_ref(which, kind == "ref-simd")
    print(json.dumps({"bytes": nbytes, "seconds": sec}))


def _measure(kind, which):
    env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1", OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--child", kind, which], env=env,
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, check=True)
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return d["bytes"] / d["seconds"] / 1e6


def main():
    if not any(f.startswith("libffrs") for f in os.listdir(os.path.join(HERE, "_ref"))):
        raise SystemExit("oracle/_ref is not built (oracle/build_ref.sh)")
    cpu = platform.processor() or platform.machine()
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.startswith("model name"):
                cpu = ln.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    out = {"what": "MB/s of algorithmic bytes on one pinned core; reference = the reference's own extension built "
                   "from its sources (oracle/build_ref.sh), port = the oracle's C restatement",
           "cpu": cpu, "machine": platform.machine(), "when": time.strftime("%Y-%m-%d"), "paths": {}}
    for which in ("rs256-encode", "rs256-decode", "rsi16-encode", "rsi16-decode"):
        port = _measure("port", which)
        ref = _measure("ref-scalar", which)
        rec = {"port_mbs": port, "reference_mbs": ref, "reference_over_port": ref / port}
        if which.startswith("rsi16"):
            simd = _measure("ref-simd", which)
            rec.update(reference_simd_mbs=simd, reference_simd_over_port=simd / port)
        out["paths"][which] = rec
        print(which, json.dumps(rec))
    with open(os.path.join(HERE, "calibration.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--child":
        _child(sys.argv[2:])
    else:
        main()
