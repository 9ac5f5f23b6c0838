"""Generate the golden fixtures in tests/golden/ with the reference itself.

Run in a container that has the reference sources and the reference extension
built by oracle/build_ref.sh:

    oracle/build_ref.sh /root/reference
    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /root/reference

Inputs are drawn from numpy PCG64 with fixed seeds; every output is produced by
the reference's own pybind11 module (W = 1 SIMD width for RSi16/CIRC16 repair,
i.e. simd_x4/x8/x16 all False).  The fixtures are small .npz files committed
beside this script; nothing at test time reads the reference.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _import_reference(ref_root):
    sys.path.insert(0, os.path.join(REPO, "oracle", "_ref"))
    sys.path.insert(0, ref_root)
    import libffrs  # noqa: F401  (the reference build)
    import ffrs

    assert "oracle/_ref" in libffrs.__file__, libffrs.__file__
    return ffrs


def corrupt_bytes(rng, cw, k):
    pos = rng.choice(cw.size, size=min(k, cw.size), replace=False)
    cw[pos] ^= rng.integers(1, 256, size=pos.size, dtype=np.uint8)
    return cw


def corrupt_words(rng, cw, k):
    """k distinct symbol errors (v + d) mod 65537 with d in [1, 65536],
    resampled while the result is 65536 (not storable in 16 bits)."""
    pos = rng.choice(cw.size, size=min(k, cw.size), replace=False)
    for p in pos:
        while True:
            d = int(rng.integers(1, 65537))
            v = (int(cw[p]) + d) % 65537
            if v != 65536:
                break
        cw[p] = v
    return cw


def gen_rs256(ffrs, out):
    rng = np.random.Generator(np.random.PCG64(0x5256))
    cases = []
    for ecc in [1, 2, 3, 4, 7, 8, 16, 17, 31, 32, 33, 64, 128, 254]:
        for bl in sorted({255, min(255, ecc + 1 + (ecc % 7) * 13), ecc + 1}):
            if bl <= ecc:
                continue
            cases.append((ecc, bl))
    d = {}
    for ci, (ecc, bl) in enumerate(cases):
        rs = ffrs.RS256(bl, ecc_len=ecc)
        ml = bl - ecc
        nb = 24
        msgs = rng.integers(0, 256, size=(nb, ml), dtype=np.uint8)
        tail = rng.integers(0, 256, size=int(rng.integers(1, ml + 1)), dtype=np.uint8)
        buf = np.concatenate([msgs.reshape(-1), tail])
        par_all = np.frombuffer(bytes(rs.encode(bytearray(buf.tobytes()))), np.uint8)
        parity = par_all[: nb * ecc].reshape(nb, ecc)
        # repairs: error counts spread over [0, ecc/2 + 3]
        cw = np.concatenate([msgs, parity], axis=1).copy()
        ks = np.array([int(rng.integers(0, ecc // 2 + 4)) for _ in range(nb)])
        for i in range(nb):
            corrupt_bytes(rng, cw[i], int(ks[i]))
        rdata, rpar = cw[:, :ml].copy(), cw[:, ml:].copy()
        status = np.zeros(nb, np.uint8)
        synds = np.zeros((nb, ecc), np.uint8)
        for i in range(nb):
            synds[i] = np.frombuffer(bytes(rs._synds(bytearray(cw[i].tobytes()))), np.uint8)
            m = bytearray(rdata[i].tobytes())
            e = bytearray(rpar[i].tobytes())
            status[i] = 1 if rs.repair(m, e) else 0
            rdata[i] = np.frombuffer(bytes(m), np.uint8)
            rpar[i] = np.frombuffer(bytes(e), np.uint8)
        p = f"c{ci}_"
        d[p + "geom"] = np.array([ecc, bl])
        d[p + "generator"] = np.frombuffer(bytes(rs.generator), np.uint8)
        d[p + "buffer"] = buf
        d[p + "encoded"] = par_all
        d[p + "received_data"] = cw[:, :ml].copy()
        d[p + "received_parity"] = cw[:, ml:].copy()
        d[p + "synds"] = synds
        d[p + "status"] = status
        d[p + "repaired_data"] = rdata
        d[p + "repaired_parity"] = rpar
    d["ncases"] = np.array([len(cases)])
    np.savez_compressed(out, **d)


def gen_rsi16(ffrs, out):
    rng = np.random.Generator(np.random.PCG64(0x16161))
    geoms = [(4, 2), (8, 2), (16, 4), (16, 8), (128, 2), (256, 32), (208, 8), (768, 8), (1024, 64), (4096, 256),
             (2048, 128), (512, 128)]
    d = {}
    for gi, (bl, ecc) in enumerate(geoms):
        rs = ffrs.RSi16(bl, ecc, simd_x4=False, simd_x8=False, simd_x16=False)
        ml = bl - ecc
        nb = 16 if bl <= 1024 else 6
        msgs = rng.integers(0, 65536, size=(nb, ml), dtype=np.uint16)
        par = np.frombuffer(bytes(rs.encode(bytearray(msgs.tobytes()))), np.uint16).reshape(nb, ecc)
        cw = np.concatenate([msgs, par], axis=1).copy()
        ks = np.array([int(rng.integers(0, ecc // 2 + 3)) for _ in range(nb)])
        for i in range(nb):
            corrupt_words(rng, cw[i], int(ks[i]))
        rdata, rpar = cw[:, :ml].copy(), cw[:, ml:].copy()
        status = np.zeros(nb, np.int16)
        synd = np.zeros((nb, ecc), np.uint32)
        loc = np.zeros((nb, ecc), np.uint32)
        ev = np.zeros((nb, ecc), np.uint32)
        for i in range(nb):
            m = bytearray(rdata[i].tobytes())
            e = bytearray(rpar[i].tobytes())
            synd[i] = np.array(rs._synd(m, e), np.uint32)
            try:
                a, b = rs._sugiyama(list(map(int, synd[i])))
                loc[i], ev[i] = a, b
            except RuntimeError:
                loc[i] = 0xFFFFFFFF
            try:
                status[i] = int(rs.repair(m, e))
            except RuntimeError:
                status[i] = -1
            rdata[i] = np.frombuffer(bytes(m), np.uint16)
            rpar[i] = np.frombuffer(bytes(e), np.uint16)
        # known-location repairs
        kcw = np.concatenate([msgs, par], axis=1).copy()
        kpos = np.zeros((nb, ecc), np.int64) - 1
        for i in range(nb):
            k = int(rng.integers(1, ecc + 1))
            pos = rng.choice(bl, size=k, replace=False)
            kcw[i, pos] = rng.integers(0, 65536, size=k, dtype=np.uint16)
            kpos[i, :k] = pos
        kdata, kpar = kcw[:, :ml].copy(), kcw[:, ml:].copy()
        kstatus = np.zeros(nb, np.int16)
        for i in range(nb):
            m = bytearray(kdata[i].tobytes())
            e = bytearray(kpar[i].tobytes())
            kstatus[i] = int(rs.repair(m, e, [int(x) for x in kpos[i] if x >= 0]))
            kdata[i] = np.frombuffer(bytes(m), np.uint16)
            kpar[i] = np.frombuffer(bytes(e), np.uint16)
        p = f"g{gi}_"
        d[p + "geom"] = np.array([bl, ecc, rs.root, rs.ntt_len])
        d[p + "msgs"] = msgs
        d[p + "parity"] = par
        d[p + "received"] = cw
        d[p + "synd"] = synd
        d[p + "locator"] = loc
        d[p + "evaluator"] = ev
        d[p + "status"] = status
        d[p + "repaired_data"] = rdata
        d[p + "repaired_parity"] = rpar
        d[p + "known_received"] = kcw
        d[p + "known_pos"] = kpos
        d[p + "known_status"] = kstatus
        d[p + "known_data"] = kdata
        d[p + "known_parity"] = kpar
    d["ngeoms"] = np.array([len(geoms)])
    np.savez_compressed(out, **d)


def gen_circ16(ffrs, out):
    rng = np.random.Generator(np.random.PCG64(0xC16))
    geoms = [(8, 2, 8, 2, 1), (16, 4, 16, 4, 1), (32, 16, 4, 2, 1), (128, 8, 128, 8, 1), (128, 2, 32, 2, 6),
             (64, 4, 32, 8, 4), (128, 8, 128, 8, 3), (100, 2, 100, 2, 3), (52, 2, 192, 64, 7), (12, 2, 24, 2, 1)]
    d = {}
    for gi, g in enumerate(geoms):
        c = ffrs.CIRC16(*g, simd_x4=False, simd_x8=False, simd_x16=False)
        msg = rng.integers(0, 65536, size=c.message_len, dtype=np.uint16)
        ecc = np.frombuffer(bytes(c.encode(bytearray(msg.tobytes()))), np.uint16).copy()
        cases_m, cases_e, out_m, out_e, rc = [], [], [], [], []
        for trial in range(3):
            m = msg.copy()
            e = ecc.copy()
            nrows = int(rng.integers(1, c.outer_ecc_len + 1)) if trial < 2 else c.outer_ecc_len + 1
            for row in rng.choice(c.outer_block_len, size=min(nrows, c.outer_block_len), replace=False):
                k = int(rng.integers(0, c.interleave))
                if row < c.outer_message_len:
                    for col in range(c.inner_message_len):
                        m[c.message_offset(k, int(row), col)] ^= int(rng.integers(1, 65536))
                else:
                    for col in range(c.inner_message_len):
                        e[c.rso_ecc_offset(k, int(row) - c.outer_message_len, col)] ^= int(rng.integers(1, 65536))
            if trial == 1:
                zpos = rng.choice(e.size, size=min(12, e.size), replace=False)
                e[zpos] = 0
            cases_m.append(m.copy())
            cases_e.append(e.copy())
            mb, eb = bytearray(m.tobytes()), bytearray(e.tobytes())
            try:
                c.repair(mb, eb)
                rc.append(0)
            except RuntimeError:
                rc.append(-1)
            out_m.append(np.frombuffer(bytes(mb), np.uint16).copy())
            out_e.append(np.frombuffer(bytes(eb), np.uint16).copy())
        p = f"g{gi}_"
        d[p + "geom"] = np.array(g)
        d[p + "msg"] = msg
        d[p + "ecc"] = ecc
        d[p + "recv_msg"] = np.stack(cases_m)
        d[p + "recv_ecc"] = np.stack(cases_e)
        d[p + "rep_msg"] = np.stack(out_m)
        d[p + "rep_ecc"] = np.stack(out_e)
        d[p + "rc"] = np.array(rc)
    d["ngeoms"] = np.array([len(geoms)])
    np.savez_compressed(out, **d)


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    ffrs = _import_reference(ref_root)
    gen_rs256(ffrs, os.path.join(HERE, "rs256.npz"))
    gen_rsi16(ffrs, os.path.join(HERE, "rsi16.npz"))
    gen_circ16(ffrs, os.path.join(HERE, "circ16.npz"))
    for f in ("rs256.npz", "rsi16.npz", "circ16.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
