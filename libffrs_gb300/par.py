"""Backup and repair of files through `.ffrs` parity files, on the GPU.

The reference's `ffrs.par backup` reads a file into one page-locked buffer
(`create_buffer`), hashes it with BLAKE2b, CIRC16-encodes the buffer and
writes the parity file (ffrs/par/backup.py:30-80, format.Writer in
ffrs/par/format.py:31-107); `ffrs.par repair` reads the parity file back,
reads the file into a buffer, repairs it in place and writes it back with its
modification time kept (ffrs/par/repair.py:84-102, fs.py:206-238).  This
module does the same work with the GPU codec and a pipeline across files:

* a reader thread reads each file into its page-locked buffer in 16 MiB
  pieces, and a hasher thread hashes every piece as soon as it has landed
  (reading and hashing overlap instead of alternating);
* the calling thread encodes a file on the GPU (host-to-device copy, CIRC16
  encode, device-to-host copy of the parity) while the reader and hasher are
  already on the next file, with two buffers in rotation;
* a writer thread writes each parity file once its hash and parity are there,
  and only then hands its buffer back to the reader.

The parity files are byte-identical to the reference's for the same file,
name, modification time and codec (tests/test_par_gpu.py checks this against
the reference's own output).  Choosing the codec for a file size is the
reference CLI's constraint solver (ffrs/par/opt.py); it is not part of this
hot path, so the caller passes the codec, or a function of the file size that
returns one.
"""

import base64
import hashlib
import json
import os
import queue
import re
import shlex
import threading

from . import libffrs

SIGNATURE = b"\x89ffrs\r\n"
PIECE = 16 << 20
_B64HEX = "0123456789abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ-_"


def b64hex(val):
    """The reference's compact integer encoding (ffrs/util.py:34-39): base 64,
    most significant digit first, zero as the empty string."""
    out = ""
    while val:
        out = _B64HEX[val & 0x3F] + out
        val >>= 6
    return out


def b64hex_dec(s):
    val = 0
    for ch in s:
        val = (val << 6) | _B64HEX.index(ch)
    return val


def serialize(codec):
    """The codec line of a parity file (ffrs/__init__.py:43-57)."""
    rsi, rso = codec.rsi, codec.rso
    return (
        "circ16"
        f" ip:{b64hex(rsi.gf.field_elements)} ig:{b64hex(rsi.gf.primitive)} ib:{b64hex(codec.inner_block_len)}"
        f" im:{b64hex(codec.inner_message_len)} ie:{b64hex(codec.inner_ecc_len)}"
        f" op:{b64hex(rso.gf.field_elements)} og:{b64hex(rso.gf.primitive)} ob:{b64hex(codec.outer_block_len)}"
        f" om:{b64hex(codec.outer_message_len)} oe:{b64hex(codec.outer_ecc_len)}"
        f" i:{b64hex(codec.interleave)}"
    ).encode("ascii")


def deserialize(line):
    """CIRC16 from a codec line (ffrs/__init__.py:59-80)."""
    text = line.decode("ascii").strip()
    if not text.startswith("circ16 "):
        raise ValueError("not a circ16 codec line")
    p = {}
    for part in text[7:].split():
        key, value = part.split(":", 1)
        p[key] = b64hex_dec(value)
    if not (p["ip"] == p["op"] == 0x10001 and p["ig"] == p["og"] and p["ib"] == p["im"] + p["ie"]
            and p["ob"] == p["om"] + p["oe"]):
        raise ValueError("inconsistent circ16 codec line")
    return libffrs.CIRC16(inner_block_len=p["ib"], inner_ecc_len=p["ie"], outer_block_len=p["ob"],
                          outer_ecc_len=p["oe"], interleave=p["i"], primitive=p["ig"])


def _quote(s):
    """A path part as the reference writes it: JSON, quotes dropped unless it
    holds whitespace (format.py:50-58)."""
    q = json.dumps(s, ensure_ascii=False)
    return q if re.findall(r"\s", q) else q[1:-1]


def _unquote(s):
    return json.loads(s if s.startswith('"') else f'"{s}"')


def parity_file_bytes(codec, path, size, mtime_ns, digest, ecc):
    """The whole parity file of one file (format.py:31-107: signature, codec
    line, directory line when the path has one, file entry, data)."""
    out = bytearray(SIGNATURE + serialize(codec) + b"\n")
    d, f = os.path.split(path)
    if _quote(d) != "":
        out += f"p p:{_quote(d)}\n".encode("utf8")
    out += f"f s:{b64hex(size)} m:{b64hex(mtime_ns)} h:b2:".encode("ascii")
    out += base64.urlsafe_b64encode(digest).strip(b"=")
    out += f" p:{_quote(f)}\n".encode("utf8")
    out += f"d s:{b64hex(len(ecc))}\n".encode("ascii")
    out += ecc
    out += b"\n"
    return bytes(out)


def read_parity_file(path):
    """(codec, [(size, mtime_ns, blake2b hex, file path)], ecc bytes), read
    as the reference's Reader does (format.py:110-204)."""
    with open(path, "rb") as f:
        if f.readline(16) != SIGNATURE:
            raise ValueError("not a parity file")
        codec = deserialize(f.readline(4096))
        files, cur = [], ""
        while True:
            line = f.readline(4096)
            if not line.endswith(b"\n"):
                raise ValueError("truncated parity file")
            kind, args = line.decode("utf8").split(" ", 1)
            p = {}
            for arg in shlex.split(args):
                k, v = arg.split(":", 1)
                p[k] = v
            path_ = _unquote(p["p"]) if "p" in p else None
            if kind == "p":
                cur = path_
            elif kind == "f":
                algo, h = p["h"].split(":", 1)
                if algo != "b2":
                    raise ValueError("unknown hash")
                files.append((b64hex_dec(p["s"]), b64hex_dec(p["m"]),
                              base64.urlsafe_b64decode(h + "==").hex(), os.path.join(cur, path_)))
            elif kind == "d":
                n = b64hex_dec(p["s"])
                ecc = f.read(n)
                if len(ecc) != n or f.read(1) != b"\n":
                    raise ValueError("truncated parity data")
                return codec, files, ecc
            else:
                raise ValueError("unsupported parity entry " + kind)


def backup(paths, codec, force=False):
    """Writes `path + ".ffrs"` for every file of `paths`, in order.  `codec` is
    a CIRC16, or a function of the file size returning one.  Empty files are
    skipped, as the reference skips them.  Returns the parity file names."""
    paths = list(paths)
    for p in paths:
        if not os.path.isfile(p):
            raise FileNotFoundError(p)
        if os.path.exists(p + ".ffrs") and not force:
            raise FileExistsError(p + ".ffrs")
    jobs = []
    for p in paths:
        st = os.stat(p)
        if st.st_size == 0:
            continue
        c = codec(st.st_size) if callable(codec) else codec
        if c.message_size < st.st_size:
            raise ValueError("%s: %d bytes do not fit the codec's %d-byte message" % (p, st.st_size,
                                                                                     c.message_size))
        jobs.append((p, st.st_size, st.st_mtime_ns, c))
    if not jobs:
        return []

    hash_q, enc_q, write_q, free = queue.Queue(), queue.Queue(), queue.Queue(), queue.Queue()
    stop = threading.Event()
    errors = []
    for _ in range(2):  # two buffers in rotation: reading one while the other is encoded
        free.put(None)

    def reader():
        try:
            for i, (p, size, _, c) in enumerate(jobs):
                buf = free.get()
                if stop.is_set():
                    return
                if buf is None or len(buf) != c.message_size:
                    buf = libffrs.create_buffer(c.message_size)
                mv = memoryview(buf)
                with open(p, "rb") as f:
                    off = 0
                    while off < size:
                        n = f.readinto(mv[off:min(size, off + PIECE)])
                        if not n:
                            raise IOError("%s: file shrank while read" % p)
                        hash_q.put((i, mv[off:off + n]))
                        off += n
                mv[size:] = bytes(c.message_size - size)
                hash_q.put((i, None))
                enc_q.put((i, buf))
        except BaseException as e:  # surfaced by the calling thread
            errors.append(e)
        finally:
            enc_q.put(None)
            hash_q.put(None)

    digests, parities, bufs = {}, {}, {}

    def hasher():
        h = None
        while True:
            item = hash_q.get()
            if item is None:
                return
            i, piece = item
            if h is None:
                h = hashlib.blake2b(digest_size=20, usedforsecurity=False)
            if piece is None:
                digests[i] = h.digest()
                write_q.put(("hash", i))
                h = None
            else:
                h.update(piece)

    def writer():
        try:
            have = {}
            for _ in range(2 * len(jobs)):
                item = write_q.get()
                if item is None:
                    return
                kind, i = item
                have.setdefault(i, set()).add(kind)
                if len(have[i]) == 2:
                    p, size, mtime, c = jobs[i]
                    data = parity_file_bytes(c, p, size, mtime, digests[i], parities.pop(i))
                    # hashed and encoded: the buffer may be read into again
                    free.put(bufs.pop(i))
                    with open(p + ".ffrs", "wb") as f:
                        f.write(data)
        except BaseException as e:
            errors.append(e)

    threads = [threading.Thread(target=t, daemon=True) for t in (reader, hasher, writer)]
    for t in threads:
        t.start()
    try:
        while True:
            item = enc_q.get()
            if item is None:
                break
            i, buf = item
            bufs[i] = buf
            parities[i] = bytes(jobs[i][3].encode(buf))  # the GPU encode of the whole message
            write_q.put(("ecc", i))
    except BaseException:
        stop.set()
        free.put(None)  # wakes the reader if it waits for a buffer
        write_q.put(None)
        raise
    finally:
        threads[0].join()
        threads[1].join()
        if errors:
            write_q.put(None)
        threads[2].join()
    if errors:
        raise errors[0]
    return [p + ".ffrs" for p, *_ in jobs]


def repair(parity_path, base_dir=None):
    """Repairs the file a parity file covers, in place, keeping its
    modification time as the reference does.  Paths in the parity file are
    taken relative to `base_dir` (default: the current directory, as the
    reference).  Returns the repaired file's path."""
    codec, files, ecc = read_parity_file(parity_path)
    if len(files) != 1:
        raise ValueError("a parity file of one file was expected")
    size, mtime_ns, _, path = files[0]
    full = os.path.join(base_dir, path) if base_dir else path
    if os.stat(full).st_size != size:
        raise ValueError("%s: file size differs from the parity file's" % full)
    data = libffrs.create_buffer(codec.message_size)
    mv = memoryview(data)
    with open(full, "rb") as f:
        off = 0
        while off < size:
            n = f.readinto(mv[off:min(size, off + PIECE)])
            if not n:
                raise IOError("%s: file shrank while read" % full)
            off += n
    mv[size:] = bytes(codec.message_size - size)
    ecc_buf = libffrs.create_buffer(codec.ecc_size)
    memoryview(ecc_buf)[:] = ecc
    codec.repair(data, ecc_buf)  # on the GPU, in place
    with open(full, "r+b") as f:
        f.write(mv[:size])
        atime = os.fstat(f.fileno()).st_atime_ns
    os.utime(full, ns=(atime, mtime_ns))
    return full
