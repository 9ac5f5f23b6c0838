"""Benchmark of the GB300 block-coding path: RS256, RSi16 and CIRC16 encode and
decode, the mixed batch and the serving loop.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload all|rs256-decode|rs256-encode|rsi16-encode|rsi16-decode|batch-mixed|serving]

One JSON line is printed by rank 0.  With the default --workload all, its top
level is the headline workload -- RS256 decode with errors: ecc_len 32,
1,048,576 blocks of 223 + 32 bytes, per block 0-16 byte errors at distinct
positions, 1% of the blocks 17-20 -- and "workloads" holds one record per
other configuration (RS256 encode of 65,536 blocks, RSi16(1024, 64) encode
and decode of 262,144 blocks, the 1 GiB mixed batch against the plain
per-request path, the serving loop with p50/p99), each with its own
roofline, CPU baseline and parity check, timed under the same clock record.

`value` is GB/s of algorithmic bytes with inputs resident in HBM (CUDA events
on the launching stream); `e2e` is the same metric through the public
``libffrs`` API on host buffers, copies inside the timed region; `roofline`
relates the dominant kernel (per-launch CUDA events) to the measured HBM copy
bandwidth; `cpu_baseline` times the oracle (a C restatement of the reference
path) on the host cores -- all threads, one core, and one pinned process per
core -- beside the measured speed of the reference's own build relative to
the oracle; `parity` compares the GPU outputs of the timed workload with the
oracle on the same seeded inputs.  All inputs are seeded numpy PCG64 draws,
generated in chunks so that any range of blocks regenerates identically on
the CPU side.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

L2_BYTES = 129 * 1024 * 1024
P16 = 65537


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(workload):
    """dram bytes per launch of the dominant kernel from the committed ncu summary."""
    p = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(p):
        d = json.load(open(p))
        v = d.get(workload)
        if v:
            return v
    return None


def load_calibration(path):
    """The reference's own build against the oracle on one core of the machine
    that built it (oracle/calibrate.py), for the CPU baseline's path."""
    p = os.path.join(REPO, "oracle", "calibration.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    rec = d.get("paths", {}).get(path)
    if not rec:
        return None
    out = {"reference_over_oracle": round(rec["reference_over_port"], 3),
           "measured_on": "%s (%s), one pinned core" % (d.get("cpu"), d.get("machine")), "path": path}
    if "reference_simd_over_port" in rec:
        out["reference_simd_over_oracle"] = round(rec["reference_simd_over_port"], 3)
        out["note"] = "the reference's x86 SIMD build is not available on an aarch64 host"
    return out


class ClockSampler:
    """SM clock and clock-event reasons sampled during the timed region.

    Uses NVML through ctypes (libnvidia-ml ships with the driver) every
    millisecond, so that even a region of a few milliseconds gets samples;
    falls back to `nvidia-smi -lms 100` when NVML cannot be opened."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}
    Q = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.samples = []  # (sm_mhz, reasons bitmask)
        self.max_mhz = None
        self.nvml = None
        self.stop = threading.Event()

    def _open_nvml(self):
        import ctypes

        try:
            L = ctypes.CDLL("libnvidia-ml.so.1")
        except OSError:
            return False
        if L.nvmlInit_v2() != 0:
            return False
        h = ctypes.c_void_p()
        bus = None
        try:
            import torch

            pr = torch.cuda.get_device_properties(self.index)
            bus = "%08x:%02x:%02x.0" % (getattr(pr, "pci_domain_id", 0), pr.pci_bus_id, pr.pci_device_id)
        except Exception:
            bus = None
        ok = bus is not None and L.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(h)) == 0
        if not ok and L.nvmlDeviceGetHandleByIndex_v2(self.index, ctypes.byref(h)) != 0:
            return False
        mx = ctypes.c_uint()
        if L.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:
            self.max_mhz = float(mx.value)
        self.reason_fn = getattr(L, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(L, "nvmlDeviceGetCurrentClocksThrottleReasons")
        self.nvml, self.handle = L, h
        return True

    def _poll_nvml(self):
        import ctypes

        clk = ctypes.c_uint()
        rs = ctypes.c_ulonglong()
        while not self.stop.is_set():
            if self.nvml.nvmlDeviceGetClockInfo(self.handle, 1, ctypes.byref(clk)) == 0:
                r = rs.value if self.reason_fn(self.handle, ctypes.byref(rs)) == 0 else 0
                self.samples.append((float(clk.value), r))
            time.sleep(0.001)

    def __enter__(self):
        try:
            if self._open_nvml():
                self.t = threading.Thread(target=self._poll_nvml, daemon=True)
                self.t.start()
                return self
        except Exception:
            self.nvml = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        self.stop.set()
        if self.nvml is not None:
            self.t.join(timeout=2)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None:
            sm = [c for c, _ in self.samples]
            reasons = set()
            for _, r in self.samples:
                for bit, name in self.REASONS.items():
                    if r & bit:
                        reasons.add(name)
            return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.max_mhz,
                    "reasons": sorted(reasons), "samples": len(sm), "source": "nvml"}
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi"}


# ---------------------------------------------------------------- seeded inputs
#
# Every workload draws its inputs from numpy PCG64 streams seeded per chunk of
# blocks ([seed, chunk index]), so that any chunk regenerates identically: on
# the GPU arm's host, in the CPU legs and in the pinned CPU worker processes.

RS_CHUNK = 65536
RSI_CHUNK = 16384


def _rng(seed, c):
    return np.random.Generator(np.random.PCG64([seed, c]))


def _first_k_of(keys, k):
    """indices of the k smallest keys per row, in increasing key order: the
    first j of them are a uniform random j-subset for every j <= k"""
    part = np.argpartition(keys, k - 1, axis=1)[:, :k]
    order = np.argsort(np.take_along_axis(keys, part, axis=1), axis=1)
    return np.take_along_axis(part, order, axis=1)


def rs256_decode_chunk(seed, c, n):
    """RS256 decode-with-errors chunk c (n blocks): data [n, 223] uint8; per
    block k ~ U[0, 16] errors (1% of the blocks U[17, 20]) at distinct uniform
    positions of the 255-byte codeword, each XORed with a uniform nonzero byte:
    pos [n, 20] and vals [n, 20] (vals 0 past the block's k)."""
    rng = _rng(seed, c)
    data = rng.integers(0, 256, size=(n, 223), dtype=np.uint8)
    k = rng.integers(0, 17, size=n)
    heavy = rng.random(n) < 0.01
    k[heavy] = rng.integers(17, 21, size=int(heavy.sum()))
    pos = _first_k_of(rng.random((n, 255), dtype=np.float32), 20).astype(np.uint8)
    vals = rng.integers(1, 256, size=(n, 20), dtype=np.uint8)
    vals *= (np.arange(20)[None, :] < k[:, None]).astype(np.uint8)
    return data, pos, vals


def rs256_encode_chunk(seed, c, n):
    return _rng(seed, c).integers(0, 256, size=(n, 223), dtype=np.uint8)


def rsi16_chunk(seed, c, n, corrupt):
    """RSi16(1024, 64) chunk c: messages [n, 960] uint16; with corrupt, per
    block k ~ U[0, 32] symbol errors at distinct uniform positions of the
    1024-word codeword, word v -> (v + d) mod 65537 with d ~ U[1, 65536]:
    pos [n, 32] and d [n, 32] (d 0 past the block's k)."""
    rng = _rng(seed, c)
    msg = rng.integers(0, 65536, size=(n, 960), dtype=np.uint16)
    if not corrupt:
        return msg, None, None
    k = rng.integers(0, 33, size=n)
    pos = _first_k_of(rng.random((n, 1024), dtype=np.float32), 32).astype(np.int16)
    d = rng.integers(1, 65537, size=(n, 32)).astype(np.int32)
    d *= (np.arange(32)[None, :] < k[:, None]).astype(np.int32)
    return msg, pos, d


def chunks(fn, seed, nblocks, chunk, first_chunk=0, **kw):
    """fn's outputs for blocks [first_chunk * chunk, + nblocks), concatenated"""
    parts = []
    c = first_chunk
    left = nblocks
    while left > 0:
        n = min(chunk, left)
        parts.append(fn(seed, c, n, **kw))
        left -= n
        c += 1
    if isinstance(parts[0], tuple):
        return tuple(None if parts[0][i] is None else np.concatenate([p[i] for p in parts])
                     for i in range(len(parts[0])))
    return np.concatenate(parts)


def rs256_apply_errors(cw, pos, vals):
    """in place on uint8 codewords [n, 255]"""
    rows = np.arange(cw.shape[0])[:, None]
    cw[rows, pos.astype(np.int64)] ^= vals


def rsi16_new_words(v, d):
    """(v + d) mod 65537, where that would be 65536 (not storable as a uint16
    word) d - 1 instead (d > 1) or 2 (d = 1); v where d = 0"""
    nv = (v + d) % P16
    alt = np.where(d > 1, (v + d - 1) % P16, (v + 2) % P16)
    nv = np.where(nv == 65536, alt, nv)
    return np.where(d > 0, nv, v)


def rsi16_apply_errors(cw, pos, d):
    """in place on int64 codeword words [n, 1024]"""
    rows = np.arange(cw.shape[0])[:, None]
    p = pos.astype(np.int64)
    cw[rows, p] = rsi16_new_words(cw[rows, p], d.astype(np.int64))


def torch_rs256_apply_errors(torch, cw, pos_h, vals_h, step=1 << 18):
    """rs256_apply_errors on a device tensor, the same pattern"""
    for s in range(0, cw.shape[0], step):
        e = min(cw.shape[0], s + step)
        pos = torch.from_numpy(pos_h[s:e].astype(np.int64)).cuda()
        vals = torch.from_numpy(vals_h[s:e]).cuda()
        rows = torch.arange(s, e, device="cuda")[:, None].expand(e - s, pos.shape[1])
        cw[rows, pos] ^= vals


def torch_rsi16_apply_errors(torch, cw, pos_h, d_h, step=1 << 15):
    """rsi16_apply_errors on a device int16 tensor [n, 1024], the same rule"""
    for s in range(0, cw.shape[0], step):
        e = min(cw.shape[0], s + step)
        pos = torch.from_numpy(pos_h[s:e].astype(np.int64)).cuda()
        d = torch.from_numpy(d_h[s:e].astype(np.int64)).cuda()
        rows = torch.arange(s, e, device="cuda")[:, None].expand(e - s, pos.shape[1])
        v = cw[rows, pos].to(torch.int64) & 0xFFFF
        nv = (v + d) % P16
        alt = torch.where(d > 1, (v + d - 1) % P16, (v + 2) % P16)
        nv = torch.where(nv == 65536, alt, nv)
        nv = torch.where(d > 0, nv, v)
        cw[rows, pos] = nv.to(torch.int32).to(torch.int16)


# ---------------------------------------------------------------- GPU arms

class TimedRange:
    """An NVTX range named "timed" around a timed region, so that a profiler
    can be restricted to it (ncu --nvtx --nvtx-include timed/)."""

    def __init__(self, torch):
        self.nvtx = torch.cuda.nvtx

    def __enter__(self):
        self.nvtx.range_push("timed")
        return self

    def __exit__(self, *exc):
        self.nvtx.range_pop()


def timed_steps(torch, args, world, run, restore, nbuf):
    """K timed steps over nbuf rotating buffers: buffer j is restored (when
    `restore` is given) in an untimed gap before each batch of nbuf steps;
    CUDA events on the launching stream around every step."""
    from libffrs_gb300 import capi

    stream = torch.cuda.current_stream()
    for i in range(args.warmup):
        if restore:
            restore(i % nbuf)
        run(i % nbuf)
    torch.cuda.synchronize()
    total_ms, kern_ms = 0.0, []
    launches0 = capi.kernel_launches()
    capi.timing_collect()
    capi.timing_enable(True)
    with ClockSampler(torch.cuda.current_device()) as clk, TimedRange(torch):
        done = 0
        while done < args.steps:
            batch = min(nbuf, args.steps - done)
            if restore:
                for j in range(batch):
                    restore(j)
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(batch + 1)]
            ev[0].record(stream)
            for j in range(batch):
                run(j)
                ev[j + 1].record(stream)
            torch.cuda.synchronize()
            total_ms += ev[0].elapsed_time(ev[batch])
            kern_ms += [ev[j].elapsed_time(ev[j + 1]) for j in range(batch)]
            done += batch
    launches = capi.kernel_launches() - launches0
    kernels = capi.timing_collect()
    capi.timing_enable(False)
    return {"total_ms": total_ms, "kern_ms": kern_ms, "launches": launches, "kernels": kernels,
            "clocks": clk.summary()}


def e2e_median(args, fn, prep=None):
    ts = []
    for i in range(0 if args.no_e2e else max(1, args.e2e_steps) + 1):
        if prep:
            prep()
        t0 = time.perf_counter()
        fn()
        t1 = time.perf_counter()
        if i:
            ts.append(t1 - t0)
    return statistics.median(ts) if ts else None


def bench_rs256_decode(args, torch, rank, world):
    from libffrs_gb300 import capi
    import libffrs_gb300

    nb, ml, ecc = args.blocks or (1 << 20), 223, 32
    seed = 1000 + rank
    data_h, pos_h, vals_h = chunks(rs256_decode_chunk, seed, nb, RS_CHUNK)
    sp = torch.cuda.current_stream().cuda_stream
    code = capi.RS256Code(ecc)
    if args.table_only:  # the per-thread table decoder instead of the bitsliced kernels
        code.set_table_only(True)
    data = torch.from_numpy(data_h).cuda()
    par = torch.zeros((nb, ecc), dtype=torch.uint8, device="cuda")
    code.encode(data.data_ptr(), nb, ml, par.data_ptr(), sp)
    cw = torch.cat([data, par], dim=1)
    torch_rs256_apply_errors(torch, cw, pos_h, vals_h)
    data0, par0 = cw[:, :ml].contiguous(), cw[:, ml:].contiguous()
    del cw, data
    nbuf = max(1, min(args.steps, 4))
    bufs = [(data0.clone(), par0.clone(), torch.zeros(nb, dtype=torch.uint8, device="cuda")) for _ in range(nbuf)]

    def restore(j):
        bufs[j][0].copy_(data0)
        bufs[j][1].copy_(par0)

    def run(j):
        d, p, s = bufs[j]
        code.decode(d.data_ptr(), p.data_ptr(), nb, ml, s.data_ptr(), sp)

    t = timed_steps(torch, args, world, run, restore, nbuf)
    S = min(nb, args.sample_rs256_decode)
    d, p, s = bufs[0]
    gpu = {"par_clean": par[:S].cpu().numpy(), "data": d[:S].cpu().numpy(), "parity": p[:S].cpu().numpy(),
           "status": s[:S].cpu().numpy(), "blocks": S, "seed": seed}
    # e2e through the public API on page-locked host buffers
    lf = libffrs_gb300.libffrs
    rs = lf.RS256(ecc_len=32)
    hd, hp = lf.create_buffer(nb * ml), lf.create_buffer(nb * ecc)
    d0, p0 = data0.cpu().numpy().tobytes(), par0.cpu().numpy().tobytes()
    st_h = []

    def prep():
        hd[:] = d0
        hp[:] = p0

    def call():
        st_h[:] = [rs.repair_blocks(hd, hp)]

    sec = e2e_median(args, call, prep)
    e2e_same = None
    if st_h:
        e2e_same = bool(np.array_equal(np.frombuffer(bytes(st_h[0]), np.uint8), s.cpu().numpy()) and
                        np.array_equal(np.frombuffer(hd, np.uint8), d.cpu().numpy().reshape(-1)) and
                        np.array_equal(np.frombuffer(hp, np.uint8), p.cpu().numpy().reshape(-1)))
    algo = nb * 256  # read 255 B + write 1 B status per block
    return dict(t, workload="rs256-decode", algo_bytes_per_step=algo, gpu=gpu, dtype="u8",
                e2e={"value": algo * world / sec / 1e9 if sec else None, "unit": "GB/s",
                     "h2d_bytes_per_step": nb * (ml + ecc), "d2h_bytes_per_step": rs_e2e_d2h_bytes(nb, ml, ecc),
                     "api": "libffrs.RS256.repair_blocks(create_buffer, create_buffer)",
                     "same_bytes_as_device_path": e2e_same},
                config={"workload": "RS256 decode ecc_len=32, 1048576 blocks x (223+32) B, 0-16 errors/block, "
                                    "1% 17-20 errors", "blocks": nb, "message_len": ml, "ecc_len": ecc,
                        "decoder": "per-thread table decoder" if args.table_only else "bitsliced",
                        "l2": "inputs larger than L2 (268 MB per step; %d rotating buffers)" % nbuf},
                status_ok_fraction=float(s.float().mean().item()))


def rs_e2e_d2h_bytes(nb, ml, ecc):
    """bytes the host repair path copies back per call: statuses plus what
    the library reports (every byte of data and parity, or the correction
    lists when it returns those)"""
    from libffrs_gb300 import capi

    return capi.rs256_host_d2h_bytes(nb, ml, ecc) if hasattr(capi, "rs256_host_d2h_bytes") else nb * (ml + ecc) + nb


def bench_rs256_encode(args, torch, rank, world):
    from libffrs_gb300 import capi
    import libffrs_gb300

    nb, ml, ecc = args.blocks or 65536, 223, 32
    nbuf = 10  # 10 x 16.7 MB rotating inputs > L2
    seed = 2000 + rank
    ins_h = [rs256_encode_chunk(seed, b, nb) for b in range(nbuf)]
    ins = [torch.from_numpy(x).cuda() for x in ins_h]
    outs = [torch.zeros((nb, ecc), dtype=torch.uint8, device="cuda") for _ in range(nbuf)]
    code = capi.RS256Code(ecc)
    sp = torch.cuda.current_stream().cuda_stream

    def run(j):
        code.encode(ins[j].data_ptr(), nb, ml, outs[j].data_ptr(), sp)

    t = timed_steps(torch, args, world, run, None, nbuf)
    gpu = {"parity": outs[0].cpu().numpy(), "blocks": nb, "seed": seed}
    lf = libffrs_gb300.libffrs
    rs = lf.RS256(ecc_len=32)
    hb = lf.create_buffer(nb * ml)
    hb[:] = ins_h[0].tobytes()
    got = []
    sec = e2e_median(args, lambda: got.__setitem__(slice(None), [rs.encode(hb)]))
    algo = nb * 255
    return dict(t, workload="rs256-encode", algo_bytes_per_step=algo, gpu=gpu, dtype="u8",
                e2e={"value": algo * world / sec / 1e9 if sec else None, "unit": "GB/s",
                     "h2d_bytes_per_step": nb * ml, "d2h_bytes_per_step": nb * ecc, "api": "libffrs.RS256.encode",
                     "same_bytes_as_device_path": bool(got) and bytes(got[0]) == gpu["parity"].tobytes()},
                config={"workload": "RS256 encode ecc_len=32, 65536 blocks x 223 B", "blocks": nb,
                        "l2": "10 rotating 16.7 MB inputs (167 MB > L2)"})


def bench_rsi16(args, torch, rank, world, decode):
    from libffrs_gb300 import capi
    import libffrs_gb300

    nb, bl, ecc = args.blocks or 262144, 1024, 64
    ml = bl - ecc
    seed = (3100 if decode else 3000) + rank
    msg_h, pos_h, d_h = chunks(rsi16_chunk, seed, nb, RSI_CHUNK, corrupt=decode)
    code = capi.RSi16Code(bl, ecc)
    sp = torch.cuda.current_stream().cuda_stream
    msg0 = torch.from_numpy(msg_h.view(np.int16)).cuda()
    par0 = torch.zeros((nb, ecc), dtype=torch.int16, device="cuda")
    code.encode(msg0.data_ptr(), nb, par0.data_ptr(), sp)
    par_clean = par0
    if decode:
        cw = torch.cat([msg0, par0], dim=1)
        torch_rsi16_apply_errors(torch, cw, pos_h, d_h)
        msg0, par0 = cw[:, :ml].contiguous(), cw[:, ml:].contiguous()
        del cw
    nbuf = 2
    if decode:
        bufs = [(msg0.clone(), par0.clone(), torch.zeros(nb, dtype=torch.uint8, device="cuda")) for _ in range(nbuf)]
    else:
        bufs = [(msg0 if i == 0 else msg0.clone(), torch.zeros_like(par0), None) for i in range(nbuf)]

    def restore(j):
        bufs[j][0].copy_(msg0)
        bufs[j][1].copy_(par0)

    def run(j):
        m, p, s = bufs[j]
        if decode:
            code.repair(m.data_ptr(), p.data_ptr(), nb, s.data_ptr(), sp)
        else:
            code.encode(m.data_ptr(), nb, p.data_ptr(), sp)

    t = timed_steps(torch, args, world, run, restore if decode else None, nbuf)
    S = min(nb, args.sample_rsi16_decode if decode else args.sample_rsi16_encode)
    m, p, s = bufs[0]
    gpu = {"parity": p[:S].cpu().numpy().view(np.uint16), "blocks": S, "seed": seed}
    if decode:
        gpu.update(par_clean=par_clean[:S].cpu().numpy().view(np.uint16), msg=m[:S].cpu().numpy().view(np.uint16),
                   status=s[:S].cpu().numpy())
    lf = libffrs_gb300.libffrs
    rs = lf.RSi16(bl, ecc)
    hm = lf.create_buffer(nb * ml * 2)
    m0 = msg0.cpu().numpy().tobytes()
    hm[:] = m0
    if decode:
        hp = lf.create_buffer(nb * ecc * 2)
        p0 = par0.cpu().numpy().tobytes()

        def prep():
            hm[:] = m0
            hp[:] = p0

        sec = e2e_median(args, lambda: rs.repair_blocks(hm, hp), prep)
        same = bool(np.array_equal(np.frombuffer(hm, np.uint16), m.cpu().numpy().view(np.uint16).reshape(-1)))
    else:
        got = []
        sec = e2e_median(args, lambda: got.__setitem__(slice(None), [rs.encode(hm)]))
        same = bool(got) and bytes(got[0]) == p.cpu().numpy().tobytes()
    algo = nb * (2048 + 4 if decode else 2048)
    if decode:
        e2e = {"value": algo * world / sec / 1e9 if sec else None, "unit": "GB/s",
               "h2d_bytes_per_step": nb * bl * 2, "d2h_bytes_per_step": nb * bl * 2 + nb,
               "api": "libffrs.RSi16.repair_blocks(create_buffer, create_buffer)", "same_bytes_as_device_path": same}
    else:
        e2e = {"value": algo * world / sec / 1e9 if sec else None, "unit": "GB/s",
               "h2d_bytes_per_step": nb * ml * 2, "d2h_bytes_per_step": nb * ecc * 2, "api": "libffrs.RSi16.encode",
               "same_bytes_as_device_path": same}
    out = dict(t, workload="rsi16-decode" if decode else "rsi16-encode", algo_bytes_per_step=algo, gpu=gpu,
               dtype="u32 mod 65537", e2e=e2e,
               config={"workload": ("RSi16(1024, 64) decode, 262144 blocks, 0-32 symbol errors/block" if decode else
                                    "RSi16(1024, 64) encode, 262144 blocks x 960 uint16 words"),
                       "blocks": nb, "l2": "inputs larger than L2 (503 MB per step)"})
    if decode:
        out["status_ok_fraction"] = float((s == 2).float().mean().item())
    return out


# ---------------------------------------------------------------- CPU legs
#
# The oracle on the same seeded inputs as the GPU arm: the CPU baseline and
# the parity check of the GPU outputs.  A leg is prep (inputs, untimed) and
# run (the timed oracle call); check compares run's outputs with the GPU's.

def _cmp(what, pairs, blocks):
    bad = [name for name, a, b in pairs if not np.array_equal(a, b)]
    rec = {"status": "ok" if not bad else "MISMATCH", "blocks": blocks, "checked": what}
    if bad:
        rec["differs"] = bad
    return rec


class LegRs256Decode:
    bytes_per_block = 256
    calibration = "rs256-decode"

    def prep(self, seed, n, threads, first_chunk=0):
        from oracle import oracle as O

        self.o = O.RS256(32)
        data, pos, vals = chunks(rs256_decode_chunk, seed, n, RS_CHUNK, first_chunk)
        self.par = self.o.encode_blocks(data, threads=threads)
        cw = np.concatenate([data, self.par], axis=1)
        rs256_apply_errors(cw, pos, vals)
        self.d, self.p = np.ascontiguousarray(cw[:, :223]), np.ascontiguousarray(cw[:, 223:])
        self.n = n

    def run(self, threads):
        self.st = self.o.decode_blocks(self.d, self.p, threads=threads)

    def check(self, gpu):
        return _cmp("GPU encoder parity of the clean blocks; decode statuses, corrected data and parity bytes",
                    [("encode", self.par, gpu["par_clean"][:self.n]), ("status", self.st, gpu["status"][:self.n]),
                     ("data", self.d, gpu["data"][:self.n]), ("parity", self.p, gpu["parity"][:self.n])], self.n)


class LegRs256Encode:
    bytes_per_block = 255
    calibration = "rs256-encode"

    def prep(self, seed, n, threads, first_chunk=0):
        from oracle import oracle as O

        self.o = O.RS256(32)
        self.data = rs256_encode_chunk(seed, first_chunk, n)
        self.n = n

    def run(self, threads):
        self.par = self.o.encode_blocks(self.data, threads=threads)

    def check(self, gpu):
        return _cmp("parity bytes", [("parity", self.par, gpu["parity"][:self.n])], self.n)


class LegRsi16Encode:
    bytes_per_block = 2048
    calibration = "rsi16-encode"

    def prep(self, seed, n, threads, first_chunk=0):
        from oracle import oracle as O

        self.o = O.RSi16(1024, 64)
        self.msg = chunks(rsi16_chunk, seed, n, RSI_CHUNK, first_chunk, corrupt=False)[0]
        self.n = n

    def run(self, threads):
        self.par = self.o.encode_blocks(self.msg, threads=threads)

    def check(self, gpu):
        return _cmp("parity words", [("parity", self.par, gpu["parity"][:self.n])], self.n)


class LegRsi16Decode:
    bytes_per_block = 2052
    calibration = "rsi16-decode"

    def prep(self, seed, n, threads, first_chunk=0):
        from oracle import oracle as O

        self.o = O.RSi16(1024, 64)
        msg, pos, d = chunks(rsi16_chunk, seed, n, RSI_CHUNK, first_chunk, corrupt=True)
        self.par = self.o.encode_blocks(msg, threads=threads)
        cw = np.concatenate([msg, self.par], axis=1).astype(np.int64)
        rsi16_apply_errors(cw, pos, d)
        self.m = np.ascontiguousarray(cw[:, :960].astype(np.uint16))
        self.p = np.ascontiguousarray(cw[:, 960:].astype(np.uint16))
        self.n = n

    def run(self, threads):
        self.st = self.o.repair_blocks(self.m, self.p, threads=threads)

    def check(self, gpu):
        st8 = np.where(self.st < 0, 255, self.st.astype(np.int16)).astype(np.uint8)
        return _cmp("GPU encoder parity of the clean blocks; RepairStatus, repaired message and parity words "
                    "(W = 1 semantics)",
                    [("encode", self.par, gpu["par_clean"][:self.n]), ("status", st8, gpu["status"][:self.n]),
                     ("message", self.m, gpu["msg"][:self.n]), ("parity", self.p, gpu["parity"][:self.n])], self.n)


# workload -> (leg, all-threads sample, one-core sample); samples are the
# workload's first blocks
CPU_LEGS = {
    "rs256-decode": (LegRs256Decode, 262144, 16384),
    "rs256-encode": (LegRs256Encode, 65536, 65536),
    "rsi16-encode": (LegRsi16Encode, 65536, 8192),
    "rsi16-decode": (LegRsi16Decode, 16384, 1024),
}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def timed_leg(leg, threads, reps=1):
    best = 1e30
    for _ in range(reps):
        t0 = time.perf_counter()
        leg.run(threads)
        best = min(best, time.perf_counter() - t0)
    return leg.n * leg.bytes_per_block / best / 1e9, best


def cpu_worker(args):
    """One pinned process of the multi-process CPU baseline: prepares its
    slice, waits for the common start time, runs the oracle on one thread and
    prints the times of that call."""
    os.sched_setaffinity(0, {args.cw_core})
    leg = CPU_LEGS[args.cpu_worker][0]()
    leg.prep(args.cw_seed, args.cw_blocks, 1, args.cw_chunk)
    while time.time() < args.cw_at:
        time.sleep(0.0005)
    t0 = time.time()
    leg.run(1)
    t1 = time.time()
    print(json.dumps({"t0": t0, "t1": t1}))


def cpu_pinned_processes(workload, seed, per_proc):
    """One process per host core, each pinned to its core and working on its
    own chunk of the workload; all start their timed oracle call at the same
    wall-clock time.  The figure is the bytes of all slices over the span from
    the first start to the last end."""
    cores = sorted(os.sched_getaffinity(0))
    leg_cls = CPU_LEGS[workload][0]
    at = time.time() + 4.0
    procs = []
    for i, core in enumerate(cores):
        cmd = [sys.executable, os.path.abspath(__file__), "--cpu-worker", workload, "--cw-seed", str(seed),
               "--cw-chunk", str(i), "--cw-blocks", str(per_proc), "--cw-core", str(core), "--cw-at", repr(at)]
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                                      env=dict(os.environ, OMP_NUM_THREADS="1")))
    res = []
    for p in procs:
        out, err = p.communicate(timeout=600)
        if p.returncode != 0:
            return {"error": (err.strip().splitlines() or ["worker failed"])[-1]}
        res.append(json.loads(out.strip().splitlines()[-1]))
    late = max(r["t0"] for r in res) - at
    span = max(r["t1"] for r in res) - min(r["t0"] for r in res)
    return {"value": per_proc * len(cores) * leg_cls.bytes_per_block / span / 1e9, "unit": "GB/s",
            "processes": len(cores), "sample": "%d blocks per process, each on its own chunk" % per_proc,
            "latest_start_s": round(late, 4)}


def cpu_baseline(workload, seed, gpu, args):
    """cpu_baseline and parity records of one workload (rank 0, N = 1 or
    every N: the host figures do not depend on N)"""
    leg_cls, sample, one = CPU_LEGS[workload]
    threads = host_threads()
    if gpu is not None:
        sample = min(sample, gpu["blocks"])
    leg = leg_cls()
    leg.prep(seed, sample, threads)
    v, dt = timed_leg(leg, threads)
    parity = leg.check(gpu) if gpu is not None else None
    rec = {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
           "sample": "%d blocks of the same seeded workload (%.2f s on %d threads)" % (sample, dt, threads)}
    if not args.no_cpu_scaling:
        leg1 = leg_cls()
        leg1.prep(seed, one, threads)
        v1, dt1 = timed_leg(leg1, 1)
        rec["single_core"] = {"value": v1, "unit": "GB/s", "sample": "%d blocks (%.2f s)" % (one, dt1)}
        rec["pinned_processes"] = cpu_pinned_processes(workload, seed, one)
    cal = load_calibration(leg_cls.calibration)
    if cal:
        rec["calibration"] = cal
    return rec, parity


# ---------------------------------------------------------------- mixed batch

def make_mixed(torch, total_bytes, seed):
    """Seeded mixed workload of uneven requests: half the codeword bytes RS256
    (ecc_len in {2..64}, block_len uniform in [ecc+1, 255]), a quarter RSi16
    (ecc_len in {16..128}, block_len in [256, 4096] rounded down to a multiple
    of ecc_len), a quarter CIRC16(128, 8, 128, 8, 4) codewords.  RS256 and
    RSi16 requests are half encode, half decode with correctable errors
    (uniform 0 .. ecc_len/2 per block at distinct positions); CIRC16 requests
    are encodes or repairs of one burst of 1..64 changed message words per
    codeword (at most a quarter of the CIRC16 bytes per request).  Blocks per
    request are log-uniform.  Decode inputs are encoded by the plain GPU path
    and corrupted on the device.

    Returns (requests, codes): every request holds its code, device tensor
    views and the pristine inputs (data0, par0) for restoring between runs."""
    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(seed))
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    st = torch.cuda.current_stream().cuda_stream
    reqs = []
    codes = {}

    def code(kind, *key):
        k = (kind,) + key
        if k not in codes:
            codes[k] = {"rs256": capi.RS256Code, "rsi16": capi.RSi16Code, "circ16": capi.CIRC16Code}[kind](*key)
        return codes[k]

    budget = {"rs256": total_bytes // 2, "rsi16": total_bytes // 4, "circ16": total_bytes // 4}
    # RS256
    used = 0
    while used < budget["rs256"]:
        ecc = int(rng.choice([2, 4, 8, 16, 32, 64]))
        bl = int(rng.integers(ecc + 1, 256))
        ml = bl - ecc
        nb = int(np.exp(rng.uniform(np.log(16), np.log(16384))))
        nb = max(1, min(nb, (budget["rs256"] - used) // bl + 1))
        dec = bool(rng.integers(0, 2))
        data = torch.randint(0, 256, (nb, ml), dtype=torch.uint8, device="cuda", generator=g)
        par = torch.zeros((nb, ecc), dtype=torch.uint8, device="cuda")
        c = code("rs256", ecc)
        r = {"kind": "rs256", "code": c, "op": "dec" if dec else "enc", "nb": nb, "ml": ml, "ecc": ecc,
             "data": data, "par": par, "status": torch.zeros(nb, dtype=torch.uint8, device="cuda")}
        if dec:
            c.encode(data.data_ptr(), nb, ml, par.data_ptr(), st)
            cw = torch.cat([data, par], dim=1)
            k = torch.randint(0, ecc // 2 + 1, (nb,), device="cuda", generator=g)
            kmax = ecc // 2
            if kmax:
                pos = torch.rand((nb, bl), device="cuda", generator=g).argsort(dim=1)[:, :kmax]
                vals = torch.randint(1, 256, (nb, kmax), dtype=torch.uint8, device="cuda", generator=g)
                vals *= (torch.arange(kmax, device="cuda")[None, :] < k[:, None]).to(torch.uint8)
                rows = torch.arange(nb, device="cuda")[:, None].expand(nb, kmax)
                cw[rows, pos] ^= vals
            data.copy_(cw[:, :ml])
            par.copy_(cw[:, ml:])
        r["data0"], r["par0"] = data.clone(), par.clone()
        reqs.append(r)
        used += nb * bl
    # RSi16
    used = 0
    while used < budget["rsi16"]:
        ecc = int(rng.choice([16, 32, 64, 128]))
        bl = int(rng.integers(256, 4097)) // ecc * ecc
        ml = bl - ecc
        nb = int(np.exp(rng.uniform(np.log(2), np.log(512))))
        nb = max(1, min(nb, (budget["rsi16"] - used) // (2 * bl) + 1))
        dec = bool(rng.integers(0, 2))
        msg = torch.randint(-32768, 32768, (nb, ml), dtype=torch.int16, device="cuda", generator=g)
        par = torch.zeros((nb, ecc), dtype=torch.int16, device="cuda")
        c = code("rsi16", bl, ecc)
        r = {"kind": "rsi16", "code": c, "op": "dec" if dec else "enc", "nb": nb, "ml": ml, "ecc": ecc,
             "data": msg, "par": par, "status": torch.zeros(nb, dtype=torch.uint8, device="cuda")}
        if dec:
            c.encode(msg.data_ptr(), nb, par.data_ptr(), st)
            cw = torch.cat([msg, par], dim=1)
            kmax = ecc // 2
            k = torch.randint(0, kmax + 1, (nb,), device="cuda", generator=g)
            pos = torch.rand((nb, bl), device="cuda", generator=g).argsort(dim=1)[:, :kmax]
            rows = torch.arange(nb, device="cuda")[:, None].expand(nb, kmax)
            v = cw[rows, pos].to(torch.int64) & 0xFFFF
            d = torch.randint(1, 65537, (nb, kmax), device="cuda", generator=g)
            nv = (v + d) % 65537
            nv = torch.where(nv == 65536, (v + d + 1) % 65537, nv)
            nv = torch.where(torch.arange(kmax, device="cuda")[None, :] < k[:, None], nv, v)
            cw[rows, pos] = nv.to(torch.int32).to(torch.int16)
            msg.copy_(cw[:, :ml])
            par.copy_(cw[:, ml:])
        r["data0"], r["par0"] = msg.clone(), par.clone()
        reqs.append(r)
        used += nb * bl * 2
    # CIRC16: half encode, half decode with one burst of 1..64 consecutive
    # message words changed per codeword
    used = 0
    c = code("circ16", 128, 8, 128, 8, 4)
    cwb = (c.message_len + c.ecc_len) * 2
    ncirc = 0
    while used < budget["circ16"]:
        nb = int(np.exp(rng.uniform(np.log(1), np.log(64))))
        nb = max(1, min(nb, (budget["circ16"] - used) // cwb + 1, budget["circ16"] // (4 * cwb)))
        # the first CIRC16 request is a decode, the second an encode
        dec = ncirc == 0 or (ncirc > 1 and bool(rng.integers(0, 2)))
        ncirc += 1
        msg = torch.randint(-32768, 32768, (nb, c.message_len), dtype=torch.int16, device="cuda", generator=g)
        ecc = torch.zeros((nb, c.ecc_len), dtype=torch.int16, device="cuda")
        r = {"kind": "circ16", "code": c, "op": "dec" if dec else "enc", "nb": nb, "data": msg, "par": ecc,
             "status": torch.zeros(nb, dtype=torch.uint8, device="cuda") if dec else None}
        if dec:
            c.encode(msg.data_ptr(), nb, ecc.data_ptr(), st)
            for i in range(nb):
                blen = int(rng.integers(1, 65))
                s0 = int(rng.integers(0, c.message_len - blen + 1))
                d = torch.from_numpy(rng.integers(1, 65536, blen).astype(np.int32)).cuda()
                v = msg[i, s0:s0 + blen].to(torch.int32) & 0xFFFF
                msg[i, s0:s0 + blen] = ((v + d) & 0xFFFF).to(torch.int16)
        r["data0"], r["par0"] = msg.clone(), ecc.clone()
        reqs.append(r)
        used += nb * cwb
    order = rng.permutation(len(reqs))
    reqs = [reqs[i] for i in order]
    torch.cuda.synchronize()
    return reqs, codes


def mixed_bytes(r):
    return r["data"].numel() * r["data"].element_size() + r["par"].numel() * r["par"].element_size()


def mixed_restore(reqs):
    for r in reqs:
        if r["op"] == "dec":
            r["data"].copy_(r["data0"])
            r["par"].copy_(r["par0"])


def mixed_plain(reqs, stream):
    """one per-code C-ABI call per request"""
    for r in reqs:
        c = r["code"]
        if r["kind"] == "rs256":
            if r["op"] == "enc":
                c.encode(r["data"].data_ptr(), r["nb"], r["ml"], r["par"].data_ptr(), stream)
            else:
                c.decode(r["data"].data_ptr(), r["par"].data_ptr(), r["nb"], r["ml"], r["status"].data_ptr(), stream)
        elif r["kind"] == "rsi16":
            if r["op"] == "enc":
                c.encode(r["data"].data_ptr(), r["nb"], r["par"].data_ptr(), stream)
            else:
                c.repair(r["data"].data_ptr(), r["par"].data_ptr(), r["nb"], r["status"].data_ptr(), stream)
        elif r["op"] == "enc":
            c.encode(r["data"].data_ptr(), r["nb"], r["par"].data_ptr(), stream)
        else:
            c.repair(r["data"].data_ptr(), r["par"].data_ptr(), r["nb"], r["status"].data_ptr(), stream)


def mixed_batch(reqs):
    from libffrs_gb300 import capi

    b = capi.Batch()
    for r in reqs:
        c = r["code"]
        op = capi.ENCODE if r["op"] == "enc" else capi.DECODE
        st = r["status"].data_ptr() if r["op"] == "dec" else None
        if r["kind"] == "rs256":
            b.add_rs256(c, op, r["data"].data_ptr(), r["par"].data_ptr(), r["nb"], r["ml"], st)
        elif r["kind"] == "rsi16":
            b.add_rsi16(c, op, r["data"].data_ptr(), r["par"].data_ptr(), r["nb"], st)
        else:
            b.add_circ16(c, r["data"].data_ptr(), r["par"].data_ptr(), r["nb"], op, st)
    return b


# ---------------------------------------------------------------- serving

def make_serving_requests(n, seed, load_gbs):
    """Seeded request stream on page-locked host buffers: Poisson arrivals at
    `load_gbs` GB/s of offered codeword bytes, log-normal payloads clipped to
    [4 KiB, 64 MiB]; codes RS256 ecc 8 / 32 (255-byte blocks), RSi16(1024, 64),
    CIRC16(128, 8, 128, 8, 4); 70% encode, 30% decode with 0..max correctable
    errors per block (CIRC16: one burst of 1..64 message words).  Decode inputs are encoded
    with the host API and corrupted on the host."""
    import ctypes

    from libffrs_gb300 import capi

    rng = np.random.Generator(np.random.PCG64(seed))
    codes = {"rs8": capi.RS256Code(8), "rs32": capi.RS256Code(32), "rsi": capi.RSi16Code(1024, 64),
             "circ": capi.CIRC16Code(128, 8, 128, 8, 4)}
    L = capi.lib()

    def pinned(nbytes, dtype):
        p = ctypes.c_void_p()
        capi.call("ffgpu_host_alloc", max(nbytes, 1), ctypes.byref(p))
        arr = np.ctypeslib.as_array((ctypes.c_uint8 * max(nbytes, 1)).from_address(p.value))
        return p, arr.view(dtype)[: nbytes // np.dtype(dtype).itemsize]

    reqs = []
    t = 0.0
    for i in range(n):
        size = int(np.clip(np.exp(rng.normal(np.log(1 << 20), 1.5)), 4096, 64 << 20))
        kind = rng.choice(["rs8", "rs32", "rsi", "circ"])
        dec = rng.random() < 0.3
        c = codes[kind]
        r = {"kind": kind, "op": "dec" if dec else "enc", "code": c, "bufs": []}
        if kind in ("rs8", "rs32"):
            ecc = c.ecc_len
            ml = 255 - ecc
            nb = max(1, size // 255)
            pa, a = pinned(nb * ml, np.uint8)
            pb, b = pinned(nb * ecc, np.uint8)
            a[:] = rng.integers(0, 256, a.size, dtype=np.uint8)
            r.update(nb=nb, ml=ml, ecc=ecc, a=a, b=b, pa=pa, pb=pb, nbytes=nb * 255)
            if dec:
                capi.call("ffgpu_rs256_encode_host", c.h, pa, nb * ml, ml, pb)
                cw = np.concatenate([a.reshape(nb, ml), b.reshape(nb, ecc)], axis=1)
                kmax = ecc // 2
                for s0 in range(0, nb, 8192):
                    s1 = min(nb, s0 + 8192)
                    m = s1 - s0
                    k = rng.integers(0, kmax + 1, m)
                    pos = np.argsort(rng.random((m, 255), dtype=np.float32), axis=1)[:, :kmax]
                    vals = rng.integers(1, 256, (m, kmax), dtype=np.uint8) * (np.arange(kmax)[None, :] < k[:, None])
                    rows = np.repeat(np.arange(s0, s1)[:, None], kmax, axis=1)
                    cw[rows, pos] ^= vals.astype(np.uint8)
                a[:] = cw[:, :ml].reshape(-1)
                b[:] = cw[:, ml:].reshape(-1)
        elif kind == "rsi":
            nb = max(1, size // 2048)
            pa, a = pinned(nb * 960 * 2, np.uint16)
            pb, b = pinned(nb * 64 * 2, np.uint16)
            a[:] = rng.integers(0, 65536, a.size, dtype=np.uint16)
            r.update(nb=nb, a=a, b=b, pa=pa, pb=pb, nbytes=nb * 2048)
            if dec:
                capi.call("ffgpu_rsi16_encode_host", c.h, pa, nb, 1, pb)
                cw = np.concatenate([a.reshape(nb, 960), b.reshape(nb, 64)], axis=1).astype(np.int64)
                for s0 in range(0, nb, 2048):
                    s1 = min(nb, s0 + 2048)
                    m = s1 - s0
                    k = rng.integers(0, 33, m)
                    pos = np.argsort(rng.random((m, 1024), dtype=np.float32), axis=1)[:, :32]
                    rows = np.repeat(np.arange(s0, s1)[:, None], 32, axis=1)
                    v = cw[rows, pos]
                    d = rng.integers(1, 65537, (m, 32))
                    nv = (v + d) % 65537
                    nv = np.where(nv == 65536, (v + d + 1) % 65537, nv)
                    cw[rows, pos] = np.where(np.arange(32)[None, :] < k[:, None], nv, v)
                a[:] = cw[:, :960].reshape(-1).astype(np.uint16)
                b[:] = cw[:, 960:].reshape(-1).astype(np.uint16)
        else:
            cwb = (c.message_len + c.ecc_len) * 2
            nb = max(1, size // cwb)
            pa, a = pinned(nb * c.message_len * 2, np.uint16)
            pb, b = pinned(nb * c.ecc_len * 2, np.uint16)
            a[:] = rng.integers(0, 65536, a.size, dtype=np.uint16)
            r.update(nb=nb, a=a, b=b, pa=pa, pb=pb, nbytes=nb * cwb)
            if dec:
                capi.call("ffgpu_circ16_encode_host", c.h, pa, nb, pb)
                m = a.reshape(nb, c.message_len)
                for j in range(nb):  # one burst of 1..64 words per codeword
                    blen = int(rng.integers(1, 65))
                    s0 = int(rng.integers(0, c.message_len - blen + 1))
                    m[j, s0:s0 + blen] += rng.integers(1, 65536, blen).astype(np.uint16)
        if dec:
            ps, s = pinned(r["nb"], np.uint8)
            r.update(ps=ps, s=s)
        r["a0"], r["b0"] = r["a"].copy(), r["b"].copy()
        t += rng.exponential(r["nbytes"] / (load_gbs * 1e9))
        r["arrival"] = t
        reqs.append(r)
    return reqs, codes


def serving_restore(reqs):
    for r in reqs:
        r["a"][:] = r["a0"]
        r["b"][:] = r["b0"]


def serve_plain_one(r):
    """the per-request host API, as a plain caller would use it"""
    from libffrs_gb300 import capi

    c = r["code"]
    if r["kind"] in ("rs8", "rs32"):
        if r["op"] == "enc":
            capi.call("ffgpu_rs256_encode_host", c.h, r["pa"], r["nb"] * r["ml"], r["ml"], r["pb"])
        else:
            capi.call("ffgpu_rs256_decode_host", c.h, r["pa"], r["pb"], r["nb"], r["ml"], r["ps"])
    elif r["kind"] == "rsi":
        if r["op"] == "enc":
            capi.call("ffgpu_rsi16_encode_host", c.h, r["pa"], r["nb"], 1, r["pb"])
        else:
            capi.call("ffgpu_rsi16_repair_host", c.h, r["pa"], r["pb"], r["nb"], 1, None, -1, r["ps"])
    elif r["op"] == "enc":
        capi.call("ffgpu_circ16_encode_host", c.h, r["pa"], r["nb"], r["pb"])
    else:
        capi.call("ffgpu_circ16_repair_host", c.h, r["pa"], r["pb"], r["nb"], r["ps"])


def serve_submit(srv, r):
    from libffrs_gb300 import capi

    op = capi.ENCODE if r["op"] == "enc" else capi.DECODE
    c = r["code"]
    if r["kind"] in ("rs8", "rs32"):
        return srv.submit_rs256(c, op, r["pa"], r["pb"], r["nb"], r["ml"], r.get("ps"))
    if r["kind"] == "rsi":
        return srv.submit_rsi16(c, op, r["pa"], r["pb"], r["nb"], r.get("ps"))
    return srv.submit_circ16(c, r["pa"], r["pb"], r["nb"], op, r.get("ps"))


def run_served(reqs, slots=4):
    from libffrs_gb300 import capi

    srv = capi.Server(slots=slots, max_batch=64)
    t0 = time.perf_counter()
    tickets = []
    for r in reqs:
        d = r["arrival"] - (time.perf_counter() - t0)
        if d > 0:
            time.sleep(d)
        tickets.append(serve_submit(srv, r))
    for tk in tickets:
        srv.wait(tk)
    info = [srv.poll(tk) for tk in tickets]
    srv.close()
    lat = [i["done"] - i["submit"] for i in info]
    span = max(i["done"] for i in info) - min(i["submit"] for i in info)
    return lat, span


def run_plain_fifo(reqs):
    t0 = time.perf_counter()
    lat, done = [], []
    for r in reqs:
        d = r["arrival"] - (time.perf_counter() - t0)
        if d > 0:
            time.sleep(d)
        serve_plain_one(r)
        t = time.perf_counter() - t0
        lat.append(t - r["arrival"])
        done.append(t)
    return lat, max(done) - reqs[0]["arrival"]



def oracle_request_expect(kind, op, ecc, ml, nb, a0, b0, codes, threads=8):
    """The oracle's outputs (a, b, status or None) for one request of the mixed
    batch or of the serving stream, from its pristine host inputs: kind
    rs256 (ecc, message_len ml), rsi16 (ecc, message_len ml) or circ16
    (CIRC16(128, 8, 128, 8, 4)); a0/b0 flat uint8 or uint16 arrays."""
    from oracle import oracle as O

    key = (kind, ecc, ml)
    if key not in codes:
        codes[key] = (O.RS256(ecc, block_len=ml + ecc) if kind == "rs256" else
                      O.RSi16(ml + ecc, ecc) if kind == "rsi16" else O.CIRC16(128, 8, 128, 8, 4))
    o = codes[key]
    dec = op == "dec"
    if kind == "rs256":
        d = a0.reshape(nb, ml).copy()
        if not dec:
            return a0.copy(), o.encode_blocks(d, threads=threads).reshape(-1), None
        p = b0.reshape(nb, ecc).copy()
        st = o.decode_blocks(d, p, threads=threads)
        return d.reshape(-1), p.reshape(-1), st
    if kind == "rsi16":
        m = a0.reshape(nb, ml).copy()
        if not dec:
            return a0.copy(), o.encode_blocks(m, threads=threads).reshape(-1), None
        p = b0.reshape(nb, ecc).copy()
        st = o.repair_blocks(m, p, threads=threads)
        return m.reshape(-1), p.reshape(-1), np.where(st < 0, 255, st.astype(np.int16)).astype(np.uint8)
    if not dec:
        return a0.copy(), o.encode(a0, threads=threads), None
    mlen, elen = o.message_len, o.ecc_len
    m = a0.reshape(nb, mlen).copy()
    e = b0.reshape(nb, elen).copy()
    st = np.zeros(nb, np.uint8)
    for i in range(nb):
        mi, ei = m[i].copy(), e[i].copy()
        rc = o.repair(mi, ei)
        m[i] = mi
        if rc < 0:
            st[i] = 255  # a raising codeword keeps its ecc
        else:
            e[i] = ei
    return m.reshape(-1), e.reshape(-1), st


def serving_expect(r, codes, threads=8):
    """oracle_request_expect for one request of make_serving_requests"""
    kind = {"rs8": "rs256", "rs32": "rs256", "rsi": "rsi16", "circ": "circ16"}[r["kind"]]
    ecc = r.get("ecc", 64 if kind == "rsi16" else 0)
    ml = r.get("ml", 960 if kind == "rsi16" else 0)
    return oracle_request_expect(kind, r["op"], ecc, ml, r["nb"], r["a0"], r["b0"], codes, threads)


def mixed_expect(r, a0, b0, codes, threads=8):
    """oracle_request_expect for one request of make_mixed (host copies of its
    pristine inputs a0 / b0)"""
    ecc = r.get("ecc", 0)
    ml = r.get("ml", 0)
    return oracle_request_expect(r["kind"], r["op"], ecc, ml, r["nb"], a0, b0, codes, threads)


def _host_u(t):
    a = t.cpu().numpy()
    return (a.view(np.uint16) if a.dtype == np.int16 else a).reshape(-1)


def bench_batch_mixed(args, torch, rank, world):
    from libffrs_gb300 import capi

    total = (args.blocks or 1024) << 20  # --blocks = MiB of codewords for this workload
    reqs, _codes = make_mixed(torch, total, 4000 + rank)
    nbytes = sum(mixed_bytes(r) for r in reqs)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def outputs():
        return [(r["data"].clone() if r["op"] == "dec" else None, r["par"].clone(),
                 r["status"].clone() if r["op"] == "dec" else None) for r in reqs]

    def run_timed(fn, steps):
        ms = []
        for _ in range(steps):
            mixed_restore(reqs)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms

    # plain per-request path (the reference's API shape: one call per request)
    for _ in range(max(1, args.warmup)):
        mixed_restore(reqs)
        mixed_plain(reqs, sp)
    torch.cuda.synchronize()
    plain_ms = run_timed(lambda: mixed_plain(reqs, sp), max(1, min(args.steps, 3)))
    ref_out = outputs()
    # batched: autotuned plan, captured graph, one replay per step
    b = mixed_batch(reqs)
    mixed_restore(reqs)
    b.plan(autotune=True, stream=sp)
    b.capture(sp)
    for _ in range(args.warmup):
        mixed_restore(reqs)
        b.launch(sp)
    torch.cuda.synchronize()
    launches0 = capi.kernel_launches()
    capi.timing_collect()
    capi.timing_enable(True)
    with ClockSampler(torch.cuda.current_device()) as clk, TimedRange(torch):
        kern_ms = run_timed(lambda: b.launch(sp), args.steps)
    launches = capi.kernel_launches() - launches0
    kernels = capi.timing_collect()
    capi.timing_enable(False)
    got = outputs()
    same = all(all((x is None and y is None) or torch.equal(x, y) for x, y in zip(o, p))
               for o, p in zip(ref_out, got))
    if not same:
        raise SystemExit("batched outputs differ from the plain per-request path")
    plain_gbs = nbytes / (statistics.median(plain_ms) / 1e3) / 1e9
    batch_gbs = nbytes / (statistics.median(kern_ms) / 1e3) / 1e9
    nk = {}
    for r in reqs:
        nk[r["kind"] + "-" + r["op"]] = nk.get(r["kind"] + "-" + r["op"], 0) + 1
    # host copies of a sample of the requests for the oracle check: every
    # `parity_every`-th request and every CIRC16 repair
    every = max(1, args.mixed_parity_every)
    sample = []
    for i, (r, (d, p, s)) in enumerate(zip(reqs, got)):
        if i % every == 0 or (r["kind"] == "circ16" and r["op"] == "dec"):
            sample.append((r, _host_u(r["data0"]), _host_u(r["par0"]),
                           (_host_u(d) if d is not None else _host_u(r["data"])), _host_u(p),
                           s.cpu().numpy() if s is not None else None))
    return {
        "workload": "batch-mixed", "total_ms": sum(kern_ms), "kern_ms": kern_ms, "algo_bytes_per_step": nbytes,
        "launches": launches, "kernels": kernels, "clocks": clk.summary(),
        "e2e": {"value": None, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "device-resident batch API; the host-buffer path of mixed requests is the serving workload"},
        "config": {"workload": "mixed batch: 1/2 RS256 (ecc 2..64, uneven lengths), 1/4 RSi16 (ecc 16..128, "
                               "block 256..4096), 1/4 CIRC16(128,8,128,8,4) with 1-64 word bursts; "
                               "half encode, half decode",
                   "bytes": nbytes, "requests": len(reqs), "requests_by_kind": nk, "plan": b.info(),
                   "l2": "inputs larger than L2 (%d MB)" % (nbytes >> 20)},
        "dtype": "u8 / u32 mod 65537",
        "mixed_sample": sample,
        "extra": {"plain_per_request_gbs": plain_gbs, "batched_gbs": batch_gbs,
                  "batched_over_plain": batch_gbs / plain_gbs, "bit_identical_to_plain": same,
                  "plain_ms": statistics.median(plain_ms)},
    }


def cpu_mixed(sample, threads):
    """the oracle over the sampled requests of the mixed batch: its time (the
    CPU baseline of the batch workload) and the parity of the batch outputs"""
    codes = {}
    nbytes, secs, bad, blocks = 0, 0.0, [], 0
    for r, a0, b0, a, b, s in sample:
        t0 = time.perf_counter()
        wa, wb, ws = mixed_expect(r, a0, b0, codes, threads)
        secs += time.perf_counter() - t0
        nbytes += a0.nbytes + (b.nbytes if r["op"] == "enc" else b0.nbytes)
        blocks += r["nb"]
        ok = np.array_equal(wb, b) and (r["op"] == "enc" or (np.array_equal(wa, a) and np.array_equal(ws, s)))
        if not ok:
            bad.append("%s-%s x%d" % (r["kind"], r["op"], r["nb"]))
    parity = {"status": "ok" if not bad else "MISMATCH", "requests": len(sample), "blocks": blocks,
              "checked": "outputs (and statuses, repaired bytes) of every sampled request against the oracle"}
    if bad:
        parity["differs"] = bad[:10]
    return nbytes / secs / 1e9, secs, nbytes, parity


def bench_serving(args, torch, rank, world):
    nreq = args.blocks or 400
    load = 40.0  # offered GB/s of codeword bytes
    reqs, _codes = make_serving_requests(nreq, 5000 + rank, load)
    nbytes = sum(r["nbytes"] for r in reqs)
    # warm up both paths on a prefix
    serving_restore(reqs)
    for r in reqs[:8]:
        serve_plain_one(r)
    run_served(reqs[:8])
    serving_restore(reqs)
    plain_lat, plain_span = run_plain_fifo(reqs)
    want = [(r["a"].copy(), r["b"].copy(), r["s"].copy() if "s" in r else None) for r in reqs]
    from libffrs_gb300 import capi

    best = None
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(max(1, args.steps)):
            serving_restore(reqs)
            n0 = capi.kernel_launches()
            lat, span = run_served(reqs)
            launched = capi.kernel_launches() - n0
            if best is None or span < best[1]:
                best = (lat, span, launched)
    lat, span, launched = best
    same = all(np.array_equal(r["a"], w[0]) and np.array_equal(r["b"], w[1]) and
               (w[2] is None or np.array_equal(r["s"], w[2])) for r, w in zip(reqs, want))
    if not same:
        raise SystemExit("served results differ from the plain per-request results")

    def pct(v, q):
        return float(np.percentile(np.array(v) * 1e3, q))

    gbs = nbytes / span / 1e9
    every = max(1, args.serving_parity_every)
    return {
        "workload": "serving", "total_ms": span * 1e3 * max(1, args.steps), "kern_ms": [span * 1e3],
        "algo_bytes_per_step": nbytes,
        "launches": launched, "kernels": {}, "clocks": clk.summary(),
        "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "api": "ffgpu_server_submit_* on page-locked host buffers"},
        "config": {"workload": "serving: Poisson arrivals at %.0f GB/s offered, log-normal payloads 4 KiB-64 MiB, "
                               "RS256 ecc 8/32, RSi16(1024,64), CIRC16(128,8,128,8,4), 70%% encode, decodes with "
                               "0..max correctable errors (CIRC16: one 1-64 word burst)" % load,
                   "requests": nreq, "bytes": nbytes, "slots": 4},
        "dtype": "u8 / u32 mod 65537",
        "serving_sample": [r for i, r in enumerate(reqs) if i % every == 0],
        "extra": {"served_p50_ms": pct(lat, 50), "served_p99_ms": pct(lat, 99), "served_gbs": gbs,
                  "plain_p50_ms": pct(plain_lat, 50), "plain_p99_ms": pct(plain_lat, 99),
                  "plain_gbs": nbytes / plain_span / 1e9, "bit_identical_to_plain": same},
    }


def cpu_serving(sample, threads):
    codes = {}
    nbytes, secs, bad = 0, 0.0, []
    for r in sample:
        t0 = time.perf_counter()
        wa, wb, ws = serving_expect(r, codes, threads)
        secs += time.perf_counter() - t0
        nbytes += r["nbytes"]
        ok = np.array_equal(wa, r["a"]) and np.array_equal(wb, r["b"]) and (ws is None or np.array_equal(ws, r["s"]))
        if not ok:
            bad.append("%s-%s x%d" % (r["kind"], r["op"], r["nb"]))
    parity = {"status": "ok" if not bad else "MISMATCH", "requests": len(sample),
              "checked": "served bytes and statuses of every sampled request against the oracle"}
    if bad:
        parity["differs"] = bad[:10]
    return nbytes / secs / 1e9, secs, nbytes, parity


# ---------------------------------------------------------------- driver

WORKLOADS = {
    "rs256-decode": bench_rs256_decode,
    "rs256-encode": bench_rs256_encode,
    "rsi16-encode": lambda a, t, r, w: bench_rsi16(a, t, r, w, False),
    "rsi16-decode": lambda a, t, r, w: bench_rsi16(a, t, r, w, True),
    "batch-mixed": bench_batch_mixed,
    "serving": bench_serving,
}
ORDER = ["rs256-decode", "rs256-encode", "rsi16-encode", "rsi16-decode", "batch-mixed", "serving"]
METRIC = "encode/decode GB/s bit-exact (RS256 decode, ecc_len 32, 1 GB300 per rank)"
SEEDS = {"rs256-decode": 1000, "rs256-encode": 2000, "rsi16-encode": 3000, "rsi16-decode": 3100}


def metric_of(workload):
    return METRIC if workload == "rs256-decode" else f"{workload} GB/s bit-exact"


def max_over_ranks(value, world, device):
    """The slowest rank's timed-region length: the whole job ends with it."""
    if world <= 1:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_gbs(bytes_per_rank_step, steps, world, total_ms):
    """Whole-job GB/s: every rank processes its own shard of bytes_per_rank_step
    per step (weak scaling), over the slowest rank's time."""
    return bytes_per_rank_step * steps * world / (total_ms / 1e3) / 1e9


def record(args, r, world, total_ms):
    """the JSON record of one workload (rank 0)"""
    steps = args.steps
    value = job_gbs(r["algo_bytes_per_step"], steps, world, total_ms)
    kernels = r.get("kernels") or {}
    ktot = sum(ms for ms, _ in kernels.values()) or 1.0
    if kernels:
        dom = max(kernels, key=lambda k: kernels[k][0])
        dom_ms = kernels[dom][0] / kernels[dom][1]
        dom_launch_per_step = kernels[dom][1] / args.steps
    else:
        dom, dom_ms, dom_launch_per_step = None, statistics.median(r["kern_ms"]), 1.0
    # algorithmic bytes per launch = per-unit bytes x units one launch processes
    achieved = r["algo_bytes_per_step"] / dom_launch_per_step / (dom_ms / 1e3) / 1e9
    peak, peak_src = load_peaks()
    rec = {
        "metric": metric_of(r["workload"]), "value": value, "unit": "GB/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": total_ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": r["dtype"], "data": "synthetic (seeded numpy PCG64 / torch generators)",
        "config": r["config"], "e2e": r["e2e"], "gpu_launches": r["launches"], "clocks": r["clocks"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src, "traffic": load_traffic(r["workload"]),
                     "kernel": dom, "kernel_ms_per_launch": dom_ms},
        "kernels": {k: {"ms_per_launch": ms / n, "launches": n, "share": ms / ktot} for k, (ms, n) in kernels.items()},
    }
    if "status_ok_fraction" in r:
        rec["status_ok_fraction"] = r["status_ok_fraction"]
    if "extra" in r:
        rec.update(r["extra"])
    return rec


def add_cpu(args, rec, r):
    """the CPU legs of one workload: baseline and parity (rank 0 only)"""
    wl = r["workload"]
    threads = host_threads()
    if wl in CPU_LEGS:
        rec["cpu_baseline"], rec["parity"] = cpu_baseline(wl, r["gpu"]["seed"], r["gpu"], args)
    elif wl == "batch-mixed":
        v, secs, nb, parity = cpu_mixed(r["mixed_sample"], threads)
        rec["cpu_baseline"] = {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
                               "sample": "the oracle on %d sampled requests, %.0f MB (%.2f s)" %
                                         (parity["requests"], nb / 1e6, secs)}
        rec["parity"] = parity
    elif wl == "serving":
        v, secs, nb, parity = cpu_serving(r["serving_sample"], threads)
        rec["cpu_baseline"] = {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
                               "sample": "the oracle on %d sampled requests, %.0f MB (%.2f s)" %
                                         (parity["requests"], nb / 1e6, secs)}
        rec["parity"] = parity


REFERENCE_CONFIG = {
    "rs256-decode": {"workload": "RS256 decode ecc_len=32, 1048576 blocks x (223+32) B, 0-16 errors/block, "
                                 "1% 17-20 errors", "blocks": 1048576, "message_len": 223, "ecc_len": 32},
    "rs256-encode": {"workload": "RS256 encode ecc_len=32, 65536 blocks x 223 B", "blocks": 65536},
    "rsi16-decode": {"workload": "RSi16(1024, 64) decode, 262144 blocks, 0-32 symbol errors/block",
                     "blocks": 262144},
    "rsi16-encode": {"workload": "RSi16(1024, 64) encode, 262144 blocks x 960 uint16 words", "blocks": 262144},
}


def reference_record(args, wl, steps):
    """the reference arm of one workload: the oracle (the reference path's C
    restatement) on all host threads, each step one pass over the sample"""
    if wl not in CPU_LEGS:
        return {"impl": "reference", "unavailable": "the reference has no batched or serving path for " + wl}
    leg_cls, sample, _ = CPU_LEGS[wl]
    threads = host_threads()
    leg = leg_cls()
    leg.prep(SEEDS[wl], sample, threads)
    for _ in range(args.warmup):
        leg.run(threads)
    vals = []
    for _ in range(max(1, steps)):
        v, _ = timed_leg(leg, threads)
        vals.append(v)
    v = statistics.median(vals)
    rec = {"impl": "reference", "metric": metric_of(wl), "value": v, "unit": "GB/s", "n_gpus": args.world,
           "steps": max(1, steps), "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "u8" if wl.startswith("rs256") else "u32 mod 65537",
           "data": "synthetic (seeded numpy PCG64, the GPU arm's inputs)",
           "config": dict(REFERENCE_CONFIG[wl], sample_blocks=sample),
           "cpu_baseline": {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
                            "sample": f"{sample} blocks of the {wl} workload per step"},
           "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    cal = load_calibration(leg_cls.calibration)
    if cal:
        rec["cpu_baseline"]["calibration"] = cal
    return rec


def run_reference(args, rank, world):
    if rank != 0:
        return
    args.world = world
    if args.workload == "all":
        line = reference_record(args, "rs256-decode", args.steps)
        line["workloads"] = {wl: reference_record(args, wl, min(args.steps, 3)) for wl in ORDER[1:]}
    else:
        line = reference_record(args, args.workload, args.steps)
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="all", choices=["all"] + ORDER)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cpu-scaling", action="store_true", help="skip the one-core and pinned-process CPU figures")
    ap.add_argument("--blocks", type=int, default=0,
                    help="override the block count (small cases for profiling; not a bench line)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer pass (profiling)")
    ap.add_argument("--table-only", action="store_true",
                    help="rs256-decode through the per-thread table decoder (profiling that kernel)")
    ap.add_argument("--sample-rs256-decode", type=int, default=262144)
    ap.add_argument("--sample-rsi16-encode", type=int, default=65536)
    ap.add_argument("--sample-rsi16-decode", type=int, default=16384)
    ap.add_argument("--mixed-parity-every", type=int, default=8)
    ap.add_argument("--serving-parity-every", type=int, default=4)
    # one pinned process of the multi-process CPU baseline (internal)
    ap.add_argument("--cpu-worker", default=None)
    ap.add_argument("--cw-seed", type=int, default=0)
    ap.add_argument("--cw-chunk", type=int, default=0)
    ap.add_argument("--cw-blocks", type=int, default=0)
    ap.add_argument("--cw-core", type=int, default=0)
    ap.add_argument("--cw-at", type=float, default=0.0)
    args = ap.parse_args()
    if args.cpu_worker:
        cpu_worker(args)
        return
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
        run_reference(args, rank, world)
        return

    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__

    if rank == 0 or not os.path.exists(os.path.join(REPO, "libffrs_gb300", "libffgpu.so")):
        __graft_entry__.build()
    if world > 1:
        torch.distributed.barrier()
    from libffrs_gb300 import capi

    capi.call("ffgpu_init", local)
    todo = ORDER if args.workload == "all" else [args.workload]
    recs = {}
    for wl in todo:
        r = WORKLOADS[wl](args, torch, rank, world)
        total_ms = max_over_ranks(r["total_ms"], world, "cuda")
        if rank == 0:
            rec = record(args, r, world, total_ms)
            if not args.no_cpu_baseline:
                add_cpu(args, rec, r)
            recs[wl] = rec
        del r
        torch.cuda.empty_cache()
    if rank == 0:
        line = recs[todo[0]]
        if len(todo) > 1:
            line["workloads"] = {wl: recs[wl] for wl in todo[1:]}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
