"""The serving engine: every request served in the mix (submitted together,
micro-batched, overlapping on several streams, admitted by an HBM budget)
gives exactly the bytes and statuses it gets when served alone through the
per-request host API, and the oracle's; requests overlap on the device;
queued requests can be cancelled; a failed allocation fails only its own
micro-batch."""

import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def stream_of_requests(built):
    import bench

    reqs, codes = bench.make_serving_requests(40, 77, 1000.0)
    # keep the test quick: trim the largest payloads
    reqs = [r for r in reqs if r["nbytes"] <= (8 << 20)][:30]
    kinds = {(r["kind"], r["op"]) for r in reqs}
    return bench, reqs, codes, kinds


def _alone(bench, reqs):
    bench.serving_restore(reqs)
    for r in reqs:
        bench.serve_plain_one(r)
    return [(r["a"].copy(), r["b"].copy(), r["s"].copy() if "s" in r else None) for r in reqs]


def _check(reqs, want):
    for r, w in zip(reqs, want):
        np.testing.assert_array_equal(r["a"], w[0])
        np.testing.assert_array_equal(r["b"], w[1])
        if w[2] is not None:
            np.testing.assert_array_equal(r["s"], w[2])


def test_served_equals_alone(stream_of_requests):
    from libffrs_gb300 import capi

    bench, reqs, _, kinds = stream_of_requests
    assert ("rs32", "dec") in kinds or ("rs8", "dec") in kinds
    want = _alone(bench, reqs)
    bench.serving_restore(reqs)
    srv = capi.Server(slots=3, max_batch=8)
    tickets = [bench.serve_submit(srv, r) for r in reqs]
    for t in tickets:
        srv.wait(t, 60.0)
    info = [srv.poll(t) for t in tickets]
    assert all(i["state"] == 2 for i in info)
    assert all(i["submit"] <= i["start"] <= i["done"] for i in info)
    srv.close()
    _check(reqs, want)


def test_budget_admission(stream_of_requests):
    """With an HBM budget smaller than the whole stream, requests wait for
    memory, still complete, and still give the same bytes."""
    from libffrs_gb300 import capi

    bench, reqs, _, _ = stream_of_requests
    want = _alone(bench, reqs)
    bench.serving_restore(reqs)
    srv = capi.Server(hbm_budget=2 << 20, slots=4, max_batch=4)
    tickets = [bench.serve_submit(srv, r) for r in reqs]
    for t in tickets:
        srv.wait(t, 120.0)
    for t in tickets:
        srv.release(t)
    srv.close()
    _check(reqs, want)


def test_server_errors(built):
    from libffrs_gb300 import capi

    srv = capi.Server(slots=1)
    c = capi.RS256Code(32)
    with pytest.raises(capi.FFGPUError):
        srv.submit_rs256(c, capi.DECODE, 1, 1, 1, 223, None)  # decode without a status array
    with pytest.raises(capi.FFGPUError):
        srv.wait(12345, 0.1)  # unknown ticket
    srv.close()


def test_served_matches_oracle(stream_of_requests):
    """Every served request (encodes and decodes of all four codes) gives the
    oracle's bytes and statuses."""
    from libffrs_gb300 import capi

    bench, reqs, _, kinds = stream_of_requests
    codes = {}
    want = [bench.serving_expect(r, codes) for r in reqs]
    bench.serving_restore(reqs)
    srv = capi.Server(slots=4, max_batch=16)
    tickets = [bench.serve_submit(srv, r) for r in reqs]
    for t in tickets:
        srv.wait(t, 60.0)
    srv.close()
    assert {k for k, _ in kinds} >= {"rsi", "circ"}
    _check(reqs, want)


def _pinned(nbytes):
    from libffrs_gb300 import capi

    p = ctypes.c_void_p()
    capi.call("ffgpu_host_alloc", nbytes, ctypes.byref(p))
    return p, np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(p.value))


def test_requests_overlap_on_device(built):
    """A small request submitted while a large one runs is admitted into
    another slot before the large one completes, and its own submit-to-done
    time is shorter than the large one's: it does not wait for the large
    request (its copies may still queue behind the large copies on a shared
    copy engine, so the two may complete close together)."""
    from libffrs_gb300 import capi

    rsi = capi.RSi16Code(1024, 64)
    rs = capi.RS256Code(32)
    nb_big = 65536  # 128 MiB of RSi16 codewords: several ms of copies and kernels
    pm, m = _pinned(nb_big * 960 * 2)
    pp, p = _pinned(nb_big * 64 * 2)
    m[:] = np.random.Generator(np.random.PCG64(5)).integers(0, 256, m.size, dtype=np.uint8)
    pa, a = _pinned(223)
    pb, b = _pinned(32)
    a[:] = np.arange(223, dtype=np.uint8)
    srv = capi.Server(slots=4, max_batch=8)
    big = srv.submit_rsi16(rsi, capi.ENCODE, pm, pp, nb_big, None)
    t0 = time.perf_counter()
    while srv.poll(big)["state"] == 0 and time.perf_counter() - t0 < 10:
        time.sleep(0.0002)
    small = srv.submit_rs256(rs, capi.ENCODE, pa, pb, 1, 223, None)
    srv.wait(small, 30.0)
    srv.wait(big, 30.0)
    ib, is_ = srv.poll(big), srv.poll(small)
    srv.close()
    assert ib["state"] == 2 and is_["state"] == 2
    assert is_["start"] < ib["done"], (ib, is_)
    assert is_["done"] - is_["submit"] < ib["done"] - ib["submit"], (ib, is_)
    from oracle import oracle as O

    np.testing.assert_array_equal(b, O.RS256(32).encode_blocks(a.reshape(1, 223)).reshape(-1))


def test_cancel_queued_request(built):
    """Requests queued behind a full slot can be withdrawn; their buffers stay
    untouched, the others complete, and an admitted request cannot be
    cancelled."""
    from libffrs_gb300 import capi

    rsi = capi.RSi16Code(1024, 64)
    nb = 16384
    bufs = [(_pinned(nb * 960 * 2), _pinned(nb * 64 * 2)) for _ in range(4)]
    for (pm, m), _ in bufs:
        m[:] = 7
    srv = capi.Server(slots=1, max_batch=1)
    tickets = [srv.submit_rsi16(rsi, capi.ENCODE, pm, pp, nb, None) for (pm, _), (pp, _) in bufs]
    srv.cancel(tickets[3])
    srv.cancel(tickets[3])  # idempotent
    with pytest.raises(capi.FFGPUError) as ei:
        srv.wait(tickets[3], 5.0)
    assert ei.value.rc == capi.ECANCELLED
    for t in tickets[:3]:
        srv.wait(t, 30.0)
    assert srv.poll(tickets[3])["state"] == 4
    with pytest.raises(capi.FFGPUError):
        srv.cancel(tickets[0])  # already served
    srv.release(tickets[3])
    srv.close()
    assert not bufs[3][1][1].any()  # the cancelled request's parity was never written
    assert bufs[0][1][1].any()


def test_allocation_failure_fails_only_its_batch(built):
    """An out-of-memory allocation (injected on the host, no device fault)
    fails the micro-batch it was for with FFGPU_ENOMEM; the server frees what
    it held and serves the next requests correctly."""
    from libffrs_gb300 import capi
    from oracle import oracle as O

    rs = capi.RS256Code(32)
    nb = 1000
    pa, a = _pinned(nb * 223)
    pb, b = _pinned(nb * 32)
    a[:] = np.random.Generator(np.random.PCG64(11)).integers(0, 256, a.size, dtype=np.uint8)
    srv = capi.Server(slots=2, max_batch=1)
    capi.call("ffgpu_server_debug_fail_allocs", 1)
    try:
        t1 = srv.submit_rs256(rs, capi.ENCODE, pa, pb, nb, 223, None)
        with pytest.raises(capi.FFGPUError) as ei:
            srv.wait(t1, 30.0)
        assert ei.value.rc == capi.ENOMEM
        assert srv.poll(t1)["state"] == 3
        assert not b.any()
        for _ in range(3):
            t2 = srv.submit_rs256(rs, capi.ENCODE, pa, pb, nb, 223, None)
            srv.wait(t2, 30.0)
            srv.release(t2)
    finally:
        capi.call("ffgpu_server_debug_fail_allocs", 0)
        srv.close()
    np.testing.assert_array_equal(b.reshape(nb, 32), O.RS256(32).encode_blocks(a.reshape(nb, 223)))
