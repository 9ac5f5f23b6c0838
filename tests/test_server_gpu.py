"""The serving engine: every request served in the mix (submitted together,
micro-batched, overlapping on several streams, admitted by an HBM budget)
gives exactly the bytes and statuses it gets when served alone through the
per-request host API."""

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
