"""Serving loop with continuous batching: every request's records equal
swift_align on it alone, also when requests of different sizes and read
lengths (50-300 bases) share merged waves; a malformed request fails alone;
a memory budget smaller than any request still serves them (one at a
time); queued requests can be polled and cancelled.
"""
import random

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from swift_gb300 import build as b
    b.build()
    import swift_gb300
    return swift_gb300


@pytest.fixture(scope="module")
def setup(sg):
    from swift_gb300 import synth
    ctx = sg.Context(0)
    names, seqs = synth.make_reference(500_000, 3, sigma=0.5, repeat_frac=0.1, n_units=30,
                                       seed=71)
    ref = synth.fasta_bytes(names, seqs)
    ix = ctx.index(ref)
    rng = random.Random(72)
    reqs = []
    for t in range(36):
        n = int(10 ** rng.uniform(0, 3.3))  # 1 .. 2000 reads
        L = rng.randint(50, 300)
        rn, rs, _ = synth.make_reads(seqs, n, L, 0.01, 0.001, 0.05, seed=100 + t)
        reqs.append(synth.reads_fasta([f"q{t}_{i}" for i in range(n)], rs))
    return ctx, ix, reqs, ref


def params(sg, **kw):
    return sg.default_params(max_read_len=300, **kw)


def test_server_matches_single_requests(sg, setup, oracle):
    ctx, ix, reqs, ref = setup
    p = params(sg)
    srv = sg.Server(ix, params=p, workers=2)
    try:
        tickets = [srv.submit(r) for r in reqs]
        results = [srv.wait(t) for t in tickets]
    finally:
        srv.close()
    merged = 0
    for r, (got, st) in zip(reqs, results):
        assert got == ctx.align(ix, r, p)
        assert st["reads"] == r.count(b">") and st["out_bytes"] == len(got)
        assert 0 <= st["queue_ms"] <= st["total_ms"] and st["device_ms"] > 0
        merged += st["wave_requests"] > 1
    assert merged > 0  # requests did share waves
    # and the same records as the oracle on a few of them (long reads too)
    op = oracle.default_params(device_mem=ctx.info()["total_mem"], max_read_len=300)
    sess = oracle.Session(ref, op)
    for r, (got, _) in list(zip(reqs, results))[:10]:
        assert got == sess.align(r)


def test_server_waves_mix_query_lengths(sg, setup):
    # one worker: every request queued behind the first shares a wave with
    # the others of its query-length class; each still gets its own records
    ctx, ix, reqs, _ = setup
    p = params(sg)
    srv = sg.Server(ix, params=p, workers=1)
    try:
        tickets = [srv.submit(r) for r in reqs]
        results = [srv.wait(t) for t in tickets]
    finally:
        srv.close()
    assert max(st["wave_requests"] for _, st in results) >= 3
    for r, (got, st) in zip(reqs, results):
        assert got == ctx.align(ix, r, p)


def test_server_failed_request_and_tiny_budget(sg, setup):
    ctx, ix, reqs, _ = setup
    p = params(sg)
    srv = sg.Server(ix, params=p, workers=2, mem_budget=1)  # every request alone
    try:
        t0 = srv.submit(reqs[0])
        bad = srv.submit(b">a\nACGT\n\n>b\nACGT\n")  # empty line: rejected
        short = srv.submit(b">a\nACGTACGTAC\n>b\nACG\n")  # a read shorter than the query
        long = srv.submit(b">a\n" + b"A" * 301 + b"\n")  # beyond max_read_len
        t1 = srv.submit(reqs[1])
        assert srv.wait(t0)[0] == ctx.align(ix, reqs[0], p)
        for t, code, text in [(bad, -2, "empty line"), (short, -2, "shorter"),
                              (long, -5, "longer than 300")]:
            with pytest.raises(sg.SwiftError) as e:
                srv.wait(t)
            assert e.value.code == code and text in str(e.value)
        assert srv.wait(t1)[0] == ctx.align(ix, reqs[1], p)
    finally:
        srv.close()


BAD_INPUTS = [b">a\nACGT\n\n>b\nACGT\n", b">a\nACGT\nACGT\n", b">a\n", b">a\nAC>GT\n",
              b">a\n" + b"A" * 350 + b"\n", b">" + b"n" * 60 + b"\nACGT\n", b"ACGT\n>a\nACGT\n",
              b">a\n>b\nACGT\n", b">a\nAC\x00GT\n", b">a\nAC\xc3GT\n", b">a\nACGT\n>b\n",
              b"", b">a\nACGT\n>b\nAC\n", b">a\r\nACGT\r\n>b\nACG"]


def test_server_checks_match_swift_align(sg, setup):
    # requests are parsed on the host by the worker that takes them: every
    # malformed input fails there, alone, with swift_align's status and message
    ctx, ix, _, _ = setup
    p = params(sg)
    srv = sg.Server(ix, params=p, workers=1)
    try:
        for bad in BAD_INPUTS:
            t = srv.submit(bad)
            try:
                want = ctx.align(ix, bad, p)
            except sg.SwiftError as e:
                want = e
            try:
                got = srv.wait(t)[0]
            except sg.SwiftError as e:
                got = e
            if isinstance(want, sg.SwiftError):
                assert isinstance(got, sg.SwiftError), bad
                assert (got.code, str(got)) == (want.code, str(want)), bad
            else:
                assert got == want, bad
    finally:
        srv.close()


def test_server_poll_and_cancel(sg, setup):
    ctx, ix, reqs, _ = setup
    p = params(sg)
    # a budget that admits one request at a time keeps the rest queued
    srv = sg.Server(ix, params=p, workers=1, mem_budget=1)
    try:
        big = max(reqs, key=len)
        tickets = [srv.submit(big) for _ in range(3)] + [srv.submit(reqs[2])]
        last = tickets[-1]
        assert srv.poll(last) in ("queued", "running", "done")
        cancelled = srv.cancel(last)
        if cancelled:
            assert srv.poll(last) == "cancelled"
            with pytest.raises(sg.SwiftError) as e:
                srv.wait(last)
            assert e.value.code == -7
        else:  # it had started already: its result stands
            assert srv.wait(last)[0] == ctx.align(ix, reqs[2], p)
        want = ctx.align(ix, big, p)
        for t in tickets[:3]:
            assert srv.wait(t)[0] == want
        done = srv.submit(reqs[3])
        srv.wait(done)
        with pytest.raises(sg.SwiftError):
            srv.poll(done)  # released by wait
        with pytest.raises(sg.SwiftError):
            srv.cancel(123456789)
    finally:
        srv.close()
