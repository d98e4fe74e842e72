"""Serving loop: every request's records equal swift_align on it alone.

Requests of different sizes and read lengths run concurrently on several
pipelines; a malformed request fails alone; a memory budget smaller than
any request still serves them (one at a time).
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
    ix = ctx.index(synth.fasta_bytes(names, seqs))
    rng = random.Random(72)
    reqs = []
    for t in range(24):
        n = int(10 ** rng.uniform(0, 3.3))  # 1 .. 2000 reads
        L = rng.randint(50, 199)
        rn, rs, _ = synth.make_reads(seqs, n, L, 0.01, 0.001, 0.05, seed=100 + t)
        reqs.append(synth.reads_fasta([f"q{t}_{i}" for i in range(n)], rs))
    return ctx, ix, reqs


def test_server_matches_single_requests(sg, setup):
    ctx, ix, reqs = setup
    srv = sg.Server(ix, workers=3)
    try:
        tickets = [srv.submit(r) for r in reqs]
        results = [srv.wait(t) for t in tickets]
    finally:
        srv.close()
    for r, (got, st) in zip(reqs, results):
        assert got == ctx.align(ix, r)
        assert st["reads"] == r.count(b">") and st["out_bytes"] == len(got)
        assert 0 <= st["queue_ms"] <= st["total_ms"] and st["device_ms"] > 0


def test_server_failed_request_and_tiny_budget(sg, setup):
    ctx, ix, reqs = setup
    srv = sg.Server(ix, workers=2, mem_budget=1)  # every request alone
    try:
        t0 = srv.submit(reqs[0])
        bad = srv.submit(b">a\nACGT\n\n>b\nACGT\n")  # empty line: rejected
        t1 = srv.submit(reqs[1])
        assert srv.wait(t0)[0] == ctx.align(ix, reqs[0])
        with pytest.raises(sg.SwiftError) as e:
            srv.wait(bad)
        assert e.value.code == -2 and "empty line" in str(e.value)
        assert srv.wait(t1)[0] == ctx.align(ix, reqs[1])
    finally:
        srv.close()
