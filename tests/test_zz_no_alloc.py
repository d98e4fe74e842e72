"""swift_sw_batch_noalloc (static scratch, no allocation) against swift_sw_batch
and against the oracle.

Collected last on purpose: it must pass both in a fresh process and after
every other test has run on the same device.  Both entry points are called
through the C ABI; every output is integer-valued, so the comparison is exact.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PAIRS = 65536


@pytest.fixture(scope="module")
def sg():
    from swift_gb300 import build as b
    b.build()
    import swift_gb300
    return swift_gb300


@pytest.fixture(scope="module")
def ctx(sg):
    return sg.Context(0)


def make_pairs(n, Q, R, seed):
    """Seeded query/window buffers in the alignSequences layout: query i at
    i*(Q+1), window i at i*(R+1).  Queries are mutated copies of a window
    slice (so most pairs align well); a few carry N or lowercase bytes."""
    rng = np.random.default_rng(seed)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    w = np.zeros((n, R + 1), np.uint8)
    q = np.zeros((n, Q + 1), np.uint8)
    w[:, :R] = acgt[rng.integers(0, 4, (n, R))]
    for i in range(n):
        off = int(rng.integers(0, max(R - Q, 0) + 1))
        src = w[i, off:off + Q].copy()
        if len(src) < Q:
            src = np.concatenate([src, acgt[rng.integers(0, 4, Q - len(src))]])
        sub = rng.random(Q) < 0.05
        src[sub] = acgt[rng.integers(0, 4, int(sub.sum()))]
        q[i, :Q] = src
        if i % 97 == 0:
            q[i, int(rng.integers(0, Q))] = ord("N")
            w[i, int(rng.integers(0, R))] = ord("n")
        if i % 89 == 0:
            q[i, :Q // 3] |= 0x20  # lowercase run
    return q, w


def run_host(sg, ctx, q, w, Q, R, n, params):
    cs = Q + R + 2
    out = dict(score=np.zeros(n, np.float32), start=np.zeros(n, np.int32),
               end=np.zeros(n, np.int32), len=np.zeros(n, np.int32),
               qcons=np.zeros((n, cs), np.uint8), rcons=np.zeros((n, cs), np.uint8))
    rc = sg.lib().swift_sw_batch(
        ctx._h, q.ctypes.data, w.ctypes.data, Q, R, n, *params,
        *(out[k].ctypes.data for k in ("score", "start", "end", "len", "qcons", "rcons")))
    assert rc == 0, sg.lib().swift_last_error(ctx._h)
    return out


def run_noalloc(sg, ctx, q, w, Q, R, n, params):
    import torch
    cs = Q + R + 2
    dq = torch.from_numpy(q).cuda()
    dw = torch.from_numpy(w).cuda()
    d = dict(score=torch.empty(n, dtype=torch.float32, device="cuda"),
             start=torch.empty(n, dtype=torch.int32, device="cuda"),
             end=torch.empty(n, dtype=torch.int32, device="cuda"),
             len=torch.empty(n, dtype=torch.int32, device="cuda"),
             qcons=torch.zeros((n, cs), dtype=torch.uint8, device="cuda"),
             rcons=torch.zeros((n, cs), dtype=torch.uint8, device="cuda"))
    torch.cuda.synchronize()
    rc = sg.lib().swift_sw_batch_noalloc(
        ctx._h, dq.data_ptr(), dw.data_ptr(), Q, R, n, *params,
        *(d[k].data_ptr() for k in ("score", "start", "end", "len", "qcons", "rcons")))
    assert rc == 0, sg.lib().swift_last_error(ctx._h)
    torch.cuda.synchronize()  # the call only enqueues; the device-wide sync covers its stream
    return {k: v.cpu().numpy() for k, v in d.items()}


def assert_same(got, want, n):
    for k in ("score", "start", "end", "len"):
        assert np.array_equal(got[k], want[k]), k
    for i in range(n):
        L = int(want["len"][i])
        assert bytes(got["qcons"][i, :L]) == bytes(want["qcons"][i, :L]), i
        assert bytes(got["rcons"][i, :L]) == bytes(want["rcons"][i, :L]), i


def test_noalloc_matches_sw_batch_two_calls(sg, ctx):
    pytest.importorskip("torch")
    cases = [(5000, 100, 300, (2, -1, -10, -1), 11),
             (3001, 64, 200, (3, -2, -5, -2), 12)]
    for n, Q, R, params, seed in cases:  # two calls in a row, different shapes
        q, w = make_pairs(n, Q, R, seed)
        want = run_host(sg, ctx, q, w, Q, R, n, params)
        got = run_noalloc(sg, ctx, q, w, Q, R, n, params)
        assert_same(got, want, n)
        assert (want["score"] > 0).mean() > 0.9  # the inputs do align


def test_noalloc_matches_oracle(sg, ctx, oracle):
    # the two entry points share the generic kernel, so the comparison above
    # alone could not catch an error in it: a few hundred pairs of each call
    # against the CPU restatement as well, two calls in a row
    pytest.importorskip("torch")
    for n, Q, R, params, seed in [(400, 100, 300, (2, -1, -10, -1), 21),
                                  (300, 150, 260, (3, -2, -6, -2), 22)]:
        q, w = make_pairs(n, Q, R, seed)
        got = run_noalloc(sg, ctx, q, w, Q, R, n, params)
        m, x, o, e = params
        for i in range(n):
            want = oracle.sw(bytes(q[i, :Q]), bytes(w[i, :R]), Q, R, m, x, o, e)
            L = want["len"]
            assert (float(got["score"][i]), int(got["start"][i]), int(got["end"][i]),
                    int(got["len"][i])) == (want["score"], want["start"], want["end"], L), i
            assert bytes(got["qcons"][i, :max(L, 0)]) == want["qcons"], i
            assert bytes(got["rcons"][i, :max(L, 0)]) == want["rcons"], i


def test_noalloc_largest_batch(sg, ctx):
    pytest.importorskip("torch")
    n, Q, R, params = MAX_PAIRS, 40, 60, (2, -1, -10, -1)
    q, w = make_pairs(n, Q, R, 13)
    want = run_host(sg, ctx, q, w, Q, R, n, params)
    got = run_noalloc(sg, ctx, q, w, Q, R, n, params)
    assert_same(got, want, n)


def test_noalloc_rejects(sg, ctx):
    torch = pytest.importorskip("torch")
    lib = sg.lib()
    Q, R = 10, 20
    buf = torch.zeros(1 << 16, dtype=torch.uint8, device="cuda")
    p = buf.data_ptr()
    # more pairs than the static scratch holds: refused before any launch
    rc = lib.swift_sw_batch_noalloc(ctx._h, p, p, Q, R, MAX_PAIRS + 1, 2, -1, -10, -1,
                                    p, p, p, p, p, p)
    assert rc == -5 and b"65536" in lib.swift_last_error(ctx._h)
    # a host pointer is refused
    host = np.zeros(64, np.uint8)
    rc = lib.swift_sw_batch_noalloc(ctx._h, host.ctypes.data, p, Q, R, 1, 2, -1, -10, -1,
                                    p, p, p, p, p, p)
    assert rc == -1
    # sizes beyond the kernel's limits
    rc = lib.swift_sw_batch_noalloc(ctx._h, p, p, 400, R, 1, 2, -1, -10, -1, p, p, p, p, p, p)
    assert rc == -5
    # scores that are not whole numbers (alignSequences takes floats; the
    # reference parses them with atoi)
    rc = lib.swift_sw_batch_noalloc(ctx._h, p, p, Q, R, 1, 2.5, -1, -10, -1, p, p, p, p, p, p)
    assert rc == -1
    # an empty batch is a no-op
    rc = lib.swift_sw_batch_noalloc(ctx._h, p, p, Q, R, 0, 2, -1, -10, -1, p, p, p, p, p, p)
    assert rc == 0
