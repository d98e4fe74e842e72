"""Pairs of varying lengths (swift_sw_pairs) against the oracle, pair by pair.

Each pair is aligned on its own query and window lengths; the batched mode
(shape-sorted launches, packed passes for ACGT pairs) and the plain mode
(everything padded to the largest shape, int32 kernel) must both reproduce
the oracle's score, coordinates and consensus strings exactly.
"""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from swift_gb300 import build as b
    b.build()
    import swift_gb300
    return swift_gb300


@pytest.fixture(scope="module")
def ctx(sg):
    return sg.Context(0)


@pytest.fixture(scope="module")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


def make_pairs(n, seed, q_range=(20, 250), extra=(20, 140), odd_every=9):
    """Reads with a mutated copy inside their window; every odd_every-th pair
    carries N, lowercase or IUPAC bytes (the int32 kernel's pairs)."""
    rng = random.Random(seed)
    qs, ws = [], []
    for i in range(n):
        Q = rng.randint(*q_range)
        R = min(1024 if Q <= 128 else 768, Q + rng.randint(*extra))
        w = bytearray(rng.choice(b"ACGT") for _ in range(R))
        a = rng.randrange(0, max(1, R - Q))
        q = bytearray(w[a:a + Q])
        while len(q) < Q:
            q.append(rng.choice(b"ACGT"))
        for k in range(Q):
            r = rng.random()
            if r < 0.03:
                q[k] = rng.choice(b"ACGT")
        if rng.random() < 0.2:  # an indel
            k = rng.randrange(1, Q - 1)
            q = q[:k] + q[k + 1:] + bytearray([rng.choice(b"ACGT")]) if rng.random() < 0.5 \
                else q[:k] + bytearray([rng.choice(b"ACGT")]) + q[k:-1]
        if i % 4 == 3:  # a decoy window
            w = bytearray(rng.choice(b"ACGT") for _ in range(R))
        if odd_every and i % odd_every == 5:
            q[rng.randrange(Q)] = ord("N")
            w[rng.randrange(R)] = rng.choice(b"nRy")
            q[: Q // 4] = q[: Q // 4].lower()
        qs.append(bytes(q))
        ws.append(bytes(w))
    return qs, ws


def pack(items):
    off = np.zeros(len(items), np.int64)
    ln = np.array([len(x) for x in items], np.int32)
    off[1:] = np.cumsum(ln[:-1])
    return b"".join(items), off, ln


def check_against_oracle(res, qs, ws, oracle, params):
    m, x, o, e = params
    for i, (q, w) in enumerate(zip(qs, ws)):
        want = oracle.sw(q, w, m=m, x=x, o=o, e=e)
        got = (int(res["score"][i]), int(res["start"][i]), int(res["end"][i]), int(res["len"][i]))
        assert got == (int(want["score"]), want["start"], want["end"], want["len"]), (i, got, want)
        if "qcons" in res:
            assert res["qcons"][i] == want["qcons"] and res["rcons"][i] == want["rcons"], i


@pytest.mark.parametrize("mode", [0, 1])
def test_pairs_vs_oracle(ctx, oracle, mode):
    qs, ws = make_pairs(1500, seed=7 + mode)
    qb, qo, ql = pack(qs)
    wb, wo, wl = pack(ws)
    res, st = ctx.sw_pairs(qb, qo, ql, wb, wo, wl, mode=mode)
    check_against_oracle(res, qs, ws, oracle, (2, -1, -10, -1))
    assert st["pairs"] == len(qs) and st["cells"] == int((ql.astype(np.int64) * wl).sum())
    if mode == 0:
        assert st["segments"] > 10 and 0 < st["generic_pairs"] < len(qs)


def test_pairs_modes_agree_and_coordinates_only(ctx, oracle):
    qs, ws = make_pairs(3000, seed=21, q_range=(36, 128), extra=(128, 128), odd_every=0)
    qb, qo, ql = pack(qs)
    wb, wo, wl = pack(ws)
    a, sa = ctx.sw_pairs(qb, qo, ql, wb, wo, wl, mode=0)
    b, _ = ctx.sw_pairs(qb, qo, ql, wb, wo, wl, mode=1)
    c, _ = ctx.sw_pairs(qb, qo, ql, wb, wo, wl, mode=0, consensus=False)
    for k in ("score", "start", "end", "len"):
        assert np.array_equal(a[k], b[k]) and np.array_equal(a[k], c[k]), k
    assert a["qcons"] == b["qcons"] and a["rcons"] == b["rcons"]
    assert sa["generic_pairs"] == 0  # every pair on the packed passes
    check_against_oracle(a, qs[:400], ws[:400], oracle, (2, -1, -10, -1))


def test_pairs_shared_buffers_and_parameters(ctx, oracle):
    # pairs may share query and window bytes (a read against many regions)
    rng = random.Random(5)
    ref = bytes(rng.choice(b"ACGT") for _ in range(20000))
    reads = [ref[p:p + L] for p, L in ((1000, 80), (5000, 150), (12000, 40))]
    qb, qo_r, ql_r = pack(reads)
    q_off, q_len, r_off, r_len = [], [], [], []
    for r in range(3):
        for t in range(40):
            pos = rng.randrange(0, 20000 - 300)
            q_off.append(qo_r[r]); q_len.append(ql_r[r])
            r_off.append(pos); r_len.append(rng.randint(50, 300))
    qs = [qb[a:a + b] for a, b in zip(q_off, q_len)]
    ws = [ref[a:a + b] for a, b in zip(r_off, r_len)]
    for params in [(2, -1, -10, -1), (3, -2, -5, -2), (1, -3, -4, -1)]:
        res, _ = ctx.sw_pairs(qb, q_off, q_len, ref, r_off, r_len, *params)
        check_against_oracle(res, qs, ws, oracle, params)


def test_pairs_limits(ctx, sg):
    qb, wb = b"A" * 5000, b"A" * 9000
    for ql, wl, code in [(4097, 100, -5), (200, 8193, -5), (0, 10, -1)]:
        with pytest.raises(sg.SwiftError) as e:
            ctx.sw_pairs(qb, [0], [ql], wb, [0], [wl])
        assert e.value.code == code
    with pytest.raises(sg.SwiftError) as e:  # plain mode needs negative penalties
        ctx.sw_pairs(qb, [0], [10], wb, [0], [10], 2, 1, -10, -1, mode=1)
    assert e.value.code == -1
    res, st = ctx.sw_pairs(b"", [], [], b"", [], [])
    assert st["pairs"] == 0 and len(res["score"]) == 0


def test_pairs_batched_workload_vs_oracle(ctx, oracle):
    # the batched workload's shapes: reads of 36-250 bp against 1-64 regions
    # each (true region and decoys, 64 bp flanks), on a small reference
    from swift_gb300 import synth
    _, seqs = synth.make_reference(2_000_000, 3, sigma=0.5, repeat_frac=0.1, seed=41)
    ref, reads, qo, ql, ro, rl = synth.pairs_workload(150, seed=42, ref=seqs)
    res, st = ctx.sw_pairs(reads, qo, ql, ref, ro, rl)
    assert 1 <= st["segments"] <= 21  # one launch set per row class (32 to 256 rows)
    qs = [reads[a:a + b] for a, b in zip(qo, ql)]
    ws = [ref[a:a + b] for a, b in zip(ro, rl)]
    check_against_oracle(res, qs, ws, oracle, (2, -1, -10, -1))
    plain, _ = ctx.sw_pairs(reads, qo, ql, ref, ro, rl, mode=1, consensus=False)
    for k in ("score", "start", "end", "len"):
        assert np.array_equal(plain[k], res[k]), k


def test_pairs_every_shape_and_autotuner_agree(ctx, oracle, sg):
    # every (lanes, rows per lane) candidate of each query class, and the
    # autotuner's choice, give the default shapes' results exactly
    from swift_gb300 import synth
    _, seqs = synth.make_reference(2_000_000, 3, sigma=0.5, repeat_frac=0.1, seed=43)
    ref, reads, qo, ql, ro, rl = synth.pairs_workload(700, seed=44, ref=seqs)
    c2 = sg.Context(0)
    try:
        c2.set_tuning(0)
        base, _ = c2.sw_pairs(reads, qo, ql, ref, ro, rl)
        seen = set()
        for k in range(2, 2 + 12):
            c2.set_tuning(k)
            res, st = c2.sw_pairs(reads, qo, ql, ref, ro, rl)
            seen |= {(q, s) for q, s in st["shapes"].items()}
            for key in ("score", "start", "end", "len", "qcons", "rcons"):
                assert res[key] == base[key] if key in ("qcons", "rcons") else \
                    np.array_equal(res[key], base[key]), (k, key)
        assert len(seen) > 7  # more than one shape per class ran
        c2.set_tuning(1)
        res, st = c2.sw_pairs(reads, qo, ql, ref, ro, rl)
        assert st["tune_ms"] > 0 and st["shapes"]
        for key in ("score", "start", "end", "len"):
            assert np.array_equal(res[key], base[key]), key
        res2, st2 = c2.sw_pairs(reads, qo, ql, ref, ro, rl)  # choices kept
        assert st2["tune_ms"] == 0 and st2["shapes"] == st["shapes"]
    finally:
        c2.close()
    rng = random.Random(45)
    pick = rng.sample(range(len(ql)), 300)
    sub = {k: np.asarray(base[k])[pick] for k in ("score", "start", "end", "len")}
    check_against_oracle(sub, [reads[qo[i]:qo[i] + ql[i]] for i in pick],
                         [ref[ro[i]:ro[i] + rl[i]] for i in pick], oracle, (2, -1, -10, -1))


def test_long_pairs_vs_oracle(ctx, oracle):
    # long queries and windows (the long-region shapes: queries to 4000,
    # windows to 8000) next to short pairs in one call
    rng = random.Random(91)
    qs, ws = [], []
    for Q, R in [(300, 600), (1000, 2000), (1500, 1200), (2100, 4000), (3000, 3500),
                 (4000, 8000), (257, 300), (150, 1000), (64, 2000), (3500, 5000)]:
        w = bytearray(rng.choice(b"ACGT") for _ in range(R))
        a = rng.randrange(0, max(1, R - Q))
        q = bytearray(w[a:a + Q])
        while len(q) < Q:
            q.append(rng.choice(b"ACGT"))
        for k in range(Q):
            if rng.random() < 0.03:
                q[k] = rng.choice(b"ACGT")
        for _ in range(Q // 400):  # indels, length kept
            k = rng.randrange(1, Q - 3)
            if rng.random() < 0.5:
                q = q[:k] + q[k + 2:] + bytearray(b"AC")
            else:
                q = q[:k] + bytearray(b"GT") + q[k:-2]
        q[rng.randrange(Q)] = ord("N")
        w[rng.randrange(R)] = ord("n")
        if Q in (1000, 3000):  # lowercase runs (still ACGTN pairs)
            q[: Q // 5] = q[: Q // 5].lower()
            w[R // 2:] = w[R // 2:].lower()
        if Q in (1500, 3500):  # IUPAC bytes: the byte-compare path
            q[rng.randrange(Q)] = ord("R")
            w[rng.randrange(R)] = ord("y")
        qs.append(bytes(q))
        ws.append(bytes(w))
    # no cell above zero, and a single matching base: first-maximum ties
    qs += [b"A" * 300, b"A" * 1100]
    ws += [b"C" * 900, b"C" * 700 + b"A" + b"C" * 600]
    sq, sw_ = make_pairs(40, seed=92)
    qs += sq
    ws += sw_
    qb, qo, ql = pack(qs)
    wb, wo, wl = pack(ws)
    res, st = ctx.sw_pairs(qb, qo, ql, wb, wo, wl)
    check_against_oracle(res, qs, ws, oracle, (2, -1, -10, -1))
    res2, _ = ctx.sw_pairs(qb, qo, ql, wb, wo, wl, 3, -2, -5, -2)
    check_against_oracle(res2, qs, ws, oracle, (3, -2, -5, -2))
    # a match score whose largest cells leave the profile path's key range
    # for 4000-row queries, and a large gap-open bias
    res3, _ = ctx.sw_pairs(qb, qo, ql, wb, wo, wl, 5, -3, -40, -2)
    check_against_oracle(res3, qs, ws, oracle, (5, -3, -40, -2))


def test_long_workload_vs_oracle(ctx, oracle):
    # the long-region workload's shapes on a small reference
    from swift_gb300 import synth
    ref, qry, qo, ql, ro, rl = synth.long_workload(24, seed=93, ref_bp=2_000_000)
    res, st = ctx.sw_pairs(qry, qo, ql, ref, ro, rl)
    qs = [qry[a:a + b] for a, b in zip(qo, ql)]
    ws = [ref[a:a + b] for a, b in zip(ro, rl)]
    check_against_oracle(res, qs, ws, oracle, (2, -1, -10, -1))
    assert (res["score"] > 1000).all()  # every query aligns across its region
