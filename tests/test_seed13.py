"""lt13 seed-and-extend seeding (search2Queries) on the GPU against the oracle.

The oracle's restatement is pinned to the reference's own lookupTable13
kernel by tests/test_oracle_vs_reference.py and the golden fixture
pipeline_out_lt13.txt; here the device path must reproduce it record for
record (Phase 1) and byte for byte (whole pipeline, both output formats).
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
def ctx(sg):
    return sg.Context(0)


@pytest.fixture(scope="module")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


def rand_seq(rng, n):
    return bytes(rng.choice(b"ACGT") for _ in range(n))


def mutate(rng, s, p_sub, p_indel):
    out = bytearray()
    for c in s:
        x = rng.random()
        if x < p_indel / 2:
            continue
        if x < p_indel:
            out += rand_seq(rng, rng.randint(1, 3))
        out.append(rng.choice(b"ACGT") if rng.random() < p_sub else c)
    return bytes(out)


def revcomp(s):
    comp = {ord("A"): ord("T"), ord("C"): ord("G"), ord("G"): ord("C")}
    return bytes(comp.get(c, ord("A")) for c in reversed(s))


def make_case(seed, n_refs, ref_len, n_reads, read_len, unit=None, n_frac=0.0):
    """References (random or copies of one unit), reads from both strands,
    some at sequence ends, some with lowercase and N; the first read is the
    shortest (Phase 2 aligns every read on the first read's length)."""
    rng = random.Random(seed)
    seqs = []
    for _ in range(n_refs):
        if unit:
            u = rand_seq(rng, unit)
            s = bytearray()
            while len(s) < ref_len:
                s += mutate(rng, u, 0.02, 0.0)
            s = bytes(s[:ref_len])
        else:
            s = rand_seq(rng, ref_len)
        if n_frac:
            s = bytes(c if rng.random() > n_frac else ord("N") for c in s)
        seqs.append(s)
    ref = b"".join(b">s%d\n" % i + b"\n".join(s[j:j + 60] for j in range(0, len(s), 60)) + b"\n"
                   for i, s in enumerate(seqs))
    reads = []
    for i in range(n_reads):
        s = seqs[rng.randrange(n_refs)]
        L = read_len if isinstance(read_len, int) else (
            read_len[0] if i == 0 else rng.randint(*read_len))
        if i % 5 == 4:
            a = len(s) - L + rng.randrange(0, 8)
            r = (s[a:] + rand_seq(rng, L))[:L]
        else:
            a = rng.randrange(0, len(s) - L - 20)
            r = mutate(rng, s[a:a + L + 10], 0.03, 0.01)[:L].ljust(L, b"G")
        if i % 2:
            r = revcomp(r)
        if i % 7 == 3:
            r = r[:L // 2].lower() + b"N" + r[L // 2 + 1:]
        reads.append(b">q%d\n%s\n" % (i, r))
    return ref, b"".join(reads)


CASES = [
    dict(n_refs=2, ref_len=9000, n_reads=200, read_len=100, k=12, t=1000),
    dict(n_refs=5, ref_len=4000, n_reads=200, read_len=(13, 150), k=12, t=1000, n_frac=0.01),
    dict(n_refs=1, ref_len=12000, n_reads=120, read_len=90, k=8, t=300, unit=120),
    dict(n_refs=3, ref_len=6000, n_reads=120, read_len=(8, 60), k=6, t=1000, unit=40),
    dict(n_refs=2, ref_len=5000, n_reads=120, read_len=100, k=10, t=5),
    dict(n_refs=64, ref_len=700, n_reads=150, read_len=100, k=11, t=1000),
]


@pytest.mark.parametrize("seed,case", list(enumerate(CASES)))
def test_lt13_records_and_pipeline(ctx, oracle, sg, seed, case):
    kw = {k: v for k, v in case.items() if k not in ("k", "t")}
    ref, reads = make_case(2300 + seed, **kw)
    ix = ctx.index(ref, case["k"], case["t"])
    op = oracle.default_params(seed_len=case["k"], ignore_thres=case["t"], seeder=1,
                               device_mem=ctx.info()["total_mem"])
    want = oracle.phase1(ref, reads, op)
    got = ctx.seed_lt13(ix, reads)
    assert got == want
    for fmt in (0, 1):
        p = sg.default_params(seed_len=case["k"], ignore_thres=case["t"], seeder=1,
                              out_format=fmt)
        op.out_format = fmt
        assert ctx.align(ix, reads, p) == oracle.align(ref, reads, op), fmt


def test_lt13_full_arrays_path(ctx, oracle, sg):
    # 1100 exact copies of a 12-base unit, k = 6, threshold 1100: a query
    # tuple has 1100 hits with the same match count, so the kept entries
    # pass the fast kernel's arrays (full-array path) and the reference's
    # 1000-entry reset fires
    rng = random.Random(78)
    u = rand_seq(rng, 12)
    s = u * 1100
    ref = b">rep\n" + b"\n".join(s[j:j + 60] for j in range(0, len(s), 60)) + b"\n"
    reads = b"".join(b">r%d\n%s\n" % (i, s[a:a + 90])
                     for i, a in enumerate(rng.randrange(0, 13000) for _ in range(40)))
    reads += b">tail\n" + s[-50:] + rand_seq(rng, 40) + b"\n"
    ix = ctx.index(ref, 6, 1100)
    op = oracle.default_params(seed_len=6, ignore_thres=1100, seeder=1,
                               device_mem=ctx.info()["total_mem"])
    assert ctx.seed_lt13(ix, reads) == oracle.phase1(ref, reads, op)
    got, st = ctx.align(ix, reads, sg.default_params(seed_len=6, ignore_thres=1100, seeder=1),
                        stats=True)
    assert st["seed_overflow_strands"] > 0
    assert got == oracle.align(ref, reads, op)


def test_lt13_limits(ctx, sg):
    rng = random.Random(5)
    many = b"".join(b">c%d\n%s\n" % (i, rand_seq(rng, 100)) for i in range(65))
    ix = ctx.index(many)
    with pytest.raises(sg.SwiftError) as e:
        ctx.seed_lt13(ix, b">r\n" + rand_seq(rng, 50) + b"\n")
    assert e.value.code == -5
    ix2 = ctx.index(b">a\n" + rand_seq(rng, 5000) + b"\n", 12, 1177)
    with pytest.raises(sg.SwiftError) as e:
        ctx.align(ix2, b">r\n" + rand_seq(rng, 50) + b"\n", sg.default_params(ignore_thres=1177,
                                                                              seeder=1))
    assert e.value.code == -5
    with pytest.raises(sg.SwiftError) as e:
        ctx.align(ix2, b">r\n" + rand_seq(rng, 50) + b"\n", sg.default_params(ignore_thres=1177,
                                                                              seeder=2))
    assert e.value.code == -1
