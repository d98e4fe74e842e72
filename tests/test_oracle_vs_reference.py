"""The oracle against the reference's own code on seeded random inputs.

Runs only where oracle/_ref was built from the reference sources (the build
container); elsewhere the committed fixtures of test_golden_fixtures.py
carry the same check.
"""
import random

import pytest

from oracle import ref as R

pytestmark = pytest.mark.skipif(not R.available(), reason="reference harness not built")


def rand_seq(rng, n, alphabet=b"ACGT"):
    return bytes(rng.choice(alphabet) for _ in range(n))


def mutate(rng, s, p_sub=0.04, p_indel=0.02):
    out = bytearray()
    for c in s:
        x = rng.random()
        if x < p_indel / 2:
            continue
        if x < p_indel:
            out += rand_seq(rng, rng.randint(1, 3))
        out.append(rng.choice(b"ACGT") if rng.random() < p_sub else c)
    return bytes(out)


def test_sw_kernel_random(oracle):
    rng = random.Random(5)
    for i in range(60):
        Q, Rl = rng.choice([(100, 300), (12, 40), (50, 120), (30, 300)])
        w = rand_seq(rng, Rl, b"ACGTacgtN" if i % 4 == 3 else b"ACGT")
        if i % 3:
            a = rng.randrange(0, max(1, Rl - Q))
            q = mutate(rng, w[a:a + Q + 5].upper())[:Q].ljust(Q, b"C")
        else:
            q = rand_seq(rng, Q)
        if i % 5 == 2:
            w = w[: rng.randint(Q // 2, Rl)]
        want = R.sw_kernel(q, w, Q, Rl)
        got = oracle.sw(q, w, Q, Rl)
        assert {k: got[k] for k in want} == want, (i, q, w)


def test_sw_kernel_scoring(oracle):
    rng = random.Random(6)
    for m, x, o, e in [(1, -3, -5, -2), (5, -4, -20, -1), (2, -1, -1, -1)]:
        for _ in range(5):
            w = rand_seq(rng, 150)
            q = mutate(rng, w[20:90])[:60].ljust(60, b"G")
            want = R.sw_kernel(q, w, 60, 150, m, x, o, e)
            got = oracle.sw(q, w, 60, 150, m, x, o, e)
            assert {k: got[k] for k in want} == want


def test_cpu_sw_agrees_on_score_and_end(oracle):
    # the reference's CPU routine has the same DP and maximum cell; its
    # traceback may continue through zero cells, so only score and end are
    # compared (src/smithWaterman.cu:194-210, 263-335)
    rng = random.Random(7)
    for _ in range(40):
        w = rand_seq(rng, 300)
        q = mutate(rng, w[50:160])[:100].ljust(100, b"T")
        a = R.sw_cpu(q, w)
        b = oracle.sw(q, w)
        assert a["score"] == b["score"] and a["end"] == b["end"]


def test_index_and_map_query(oracle):
    rng = random.Random(8)
    parts = []
    seqs = []
    for r in range(3):
        s = rand_seq(rng, rng.randint(3000, 6000))
        unit = rand_seq(rng, 48)
        s = s[:1000] + unit * 30 + s[1000:]
        seqs.append(s)
        w = rng.choice([60, 61, 50])
        parts.append(b">c%d\n" % r + b"\n".join(s[i:i + w] for i in range(0, len(s), w)) + b"\n")
    fa = b"".join(parts)
    for k, t in [(12, 1000), (8, 10)]:
        look, rep, ri, rp = R.index(fa, k, t)
        ox = oracle.Index(fa, k, t)
        ori, orp = ox.postings()
        assert list(ori) == ri and list(orp) == rp
        assert all(ox.start(h) == look[h] and ox.repeats(h) == rep[h]
                   for h in range(0, len(look), 7))
        for _ in range(40):
            s = seqs[rng.randrange(3)]
            a = rng.randrange(0, len(s) - 100)
            q = mutate(rng, s[a:a + 100], 0.02, 0.005)[:100]
            rc = oracle.revcomp(q)
            assert R.map_query(q, rc, 0) == ox.map_query(q, 3)
            assert R.map_query(q, rc, 1) == ox.map_query(rc, 3)


def test_pipeline_random(oracle):
    rng = random.Random(9)
    seqs = [rand_seq(rng, n) for n in (7000, 5000)]
    ref = b"".join(b">s%d\n" % i + b"\n".join(s[j:j + 60] for j in range(0, len(s), 60)) + b"\n"
                   for i, s in enumerate(seqs))
    reads = []
    for i in range(37):
        s = seqs[rng.randrange(2)]
        a = rng.randrange(0, len(s) - 110)
        r = mutate(rng, s[a:a + 110], 0.02, 0.005)[:100].ljust(100, b"A")
        if i % 2:
            r = oracle.revcomp(r)
        reads.append(b">q%d\n%s\n" % (i, r))
    reads = b"".join(reads)
    dm = 288_000_000_000
    want = R.pipeline(ref, reads, dm)
    got = oracle.align(ref, reads, oracle.default_params(device_mem=dm))
    assert got == want


def test_pipeline_sam_random(oracle):
    # SAM records (-f 1): every record of every batch, CIGAR from the
    # reversed consensus; small batches so the stale repeats and batch ends
    # are in the output, reads with indels so D and I runs appear
    rng = random.Random(10)
    seqs = [rand_seq(rng, n) for n in (6000, 4000, 3000)]
    ref = b"".join(b">chr%d\n" % i + b"\n".join(s[j:j + 60] for j in range(0, len(s), 60)) + b"\n"
                   for i, s in enumerate(seqs))
    reads = []
    for i in range(29):
        s = seqs[rng.randrange(3)]
        a = rng.randrange(0, len(s) - 110)
        r = mutate(rng, s[a:a + 110], 0.03, 0.02)[:90].ljust(90, b"C")
        if i % 3 == 1:
            r = oracle.revcomp(r)
        if i % 7 == 3:
            r = r[:40] + b"N" + r[41:]
        reads.append(b">read_%d\n%s\n" % (i, r))
    reads = b"".join(reads)
    for dm in (288_000_000_000, 100_000_000 + 17 * 1000):
        want = R.pipeline(ref, reads, dm, out_format=1)
        got = oracle.align(ref, reads, oracle.default_params(device_mem=dm, out_format=1))
        assert got == want
        assert want.count(b"\n") > 29 and b"D" in want and b"I" in want


def _lt13_case(rng, n_refs, ref_len, n_reads, read_len, unit=None, n_frac=0.0):
    seqs = []
    for i in range(n_refs):
        if unit:  # copies of one unit with light divergence: many equal hits
            u = rand_seq(rng, unit)
            s = bytearray()
            while len(s) < ref_len:
                s += mutate(rng, u, 0.02, 0.0)
            s = bytes(s[:ref_len])
        else:
            s = rand_seq(rng, ref_len)
        seqs.append(s)
    if n_frac:
        seqs = [bytes(c if rng.random() > n_frac else ord("N") for c in s) for s in seqs]
    ref = b"".join(b">c%d\n" % i + b"\n".join(s[j:j + 60] for j in range(0, len(s), 60)) + b"\n"
                   for i, s in enumerate(seqs))
    reads = []
    for i in range(n_reads):
        s = seqs[rng.randrange(n_refs)]
        # the first read is the shortest: Phase 2 aligns every read on the
        # first read's length (reads shorter than that read stale buffers)
        L = read_len if isinstance(read_len, int) else (
            read_len[0] if i == 0 else rng.randint(*read_len))
        if i % 5 == 4:  # a read at a sequence end (extensions walk past it)
            a = len(s) - L + rng.randrange(0, 8)
            r = (s[a:] + rand_seq(rng, L))[:L]
        else:
            a = rng.randrange(0, len(s) - L - 20)
            r = mutate(rng, s[a:a + L + 10], 0.03, 0.01)[:L].ljust(L, b"G")
        if i % 2:
            r = oracle_revcomp(r)
        if i % 7 == 3:
            r = r[:L // 2].lower() + b"N" + r[L // 2 + 1:]
        reads.append(b">q%d\n%s\n" % (i, r))
    return ref, b"".join(reads)


def oracle_revcomp(s):
    comp = {ord("A"): ord("T"), ord("C"): ord("G"), ord("G"): ord("C")}
    return bytes(comp.get(c, ord("A")) for c in reversed(s))


@pytest.mark.parametrize("seed,case", list(enumerate([
    dict(n_refs=2, ref_len=9000, n_reads=40, read_len=100, k=12, t=1000),
    dict(n_refs=4, ref_len=3000, n_reads=40, read_len=(13, 150), k=12, t=1000, n_frac=0.01),
    dict(n_refs=1, ref_len=12000, n_reads=30, read_len=90, k=8, t=300, unit=120),
    dict(n_refs=3, ref_len=6000, n_reads=30, read_len=(8, 60), k=6, t=1000, unit=40),
    dict(n_refs=2, ref_len=5000, n_reads=30, read_len=100, k=10, t=5),
])))
def test_lt13_phase1_and_pipeline(oracle, seed, case):
    # the reference's lookupTable13MapQry2_gpu (run on CPU fibers) against the
    # oracle's restatement: Phase-1 records and the whole default output
    rng = random.Random(1300 + seed)
    kw = {k: v for k, v in case.items() if k not in ("k", "t")}
    ref, reads = _lt13_case(rng, **kw)
    dm = 288_000_000_000
    out, recs = R.pipeline_with_matches(ref, reads, dm, seed_len=case["k"], thres=case["t"],
                                        seeder=1)
    p = oracle.default_params(device_mem=dm, seed_len=case["k"], ignore_thres=case["t"],
                              seeder=1)
    names = [l[1:].decode() for l in reads.split(b"\n") if l.startswith(b">")]
    got = [(names[r], s, ri, sh, rp) for r, s, ri, sh, rp in oracle.phase1(ref, reads, p)]
    assert got == recs
    assert oracle.align(ref, reads, p) == out
    assert len(recs) > 0


def test_lt13_kept_entries_reset(oracle):
    # 1100 exact copies of a 12-base unit, k = 6, threshold 1100: one query
    # tuple keeps more than 1000 entries, so the kernel's reset fires
    rng = random.Random(78)
    u = rand_seq(rng, 12)
    s = u * 1100
    ref = b">rep\n" + b"\n".join(s[j:j + 60] for j in range(0, len(s), 60)) + b"\n"
    reads = b"".join(b">r%d\n%s\n" % (i, s[a:a + 90])
                     for i, a in enumerate(rng.randrange(0, 13000) for _ in range(12)))
    reads += b">tail\n" + s[-50:] + rand_seq(rng, 40) + b"\n"
    dm = 288_000_000_000
    out, recs = R.pipeline_with_matches(ref, reads, dm, seed_len=6, thres=1100, seeder=1)
    p = oracle.default_params(device_mem=dm, seed_len=6, ignore_thres=1100, seeder=1)
    names = [l[1:].decode() for l in reads.split(b"\n") if l.startswith(b">")]
    got = [(names[r], st, ri, sh, rp) for r, st, ri, sh, rp in oracle.phase1(ref, reads, p)]
    assert got == recs
    assert oracle.align(ref, reads, p) == out


def _paired_case(rng, n_refs, ref_len, n_pairs, L, widths=(60,), repeats=False, frag=(150, 700),
                 lowcomplex=False):
    comp = bytes.maketrans(b"ACGT", b"TGCA")
    seqs = []
    for i in range(n_refs):
        if repeats:
            u = rand_seq(rng, 200)
            s = bytearray()
            while len(s) < ref_len:
                s += mutate(rng, u, 0.02, 0.0) if rng.random() < 0.6 else rand_seq(rng, 200)
            s = bytes(s[:ref_len])
        else:
            s = rand_seq(rng, ref_len)
        if i % 2 == 1:
            s = s[:500].lower() + s[500:]
        if lowcomplex and i == 0:  # a 12-mer over the 1000-occurrence threshold
            s = s[:3000] + b"ACGTTGCAACGT" * 1200 + s[3000:]
        seqs.append(s)
    recs = []
    for i, s in enumerate(seqs):
        w = widths[i % len(widths)]
        lines = [s[j:j + w] for j in range(0, len(s), w)]
        if i == 1 and len(lines) > 8:  # a blank line and a longer line in the middle
            lines[3] = lines[3] + lines[4]
            del lines[4]
            lines.insert(6, b"")
        recs.append(b">ref%d\n" % i + b"\n".join(lines) + b"\n")
    ref = b"".join(recs)
    r1, r2 = [], []
    for i in range(n_pairs):
        si = rng.randrange(n_refs)
        s = seqs[si]
        f = rng.randint(*frag)
        a = rng.randrange(0, max(1, len(s) - f - 5))
        m1 = mutate(rng, s[a:a + L + 5], 0.02, 0.01)[:L].ljust(L, b"A")
        m2 = mutate(rng, s[a + f - L:a + f + 5], 0.02, 0.01)[:L].ljust(L, b"C")
        m2 = m2.translate(comp)[::-1]
        if i % 5 == 2:
            m1, m2 = m2, m1
        if i % 7 == 3:  # mate 2 from another sequence
            o = seqs[(si + 1) % n_refs]
            b = rng.randrange(0, len(o) - L)
            m2 = o[b:b + L].upper()
        if i % 11 == 5:
            m1 = rand_seq(rng, L)
        if i % 13 == 6:
            m1 = m1[:20] + b"N" + m1[21:]
        r1.append(b">pair%d/1\n%s\n" % (i, m1))
        r2.append(b">pair%d/2\n%s\n" % (i, m2))
    return ref, b"".join(r1), b"".join(r2)


@pytest.mark.parametrize("seed,case", list(enumerate([
    dict(n_refs=1, ref_len=20000, n_pairs=30, L=100),
    dict(n_refs=3, ref_len=8000, n_pairs=40, L=90, widths=(60, 70, 50)),
    dict(n_refs=2, ref_len=12000, n_pairs=40, L=100, repeats=True),
    dict(n_refs=2, ref_len=6000, n_pairs=30, L=60, frag=(50, 900)),
    dict(n_refs=2, ref_len=9000, n_pairs=40, L=100, widths=(50, 62), lowcomplex=True),
])))
@pytest.mark.parametrize("dm,fmt", [(288_000_000_000, 0), (100_000_000 + 37 * 1700, 0),
                                    (288_000_000_000, 1)])
def test_paired_pipeline(oracle, seed, case, dm, fmt):
    # the reference's searchQueries_paired2 (lookupTable2, hit lists, the
    # cluster picks) and alignQueries_paired2 (getSeq windows of 3Q, the
    # kernel on fibers, chooseBestAlignment_paired3, printOutput_paired2)
    # against the oracle: records and output, one batch and small batches
    rng = random.Random(1400 + seed)
    ref, r1, r2 = _paired_case(rng, **case)
    out, recs = R.pipeline_paired(ref, r1, r2, dm, out_format=fmt)
    p = oracle.default_params(device_mem=dm, out_format=fmt)
    names = [[l[1:].decode() for l in r.split(b"\n") if l.startswith(b">")] for r in (r1, r2)]
    got = [(i, names[m - 1][rd], rv, m, ri, sh, of)
           for i, rv, m, ri, sh, of, rd in oracle.phase1_paired(ref, r1, r2, p)]
    assert got == recs
    assert oracle.align_paired(ref, r1, r2, p) == out
    assert len(recs) > 0 and len(out) > 0


def test_cpu_sw_cost_against_the_reference_routine(oracle, capsys):
    # the CPU baseline times the port's Smith-Waterman; this ties its cost to
    # the reference's own CPU routine (smithWaterman_cpu,
    # src/smithWaterman.cu:44-335) on the same 100 x 300 pairs, one thread
    # each, and checks they agree on score and end
    import time
    rng = random.Random(9)
    pairs = []
    for _ in range(60):
        w = rand_seq(rng, 300)
        pairs.append((mutate(rng, w[80:190])[:100].ljust(100, b"A"), w))
    t0 = time.perf_counter()
    ref = [R.sw_cpu(q, w) for q, w in pairs]
    t_ref = time.perf_counter() - t0
    t0 = time.perf_counter()
    port = [oracle.sw(q, w) for q, w in pairs]
    t_port = time.perf_counter() - t0
    for a, b in zip(ref, port):
        assert a["score"] == b["score"] and a["end"] == b["end"]
    cells = 60 * 100 * 300
    with capsys.disabled():
        print(f"\nCPU Smith-Waterman, one thread: reference smithWaterman_cpu "
              f"{cells / t_ref / 1e6:.0f} Mcells/s, port {cells / t_port / 1e6:.0f} Mcells/s "
              f"(port / reference = {t_ref / t_port:.2f})")
    assert t_ref > 0 and t_port > 0
