"""CUDA path against the CPU oracle: bit-exact on every output.

Each test builds inputs with a fixed seed, runs the device path through the
C ABI and compares with the oracle restatement of the reference.
"""
import os
import random
import subprocess
import tempfile

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


def oparams(ctx, O, **kw):
    return O.default_params(device_mem=ctx.info()["total_mem"], **kw)


def first_diff(a: bytes, b: bytes) -> int:
    n = min(len(a), len(b))
    for i in range(n):
        if a[i] != b[i]:
            return i
    return n


# ---------------------------------------------------------------------------
# index

GOLDEN_FASTA = [
    (b">ref1\nACGTACGTGTACGTAACATC\n", 8, 15),
    (b">ref1\nACGTACGTAATAACGTACGTATTTACGTACACCCGTACGT\n>ref2\n"
     b"GCCGTACGACGTACGTAAACGTAACGTACGTATTTACG\n"
     b">ref3\nCGTACGTAAAATAACGTCGTACGTAAACGTACGTACGTAA", 8, 15),
    (b">ref1\nACGTACGTAATAACGTACGTATTT\nACGTACACCCGTACGT\n>ref2\n"
     b"GCCGTACGACGTACGTAAACGTAA\nCGTACGTATTTACG\n"
     b">ref3\nCGTACGTAAA\nATAACGTCGT\nACGTAAACGT\nACGTACGTAA", 8, 4),
    (b">ref1\nACGTACGTAATAACGTACGTATTT\nACGTACACCCGTACGT\n>ref2\n"
     b"GCCGTACGACGTACGTAAACGTAA\nCGTACGTATTTACG\n"
     b">ref3\nCGTACGTAAA\nATAACGTCGT\nACGTAAACGT\nACGTACGTAA", 4, 7),
]


def messy_reference(seed=3, n_seqs=5, total=120_000):
    """Multi-record FASTA with lowercase runs, N runs, IUPAC letters, blank
    lines and uneven line widths."""
    rng = random.Random(seed)
    out = []
    for r in range(n_seqs):
        n = total // n_seqs + rng.randint(-5000, 5000)
        s = bytearray(rng.choice(b"ACGT") for _ in range(n))
        for _ in range(20):
            a = rng.randrange(n)
            for i in range(a, min(n, a + rng.randint(1, 40))):
                s[i] = (s[i] | 0x20) if rng.random() < 0.7 else ord("N")
        for _ in range(5):
            s[rng.randrange(n)] = rng.choice(b"RYKMSW")
        out.append(b">seq%d some description\n" % r)
        width = rng.choice([50, 60, 61, 70])
        for i in range(0, n, width):
            out.append(bytes(s[i:i + width]) + b"\n")
            if rng.random() < 0.002:
                out.append(b"\n")
    return b"".join(out)


@pytest.mark.parametrize("case", range(len(GOLDEN_FASTA)))
def test_index_golden(ctx, oracle, case):
    fa, k, t = GOLDEN_FASTA[case]
    ix = ctx.index(fa, k, t)
    look, rep, ri, rp = ix.export()
    ox = oracle.Index(fa, k, t)
    ori, orp = ox.postings()
    assert list(ri) == list(ori) and list(rp) == list(orp)
    for h in range(ox.num_buckets):
        assert look[h] == ox.start(h) and rep[h] == ox.repeats(h)


def test_index_messy_reference(ctx, oracle):
    fa = messy_reference()
    for k, t in [(12, 1000), (8, 3)]:
        ix = ctx.index(fa, k, t)
        look, rep, ri, rp = ix.export()
        ox = oracle.Index(fa, k, t)
        ori, orp = ox.postings()
        assert np.array_equal(ri, ori) and np.array_equal(rp, orp)
        nb = ox.num_buckets
        assert all(look[h] == ox.start(h) for h in range(0, nb, max(1, nb // 50000)))


# ---------------------------------------------------------------------------
# Smith-Waterman (alignSequences contract)

def test_sw_golden(ctx):
    # test/testSmithWaterman.cu:29-124 and :304-386
    r = ctx.sw_batch([b"ACGTACGTAA"], [b"CCCCAAAACGTCCGTTACGT"], 10, 20)[0]
    assert (r["score"], r["start"], r["end"], r["len"]) == (14.0, 8, 17, 10)
    assert r["qcons"] == b"AATGCATGCA" and r["rcons"] == b"ATTGCCTGCA"
    r = ctx.sw_batch([b"CTTGTCACCATCCA"], [b"CTTGTCACCATCA"], 14, 13)[0]
    assert r["score"] == 24.0
    r = ctx.sw_batch([b"ACGTACGTAA"], [b"CCCCAAAACGTCCGTTACGT"], 10, 25)[0]
    assert r["score"] == 14.0


def mutate(rng, s: bytes, p_sub=0.05, p_indel=0.02) -> bytes:
    out = bytearray()
    for c in s:
        x = rng.random()
        if x < p_indel / 2:
            continue
        if x < p_indel:
            out += bytes(rng.choice(b"ACGT") for _ in range(rng.randint(1, 4)))
        out.append(rng.choice(b"ACGT") if rng.random() < p_sub else c)
    return bytes(out)


def random_pairs(seed, n, Q, R, alphabet=b"ACGT"):
    rng = random.Random(seed)
    qs, ws = [], []
    for i in range(n):
        kind = i % 5
        w = bytes(rng.choice(alphabet) for _ in range(R))
        if kind == 0:
            q = bytes(rng.choice(alphabet) for _ in range(Q))
        else:
            a = rng.randrange(0, max(1, R - Q))
            q = mutate(rng, w[a:a + Q + 10])[:Q]
            q = q.ljust(Q, b"A")
        if kind == 2:  # window cut short: NUL padding
            w = w[: rng.randint(min(R, Q // 2), R)]
        if kind == 3:  # case and N
            w = bytes(((c | 0x20) if rng.random() < 0.3 else c) for c in w)
            q = bytes((ord("N") if rng.random() < 0.02 else c) for c in q)
        qs.append(q)
        ws.append(w)
    return qs, ws


@pytest.mark.parametrize("Q,R", [(100, 300), (37, 300), (128, 200), (200, 300), (256, 64)])
def test_sw_random_vs_oracle(ctx, oracle, Q, R):
    qs, ws = random_pairs(11 + Q + R, 300, Q, R)
    got = ctx.sw_batch(qs, ws, Q, R)
    for i, (q, w) in enumerate(zip(qs, ws)):
        want = oracle.sw(q, w, Q, R)
        for key in ("score", "start", "end", "len", "qcons", "rcons"):
            assert got[i][key] == want[key], (i, key, got[i][key], want[key])


def test_sw_scoring_parameters(ctx, oracle):
    qs, ws = random_pairs(5, 100, 60, 150)
    for m, x, o, e in [(1, -3, -5, -2), (5, -4, -20, -1), (2, -1, -1, -1)]:
        got = ctx.sw_batch(qs, ws, 60, 150, m, x, o, e)
        for i, (q, w) in enumerate(zip(qs, ws)):
            want = oracle.sw(q, w, 60, 150, m, x, o, e)
            assert (got[i]["score"], got[i]["start"], got[i]["end"], got[i]["len"],
                    got[i]["qcons"], got[i]["rcons"]) == (
                want["score"], want["start"], want["end"], want["len"], want["qcons"],
                want["rcons"])


def test_sw_zero_pairs_and_limits(ctx, sg):
    assert ctx.sw_batch([], [], 10, 10) == []
    with pytest.raises(sg.SwiftError):
        ctx.sw_batch([b"A" * 10], [b"A" * 10], 400, 10)
    # scores must be whole numbers (float in alignSequences, atoi in the CLI)
    with pytest.raises(sg.SwiftError) as e:
        ctx.sw_batch([b"ACGT"], [b"ACGT"], 4, 4, match=1.5)
    assert e.value.code == -1


@pytest.mark.parametrize("Q,R", [(256, 1024), (129, 787), (128, 1024), (320, 1024), (257, 300)])
def test_sw_largest_shapes(ctx, oracle, Q, R):
    # the documented maximum shapes, whose direction words need fewer warps
    # per block to fit shared memory
    qs, ws = random_pairs(31 + Q + R, 24, Q, R)
    got = ctx.sw_batch(qs, ws, Q, R)
    for i, (q, w) in enumerate(zip(qs, ws)):
        want = oracle.sw(q, w, Q, R)
        for key in ("score", "start", "end", "len", "qcons", "rcons"):
            assert got[i][key] == want[key], (i, key)


def test_sw_foreign_device_pointer(ctx, sg):
    # a device buffer of another GPU than the context's is refused
    torch = pytest.importorskip("torch")
    if torch.cuda.device_count() < 2:
        pytest.skip("one GPU: the check against the context's device cannot be exercised")
    other = torch.zeros(1 << 12, dtype=torch.uint8, device="cuda:1")
    p = other.data_ptr()
    assert sg.lib().swift_sw_batch(ctx._h, p, p, 4, 4, 1, 2, -1, -10, -1, *([p] * 6)) == -1
    assert sg.lib().swift_sw_batch_noalloc(ctx._h, p, p, 4, 4, 1, 2, -1, -10, -1,
                                           *([p] * 6)) == -1


# ---------------------------------------------------------------------------
# Phase 1

def small_case(n_reads=2000, seed=21, ref_bp=200_000, n_seqs=3):
    from swift_gb300 import synth
    names, seqs = synth.make_reference(ref_bp, n_seqs, sigma=0.5, seed=seed)
    ref = synth.fasta_bytes(names, seqs)
    rn, rs, _ = synth.make_reads(seqs, n_reads, 100, 0.01, 0.001, 0.05, seed=seed + 1)
    return ref, synth.reads_fasta(rn, rs)


def test_seed_vs_oracle(ctx, oracle):
    ref, reads = small_case()
    ix = ctx.index(ref)
    got = ctx.seed(ix, reads)
    want = oracle.phase1(ref, reads, oparams(ctx, oracle))
    assert got == want


def test_seed_overflow_path(ctx, oracle):
    # 100 exact copies of a 120-bp unit: reads over it hit ~800 postings per
    # strand, more than the on-chip path holds
    rng = random.Random(9)
    unit = bytes(rng.choice(b"ACGT") for _ in range(120))
    body = b"".join(unit for _ in range(100))
    tail = bytes(rng.choice(b"ACGT") for _ in range(3000))
    seq = tail + body + tail
    ref = b">rep\n" + b"\n".join(seq[i:i + 60] for i in range(0, len(seq), 60)) + b"\n"
    reads = []
    for i in range(40):
        a = rng.randrange(0, len(seq) - 100)
        reads.append(b">q%d\n%s\n" % (i, seq[a:a + 100]))
    reads = b"".join(reads)
    ix = ctx.index(ref)
    got = ctx.seed(ix, reads)
    want = oracle.phase1(ref, reads, oparams(ctx, oracle))
    assert got == want
    _, st = ctx.align(ix, reads, stats=True)
    assert st["seed_overflow_strands"] > 0


@pytest.mark.parametrize("max_hits", [1, 3, 4, 9])
def test_seed_every_hit_class(ctx, oracle, max_hits):
    # half of the reference is diverged copies of 20 repeat units: of the 800
    # strands of reads of 100-199 bases, about 570 have at most 32 hits, 50
    # 33-128, 180 129-512 and a few more (the warp-match, both hash-table and
    # the overflow kernels); more than three clusters per strand take the
    # hash-table kernels past their kept keys
    from swift_gb300 import synth
    names, seqs = synth.make_reference(1_000_000, 2, sigma=0.3, repeat_frac=0.5, n_units=20,
                                       unit_len=300, divergence=0.05, seed=3)
    ref = synth.fasta_bytes(names, seqs)
    rn, rs, _ = synth.make_reads(seqs, 400, 150, 0.01, 0.001, 0.05, seed=4, len_range=(100, 199))
    reads = synth.reads_fasta(rn, rs)
    ix = ctx.index(ref)
    got = ctx.seed(ix, reads, max_hits=max_hits)
    want = oracle.phase1(ref, reads, oparams(ctx, oracle, max_hits=max_hits))
    assert got == want


# ---------------------------------------------------------------------------
# whole pipeline

def test_align_small_workload(ctx, oracle):
    from swift_gb300 import synth
    ref, reads, _ = synth.workload("small")
    ix = ctx.index(ref)
    got = ctx.align(ix, reads)
    want = oracle.align(ref, reads, oparams(ctx, oracle))
    assert len(got) == len(want) and got == want, first_diff(got, want)


@pytest.mark.parametrize("n_reads", [1, 15, 16, 17, 33, 250])
def test_align_read_counts(ctx, oracle, n_reads):
    # trailing 16-read batches of searchQueries3 repeat stale reads
    ref, reads = small_case(n_reads=n_reads, seed=40 + n_reads)
    ix = ctx.index(ref)
    got = ctx.align(ix, reads)
    want = oracle.align(ref, reads, oparams(ctx, oracle))
    assert got == want, first_diff(got, want)


def test_align_messy_inputs(ctx, oracle):
    fa = messy_reference(seed=8)
    # reads drawn from the messy reference (lowercase, N), some reverse
    # complemented, some shorter than the seed length
    seqs = []
    cur = None
    for line in fa.split(b"\n"):
        if line.startswith(b">"):
            cur = bytearray()
            seqs.append(cur)
        elif cur is not None:
            cur += line
    rng = random.Random(12)
    parts = []
    for i in range(600):
        s = seqs[rng.randrange(len(seqs))]
        a = rng.randrange(0, len(s) - 100)
        r = bytes(s[a:a + 100])
        if i % 3 == 1:
            r = oracle.revcomp(r)
        if i % 7 == 3:
            r = bytes(rng.choice(b"ACGTN") for _ in range(100))
        parts.append(b">read_%d/x\n%s\n" % (i, r))
    reads = b"".join(parts)
    ix = ctx.index(fa)
    got = ctx.align(ix, reads)
    want = oracle.align(fa, reads, oparams(ctx, oracle))
    assert got == want, first_diff(got, want)


def test_align_line_layouts(ctx, oracle):
    # windows come from the concatenated sequence when every line but the
    # last has the record's width, and from the file bytes otherwise; both
    # must follow the reference's file-offset arithmetic
    rng = random.Random(61)
    seqs = [bytes(rng.choice(b"ACGT") for _ in range(rng.randint(3000, 6000))) for _ in range(7)]
    def lines(s, widths, eol=b"\n"):
        out, i, t = [], 0, 0
        while i < len(s):
            w = widths[min(t, len(widths) - 1)] if callable(widths) is False else widths(t)
            out.append(s[i:i + w] + eol)
            i += w
            t += 1
        return b"".join(out)
    recs = [
        b">uniform\n" + lines(seqs[0], [60]),
        b">long_middle\n" + lines(seqs[1], lambda t: 75 if t == 10 else 60),
        b">blank_line\n" + lines(seqs[2][:1500], [60]) + b"\n" + lines(seqs[2][1500:], [60]),
        b">single\n" + seqs[3] + b"\n",
        b">long_last\n" + lines(seqs[4][:-100], [50]) + seqs[4][-100:] + b"\n",
        b">crlf\n" + lines(seqs[5], [61], b"\r\n"),
        b">uniform_no_eol\n" + lines(seqs[6], [70])[:-1],
    ]
    ref = b"".join(recs)
    reads = []
    for r, sq in enumerate(seqs):
        for t in range(60):
            a = rng.randrange(0, len(sq) - 100)
            rd = bytearray(sq[a:a + 100])
            if t % 2:
                rd = bytearray(rd[::-1].translate(bytes.maketrans(b"ACGT", b"TGCA")))
            reads.append(b">r%d_%d\n" % (r, t) + bytes(rd) + b"\n")
    reads = b"".join(reads)
    ix = ctx.index(ref)
    got = ctx.align(ix, reads)
    want = oracle.align(ref, reads, oparams(ctx, oracle))
    assert got == want, first_diff(got, want)


def test_align_scoring_and_seed_parameters(ctx, oracle, sg):
    ref, reads = small_case(n_reads=300, seed=77)
    for kw in [dict(seed_len=10, ignore_thres=50), dict(match=3, mismatch=-2, gap_open=-6,
                                                        gap_ext=-2), dict(max_hits=1)]:
        k = kw.get("seed_len", 12)
        t = kw.get("ignore_thres", 1000)
        ix = ctx.index(ref, k, t)
        p = sg.default_params(**kw)
        got = ctx.align(ix, reads, p)
        want = oracle.align(ref, reads, oparams(ctx, oracle, **kw))
        assert got == want, (kw, first_diff(got, want))


def test_align_longer_reads_than_query_length(ctx, oracle, sg):
    ref, reads = small_case(n_reads=200, seed=91)
    ix = ctx.index(ref)
    p = sg.default_params(qry_len=80)
    got = ctx.align(ix, reads, p)
    want = oracle.align(ref, reads, oparams(ctx, oracle, qry_len=80))
    assert got == want


def test_align_resident_matches_host_call(ctx, oracle):
    ref, reads = small_case(n_reads=500, seed=93)
    ix = ctx.index(ref)
    host = ctx.align(ix, reads)
    rd = ctx.reads(reads)
    n, st = ctx.align_resident(ix, rd)
    assert ctx.fetch_output(n) == host
    n2, _ = ctx.align_resident(ix, rd)
    assert n2 == n and ctx.fetch_output(n2) == host


def test_input_errors(ctx, sg):
    ref, _ = small_case(n_reads=1, seed=5)
    ix = ctx.index(ref)
    for bad, code in [(b">a\nACGT\n\n>b\nACGT\n", -2),       # empty line
                      (b">a\nACGT\nACGT\n", -2),             # multi-line read
                      (b">a\n", -2),                          # header without sequence
                      (b">a\nAC>GT\n", -2),                  # '>' inside a line
                      (b">a\n" + b"A" * 250 + b"\n", -5),    # read over 199 bases
                      (b">" + b"n" * 60 + b"\nACGT\n", -5),  # name over 48 characters
                      (b"ACGT\n>a\nACGT\n", -2),           # sequence before a header
                      (b">a\n>b\nACGT\n", -2),              # header without sequence
                      (b">a\nAC\x00GT\n", -2),              # NUL byte
                      (b">a\nAC\xc3GT\n", -2),              # byte >= 128
                      (b">a\nACGT\n>b\n", -2),             # trailing header
                      (b"", -5)]:                             # no reads: query length 0
        with pytest.raises(sg.SwiftError) as e:
            ctx.align(ix, bad)
        assert e.value.code == code
    with pytest.raises(sg.SwiftError):
        ctx.index(b"ACGT\n>x\nACGT\n")


def test_reads_without_final_newline(ctx, oracle):
    # the first read's length is strlen(line) - 1 (getSeqSize); when that line
    # ends the file without a newline the query is one base shorter
    ref, reads = small_case(n_reads=200, seed=77)
    ix = ctx.index(ref)
    trimmed = reads.rstrip(b"\n")
    got = ctx.align(ix, trimmed)
    assert got == oracle.align(ref, trimmed, oparams(ctx, oracle))
    one = b">only\n" + reads.split(b"\n")[1]
    got = ctx.align(ix, one)
    assert got == oracle.align(ref, one, oparams(ctx, oracle))


def test_align_into_caller_buffer(ctx, oracle, sg):
    import ctypes
    ref, reads = small_case(n_reads=500, seed=78)
    ix = ctx.index(ref)
    want = ctx.align(ix, reads)
    src = ctypes.create_string_buffer(reads, len(reads))
    buf = ctypes.create_string_buffer(len(want) + 16)
    n, st = ctx.align_into(ix, ctypes.addressof(src), len(reads), ctypes.addressof(buf), len(buf))
    assert n == len(want) and buf.raw[:n] == want
    assert st["printed"] > 0
    small = ctypes.create_string_buffer(8)
    with pytest.raises(sg.SwiftError) as e:
        ctx.align_into(ix, ctypes.addressof(src), len(reads), ctypes.addressof(small), 8)
    assert e.value.code == -5


def test_align_into_overlapped_copies(ctx, sg):
    # enough records for the text to go to the host in record ranges, each
    # copied while the next is written: the same bytes as the one-piece path
    import ctypes
    import torch
    from swift_gb300 import synth
    names, seqs = synth.make_reference(600_000, 6, sigma=0.6, repeat_frac=0.1, n_units=30,
                                       unit_len=300, divergence=0.03, seed=12)
    ref = synth.fasta_bytes(names, seqs)
    rn, rs, _ = synth.make_reads(seqs, 60_000, 100, 0.02, 0.002, 0.05, seed=13)
    reads = synth.reads_fasta(rn, rs)
    ix = ctx.index(ref)
    src = torch.empty(len(reads), dtype=torch.uint8, pin_memory=True)
    src.numpy()[:] = memoryview(reads)
    for fmt in (0, 1):
        p = sg.default_params(out_format=fmt)
        want, st = ctx.align(ix, reads, p, stats=True)
        assert st["records"] >= 65536
        out = torch.zeros(len(want), dtype=torch.uint8, pin_memory=True)  # exact size
        n, st2 = ctx.align_into(ix, src.data_ptr(), len(reads), out.data_ptr(), len(want), p)
        assert n == len(want) and out.numpy().tobytes() == want, fmt
        pageable = ctypes.create_string_buffer(len(want) + 1)
        n, _ = ctx.align_into(ix, src.data_ptr(), len(reads), ctypes.addressof(pageable),
                              len(pageable), p)
        assert pageable.raw[:n] == want
        with pytest.raises(sg.SwiftError) as e:
            ctx.align_into(ix, src.data_ptr(), len(reads), out.data_ptr(), len(want) - 1, p)
        assert e.value.code == -5


def test_align_into_large_calls(ctx, sg):
    # 140,007 reads through the host-buffer call (text in record ranges,
    # each copied while the next is written): the same bytes as swift_align,
    # with a stale 16-read tail, both output formats and both seeders, also
    # where every read has the same name (one best-per-read group)
    import torch
    from swift_gb300 import synth
    names, seqs = synth.make_reference(2_000_000, 4, sigma=0.5, repeat_frac=0.1, n_units=30,
                                       unit_len=300, divergence=0.03, seed=14)
    ref = synth.fasta_bytes(names, seqs)
    rn, rs, _ = synth.make_reads(seqs, 140_007, 100, 0.01, 0.001, 0.05, seed=15)
    ix = ctx.index(ref)
    for reads in (synth.reads_fasta(rn, rs), synth.reads_fasta(["dup"] * len(rs), rs)):
        src = torch.empty(len(reads), dtype=torch.uint8, pin_memory=True)
        src.numpy()[:] = memoryview(reads)
        for kw in (dict(), dict(out_format=1), dict(seeder=1)):
            p = sg.default_params(**kw)
            want, st = ctx.align(ix, reads, p, stats=True)
            out = torch.zeros(len(want) + 16, dtype=torch.uint8, pin_memory=True)
            n, st2 = ctx.align_into(ix, src.data_ptr(), len(reads), out.data_ptr(), len(out), p)
            assert n == len(want) and out.numpy()[:n].tobytes() == want, kw
            assert st2["reads"] == st["reads"] and st2["printed"] == st["printed"], kw


def test_cli_matches_oracle(ctx, oracle, sg):
    ref, reads = small_case(n_reads=300, seed=55)
    with tempfile.TemporaryDirectory() as d:
        rp, qp, op = (os.path.join(d, f) for f in ("ref.fa", "reads.fa", "out.txt"))
        open(rp, "wb").write(ref)
        open(qp, "wb").write(reads)
        # the reference CLI's GPU branch: lt13 seed-and-extend Phase 1
        r = subprocess.run([sg.CLI_PATH, "-q", qp, "-r", rp, "-o", op], capture_output=True)
        assert r.returncode == 0, r.stderr
        got = open(op, "rb").read()
        # SSAHA seeding (searchQueries3)
        r = subprocess.run([sg.CLI_PATH, "-q", qp, "-r", rp, "-o", op, "-seeder", "0"],
                           capture_output=True)
        assert r.returncode == 0, r.stderr
        got0 = open(op, "rb").read()
    assert got == oracle.align(ref, reads, oparams(ctx, oracle, seeder=1))
    assert got0 == oracle.align(ref, reads, oparams(ctx, oracle))


def test_packed_and_generic_paths_agree(ctx, oracle):
    # bounded selection (default), the exact score of every pair, and the
    # generic kernel for every pair must print exactly the same records
    ref, reads = small_case(n_reads=3000, seed=101)
    ix = ctx.index(ref)
    fast, st = ctx.align(ix, reads, stats=True)
    assert st["sw_generic_pairs"] < st["records"]  # the packed passes ran
    assert st["bound_pruned"] > 0
    outs = {}
    for path in (1, 2):
        ctx.set_sw_path(path)
        try:
            outs[path], sts = ctx.align(ix, reads, stats=True)
        finally:
            ctx.set_sw_path(0)
        if path == 1:
            assert sts["sw_generic_pairs"] == sts["records"]
        assert sts["printed"] == st["printed"]
    assert fast == outs[1] == outs[2]
    assert fast == oracle.align(ref, reads, oparams(ctx, oracle))


def test_bounded_selection_with_repeats(ctx, oracle):
    # a repeat-rich reference gives reads several near-equal candidates, so
    # the bound keeps pairs for exact scoring and some reads' most promising
    # pair is not their best (second traceback round)
    from swift_gb300 import synth
    names, seqs = synth.make_reference(400_000, 4, sigma=0.5, repeat_frac=0.3, n_units=40,
                                       unit_len=300, divergence=0.02, seed=211)
    ref = synth.fasta_bytes(names, seqs)
    rn, rs, _ = synth.make_reads(seqs, 6000, 100, 0.02, 0.004, 0.05, seed=212)
    reads = synth.reads_fasta(rn, rs)
    ix = ctx.index(ref)
    got, st = ctx.align(ix, reads, stats=True)
    assert st["retraced_pairs"] > 0
    assert st["bound_pruned"] < st["records"] - st["sw_generic_pairs"]
    # the LCS bound rules out some pairs and leaves others to the exact pass
    fast = st["records"] - st["sw_generic_pairs"]
    assert 0 < st["lcs_kept"] < fast
    ctx.set_sw_path(2)
    try:
        exact = ctx.align(ix, reads)
    finally:
        ctx.set_sw_path(0)
    assert got == exact
    assert got == oracle.align(ref, reads, oparams(ctx, oracle)), first_diff(got, oracle.align(ref, reads, oparams(ctx, oracle)))


@pytest.mark.parametrize("Q", [20, 50, 64, 100, 128, 150, 199])
def test_packed_path_query_lengths(ctx, oracle, sg, Q):
    # every rows-per-lane variant of the packed score pass
    from swift_gb300 import synth
    names, seqs = synth.make_reference(100_000, 2, sigma=0.3, seed=300 + Q)
    ref = synth.fasta_bytes(names, seqs)
    rn, rs, _ = synth.make_reads(seqs, 400, Q, 0.02, 0.002, 0.05, seed=301 + Q)
    reads = synth.reads_fasta(rn, rs)
    ix = ctx.index(ref)
    got = ctx.align(ix, reads)
    want = oracle.align(ref, reads, oparams(ctx, oracle))
    assert got == want, first_diff(got, want)


# ---------------------------------------------------------------------------
# SAM output (-f 1): every record, CIGAR from the reversed consensus

@pytest.mark.parametrize("n_reads", [1, 17, 250])
def test_sam_read_counts(ctx, oracle, sg, n_reads):
    ref, reads = small_case(n_reads=n_reads, seed=140 + n_reads)
    ix = ctx.index(ref)
    got, st = ctx.align(ix, reads, sg.default_params(out_format=1), stats=True)
    want = oracle.align(ref, reads, oparams(ctx, oracle, out_format=1))
    assert got == want, first_diff(got, want)
    assert st["printed"] == st["records"] == got.count(b"\n")


def test_sam_messy_inputs_and_paths(ctx, oracle, sg):
    # lowercase and N in the reference, random reads with N (generic kernel
    # pairs), both strands; the packed and generic paths print the same SAM
    fa = messy_reference(seed=18)
    seqs, cur = [], None
    for line in fa.split(b"\n"):
        if line.startswith(b">"):
            cur = bytearray()
            seqs.append(cur)
        elif cur is not None:
            cur += line
    rng = random.Random(19)
    parts = []
    for i in range(400):
        s = seqs[rng.randrange(len(seqs))]
        a = rng.randrange(0, len(s) - 100)
        r = bytes(s[a:a + 100])
        if i % 3 == 1:
            r = oracle.revcomp(r)
        if i % 7 == 3:
            r = bytes(rng.choice(b"ACGTN") for _ in range(100))
        parts.append(b">read_%d\n%s\n" % (i, r))
    reads = b"".join(parts)
    ix = ctx.index(fa)
    p = sg.default_params(out_format=1)
    got, st = ctx.align(ix, reads, p, stats=True)
    want = oracle.align(fa, reads, oparams(ctx, oracle, out_format=1))
    assert got == want, first_diff(got, want)
    assert st["sw_generic_pairs"] > 0 and st["traced_pairs"] > 0
    ctx.set_sw_path(1)
    try:
        assert ctx.align(ix, reads, p) == want
    finally:
        ctx.set_sw_path(0)


def test_sam_scoring_and_query_lengths(ctx, oracle, sg):
    from swift_gb300 import synth
    for Q, kw in [(36, dict(match=3, mismatch=-2, gap_open=-6, gap_ext=-2)), (150, {}),
                  (199, dict(max_hits=1))]:
        names, seqs = synth.make_reference(80_000, 2, sigma=0.3, seed=500 + Q)
        ref = synth.fasta_bytes(names, seqs)
        rn, rs, _ = synth.make_reads(seqs, 300, Q, 0.03, 0.01, 0.05, seed=501 + Q)
        reads = synth.reads_fasta(rn, rs)
        ix = ctx.index(ref)
        got = ctx.align(ix, reads, sg.default_params(out_format=1, **kw))
        want = oracle.align(ref, reads, oparams(ctx, oracle, out_format=1, **kw))
        assert got == want, (Q, kw, first_diff(got, want))


def test_sam_cli(ctx, oracle, sg):
    ref, reads = small_case(n_reads=120, seed=57)
    with tempfile.TemporaryDirectory() as d:
        rp, qp, op = (os.path.join(d, f) for f in ("ref.fa", "reads.fa", "out.sam"))
        open(rp, "wb").write(ref)
        open(qp, "wb").write(reads)
        r = subprocess.run([sg.CLI_PATH, "-q", qp, "-r", rp, "-o", op, "-f", "1"],
                           capture_output=True)
        assert r.returncode == 0, r.stderr
        got = open(op, "rb").read()
        # any other -f value prints the default records, as the reference does
        r = subprocess.run([sg.CLI_PATH, "-q", qp, "-r", rp, "-o", op, "-f", "2"],
                           capture_output=True)
        assert r.returncode == 0, r.stderr
        got2 = open(op, "rb").read()
    assert got == oracle.align(ref, reads, oparams(ctx, oracle, out_format=1, seeder=1))
    assert got2 == oracle.align(ref, reads, oparams(ctx, oracle, seeder=1))
