"""Paired-end alignment (-q / -q2) on the GPU against the oracle.

The oracle's restatement is pinned to the reference's own paired-end code
(lookupTable2, chooseBestAlignment_paired3, printOutput_paired2) by
tests/test_oracle_vs_reference.py; here swift_align_paired must produce the
same bytes for layouts, repeats, a threshold-crossing 12-mer, fragment
limits, small batches, SAM output, another index threshold and the CLI.
"""
import os
import random
import subprocess
import tempfile

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


def paired_case(seed, n_refs, ref_len, n_pairs, L, widths=(60,), repeats=False,
                frag=(150, 700), lowcomplex=False):
    rng = random.Random(seed)
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
        if lowcomplex and i == 0:
            s = s[:3000] + b"ACGTTGCAACGT" * 1200 + s[3000:]
        seqs.append(s)
    recs = []
    for i, s in enumerate(seqs):
        w = widths[i % len(widths)]
        lines = [s[j:j + w] for j in range(0, len(s), w)]
        if i == 1 and len(lines) > 8:
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
        if i % 7 == 3:
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


CASES = [
    dict(n_refs=1, ref_len=20000, n_pairs=200, L=100),
    dict(n_refs=3, ref_len=8000, n_pairs=200, L=90, widths=(60, 70, 50)),
    dict(n_refs=2, ref_len=12000, n_pairs=200, L=100, repeats=True),
    dict(n_refs=2, ref_len=6000, n_pairs=150, L=60, frag=(50, 900)),
    dict(n_refs=2, ref_len=9000, n_pairs=150, L=100, widths=(50, 62), lowcomplex=True),
]


@pytest.mark.parametrize("seed,case", list(enumerate(CASES)))
def test_paired_vs_oracle(ctx, oracle, sg, seed, case):
    ref, r1, r2 = paired_case(1500 + seed, **case)
    ix = ctx.index(ref)
    for dm, fmt, frag in [(288_000_000_000, 0, (99, 600)), (100_000_000 + 91 * 1700, 0, (99, 600)),
                          (288_000_000_000, 1, (99, 600)), (288_000_000_000, 0, (200, 300))]:
        p = sg.default_params(device_mem=dm, out_format=fmt)
        got, st = ctx.align_paired(ix, r1, r2, p, frag[0], frag[1], stats=True)
        want = oracle.align_paired(ref, r1, r2, oracle.default_params(device_mem=dm,
                                                                      out_format=fmt),
                                   frag[0], frag[1])
        assert got == want, (dm, fmt, frag)
        assert st["records"] > 0 and len(got) > 0


def test_paired_index_threshold_and_cli(ctx, oracle, sg):
    # an index built with another threshold: the paired path keeps the
    # reference's fixed 1000 (a second, internal index)
    ref, r1, r2 = paired_case(1600, n_refs=2, ref_len=10000, n_pairs=120, L=100, repeats=True)
    want = oracle.align_paired(ref, r1, r2, oracle.default_params(
        device_mem=ctx.info()["total_mem"]))
    ix = ctx.index(ref, 12, 5)
    assert ctx.align_paired(ix, r1, r2, sg.default_params(ignore_thres=5)) == want
    with tempfile.TemporaryDirectory() as d:
        paths = [os.path.join(d, f) for f in ("ref.fa", "r1.fa", "r2.fa", "out.txt")]
        for pth, data in zip(paths, (ref, r1, r2)):
            open(pth, "wb").write(data)
        r = subprocess.run([sg.CLI_PATH, "-q", paths[1], "-q2", paths[2], "-r", paths[0],
                            "-o", paths[3], "-ms", "150", "-MS", "500"], capture_output=True)
        assert r.returncode == 0, r.stderr
        got = open(paths[3], "rb").read()
    assert got == oracle.align_paired(ref, r1, r2, oracle.default_params(
        device_mem=ctx.info()["total_mem"]), 150, 500)


def test_paired_input_errors(ctx, sg):
    rng = random.Random(3)
    s = rand_seq(rng, 5000)
    ref = b">a\n" + s + b"\n"
    ix = ctx.index(ref)
    comp = bytes.maketrans(b"ACGT", b"TGCA")
    one = b">p/1\n" + s[:100] + b"\n"
    two = b">p/2\n" + s[300:400].translate(comp)[::-1] + b"\n"  # a 400-base fragment
    for r1, r2 in [(one, two + two.replace(b"p/2", b"q/2")),       # unequal counts
                   (one, b">p/2\n" + s[:50] + b"\n"),              # mate shorter than Q
                   (one.replace(b"p/1", b"pa"), two)]:             # name not ending in 1/2
        with pytest.raises(sg.SwiftError) as e:
            ctx.align_paired(ix, r1, r2)
        assert e.value.code == -2
    assert ctx.align_paired(ix, one, two).startswith(b"\n***")


def test_paired_into_caller_buffer(ctx, sg):
    # enough records for the text to reach the host in record ranges copied
    # while the next range is written: the same bytes as swift_align_paired
    import ctypes
    import torch
    from swift_gb300 import synth
    names, seqs = synth.make_reference(2_000_000, 6, sigma=0.6, repeat_frac=0.1, n_units=40,
                                       unit_len=300, divergence=0.03, seed=21)
    ref = synth.fasta_bytes(names, seqs)
    r1, r2 = synth.paired_reads(seqs, 20_000, 100, (200, 500), 0.01, seed=22)
    ix = ctx.index(ref)
    pin = []
    for r in (r1, r2):
        t = torch.empty(len(r), dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = memoryview(r)
        pin.append(t)
    for fmt in (0, 1):
        p = sg.default_params(out_format=fmt)
        want, st = ctx.align_paired(ix, r1, r2, p, stats=True)
        assert st["records"] >= 65536
        out = torch.zeros(len(want), dtype=torch.uint8, pin_memory=True)  # exact size
        n, _ = ctx.align_paired_into(ix, pin[0].data_ptr(), len(r1), pin[1].data_ptr(), len(r2),
                                     out.data_ptr(), len(want), p)
        assert n == len(want) and out.numpy().tobytes() == want, fmt
        pageable = ctypes.create_string_buffer(len(want) + 1)
        n, _ = ctx.align_paired_into(ix, pin[0].data_ptr(), len(r1), pin[1].data_ptr(), len(r2),
                                     ctypes.addressof(pageable), len(pageable), p, 150, 500)
        assert pageable.raw[:n] == ctx.align_paired(ix, r1, r2, p, 150, 500)
        with pytest.raises(sg.SwiftError) as e:
            ctx.align_paired_into(ix, pin[0].data_ptr(), len(r1), pin[1].data_ptr(), len(r2),
                                  out.data_ptr(), len(want) - 1, p)
        assert e.value.code == -5
