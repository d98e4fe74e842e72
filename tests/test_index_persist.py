"""Index persistence (swift_index_save / swift_index_load) for warm starts.

A loaded index must be the built one: the same exported buckets, and the
same output for both seeders and both output formats, also from another
context; damaged, truncated or foreign files are refused.
"""
import os
import random
import tempfile

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from swift_gb300 import build as b
    b.build()
    import swift_gb300
    return swift_gb300


def case(seed=3):
    from swift_gb300 import synth
    names, seqs = synth.make_reference(400_000, 5, sigma=0.6, repeat_frac=0.1, n_units=30,
                                       unit_len=300, divergence=0.03, seed=seed)
    ref = synth.fasta_bytes(names, seqs)
    rn, rs, _ = synth.make_reads(seqs, 3000, 100, 0.02, 0.002, 0.05, seed=seed + 1)
    return ref, synth.reads_fasta(rn, rs)


def test_save_load_roundtrip(sg):
    import numpy as np
    ref, reads = case()
    ctx = sg.Context(0)
    ix = ctx.index(ref, 11, 500)
    want = {(s, f): ctx.align(ix, reads, sg.default_params(seed_len=11, ignore_thres=500,
                                                             seeder=s, out_format=f))
            for s in (0, 1) for f in (0, 1)}  # seeder 1 builds the lt13 tables first
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ref.swidx")
        ix.save(path)
        ctx2 = sg.Context(0)
        ix2 = sg.Index.load(ctx2, path)
        assert (ix2.seed_len, ix2.ignore_thres) == (11, 500)
        for a, b in zip(ix.export(), ix2.export()):
            assert np.array_equal(a, b)
        for (s, f), w in want.items():
            got = ctx2.align(ix2, reads, sg.default_params(seed_len=11, ignore_thres=500,
                                                           seeder=s, out_format=f))
            assert got == w, (s, f)
        assert ctx2.seed_lt13(ix2, reads) == ctx.seed_lt13(ix, reads)
        # an index saved before its lt13 tables exist builds them after loading
        ix3 = ctx.index(ref, 11, 500)
        p3 = os.path.join(d, "plain.swidx")
        ix3.save(p3)
        ix4 = sg.Index.load(ctx, p3)
        assert ctx.align(ix4, reads, sg.default_params(seed_len=11, ignore_thres=500,
                                                       seeder=1)) == want[(1, 0)]
        assert os.path.getsize(p3) < os.path.getsize(path)


def test_load_refuses_bad_files(sg):
    ref, _ = case(seed=9)
    ctx = sg.Context(0)
    ix = ctx.index(ref)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "i.swidx")
        ix.save(path)
        blob = open(path, "rb").read()
        rng = random.Random(1)
        bad = []
        flip = bytearray(blob)
        flip[rng.randrange(200, len(blob))] ^= 0x40          # payload damaged
        bad.append(("flip", bytes(flip), -2))
        bad.append(("trunc", blob[: len(blob) - 100], -2))    # truncated
        bad.append(("extra", blob + b"x", -2))                # trailing bytes
        bad.append(("magic", b"NOTANIDX" + blob[8:], -2))     # foreign file
        hdr = bytearray(blob)
        hdr[12] = 40                                          # seed length 40
        bad.append(("header", bytes(hdr), -2))
        bad.append(("empty", b"", -2))
        for name, data, code in bad:
            p = os.path.join(d, name)
            open(p, "wb").write(data)
            with pytest.raises(sg.SwiftError) as e:
                sg.Index.load(ctx, p)
            assert e.value.code == code, name
        with pytest.raises(sg.SwiftError) as e:
            sg.Index.load(ctx, os.path.join(d, "missing.swidx"))
        assert e.value.code == -1


def _rechecksum(blob: bytearray):
    """Recomputes the payload checksum of an index file in place (the
    word-wise FNV-1a-style mix of persist.cpp), so that a patched payload
    passes the checksum and only the content checks remain."""
    import numpy as np
    payload = bytes(blob[96:])
    h, P, M = 1469598103934665603, 1099511628211, (1 << 64) - 1
    n8 = len(payload) // 8
    for w in np.frombuffer(payload[:8 * n8], dtype="<u8").tolist():
        h = ((h ^ w) * P) & M
    for b in payload[8 * n8:]:
        h = ((h ^ b) * P) & M
    blob[88:96] = h.to_bytes(8, "little")


def test_load_refuses_records_outside_the_reference(sg):
    # a file whose checksum holds but whose sequence records point outside
    # the reference would steer the kernels' reads out of bounds
    ref, _ = case(seed=11)
    ctx = sg.Context(0)
    ix = ctx.index(ref, 8, 1000)  # k = 8 keeps the file small
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "i.swidx")
        ix.save(path)
        blob = bytearray(open(path, "rb").read())
        ok = bytearray(blob)
        _rechecksum(ok)
        assert ok == blob  # the restated checksum is the file's own
        p = os.path.join(d, "ok.swidx")
        open(p, "wb").write(bytes(ok))
        sg.Index.load(ctx, p).close()
        rec1 = 96 + 96  # second record
        for name, field, value in [("cat_start", 24, 1 << 40), ("cat_len", 32, 1 << 40),
                                   ("seq_off", 8, 1 << 50), ("name_off", 0, 1 << 50)]:
            bad = bytearray(blob)
            bad[rec1 + field:rec1 + field + 8] = value.to_bytes(8, "little")
            _rechecksum(bad)
            p = os.path.join(d, name)
            open(p, "wb").write(bytes(bad))
            with pytest.raises(sg.SwiftError) as e:
                sg.Index.load(ctx, p)
            assert e.value.code == -2, name
