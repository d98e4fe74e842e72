"""Parity at the scale of the headline workload.

The 50 Mbp reference of the throughput benchmark (24 sequences with
log-normal lengths, 10 % of it diverged copies of 300-bp repeat units) and
320,000 reads of its generator: more
than one chunk (262,144 pairs) of the candidates' trace pass and walk, the
repeat-rich index, the stale trailing batch of the 16-read loop and the
selection over about 1.3 M records, all compared byte for byte with the
oracle.  The index of the same reference is compared bucket by bucket.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_READS = 320_000
TRACE_CHUNK = 262_144


@pytest.fixture(scope="module")
def sg():
    from swift_gb300 import build as b
    b.build()
    import swift_gb300
    return swift_gb300


@pytest.fixture(scope="module")
def workload():
    from swift_gb300 import synth
    names, seqs = synth.make_reference(50_000_000, 24, sigma=0.8, repeat_frac=0.10,
                                       n_units=500, unit_len=300, divergence=0.03, seed=0)
    rn, rs, _ = synth.make_reads(seqs, N_READS, 100, 0.01, 0.001, 0.05, seed=1)
    return synth.fasta_bytes(names, seqs), synth.reads_fasta(rn, rs)


@pytest.fixture(scope="module")
def ctx(sg):
    return sg.Context(0)


@pytest.fixture(scope="module")
def index(ctx, workload):
    return ctx.index(workload[0])


@pytest.fixture(scope="module")
def session(ctx, oracle, workload):
    p = oracle.default_params(device_mem=ctx.info()["total_mem"], threads=os.cpu_count() or 1)
    return oracle.Session(workload[0], p), p


def first_diff(a: bytes, b: bytes) -> int:
    n = min(len(a), len(b))
    x = np.frombuffer(a[:n], np.uint8) != np.frombuffer(b[:n], np.uint8)
    return int(np.argmax(x)) if x.any() else n


def test_scale_index_matches_oracle(index, oracle, workload):
    look, rep, ri, rp = index.export()
    ox = oracle.Index(workload[0])
    olook, orep = ox.buckets()
    ori, orp = ox.postings()
    assert ox.total == index.info()["total"]
    assert np.array_equal(look, olook) and np.array_equal(rep, orep)
    assert np.array_equal(ri, ori) and np.array_equal(rp, orp)
    assert rep.max() > 1  # k-mers of the diverged repeat copies recur


def test_scale_alignment_matches_oracle(ctx, index, session, workload):
    sess, _ = session
    got, st = ctx.align(index, workload[1], stats=True)
    # more than one chunk of the candidates' trace pass and walk ran
    assert st["traced_pairs"] > TRACE_CHUNK
    assert st["records"] > 4 * N_READS and st["printed"] == N_READS
    want = sess.align(workload[1])
    assert len(got) == len(want) and got == want, first_diff(got, want)


def test_scale_sam_matches_oracle(ctx, index, oracle, workload, sg):
    # SAM traces every packed pair; a third of the reads (about 440 K
    # pairs, two trace chunks) keeps the oracle's share of the test short
    lines = workload[1].split(b"\n", 2 * (N_READS // 3))
    reads = b"\n".join(lines[: 2 * (N_READS // 3)]) + b"\n"
    got, st = ctx.align(index, reads, sg.default_params(out_format=1), stats=True)
    assert st["traced_pairs"] > TRACE_CHUNK
    p = oracle.default_params(device_mem=ctx.info()["total_mem"], threads=os.cpu_count() or 1,
                              out_format=1)
    want = oracle.Session(workload[0], p).align(reads)
    assert len(got) == len(want) and got == want, first_diff(got, want)
