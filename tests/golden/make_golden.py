"""Generates the golden fixtures of this directory by running the reference's
own code (oracle/_ref, built from the reference sources by
oracle/ref_harness) on seeded inputs.

  python tests/golden/make_golden.py

Fixtures:
  sw_pairs.json      inputs and outputs of the reference GPU kernel
                     smithWaterman (run on CPU fibers) for seeded pairs
  index_k8.json      lookupTable5Create tables for a messy multi-record FASTA
  pipeline_ref.fa, pipeline_reads.fa, pipeline_out.txt
                     the SSAHA -> GPU-kernel SW -> best-per-read pipeline
                     built from the reference's functions, file to file
The device-memory size that sets the Phase-2 batch size is recorded in
pipeline_meta.json; with it the batches are the same on any GPU.
"""
import json
import os
import random
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref as R  # noqa: E402

DEVICE_MEM = 288_000_000_000  # bytes; sizes Phase-2 batches as on a GB300
SAM_SMALL_MEM = 100_000_000 + 24 * 1220  # Phase-2 batches of 24 records at Q = 100


def mutate(rng, s, p_sub=0.05, p_indel=0.02):
    out = bytearray()
    for c in s:
        x = rng.random()
        if x < p_indel / 2:
            continue
        if x < p_indel:
            out += bytes(rng.choice(b"ACGT") for _ in range(rng.randint(1, 4)))
        out.append(rng.choice(b"ACGT") if rng.random() < p_sub else c)
    return bytes(out)


def sw_pairs(rng, n=160):
    cases = []
    for i in range(n):
        Q = rng.choice([10, 37, 64, 100])
        Rl = rng.choice([20, 120, 300])
        w = bytes(rng.choice(b"ACGT") for _ in range(Rl))
        kind = i % 5
        if kind == 0:
            q = bytes(rng.choice(b"ACGT") for _ in range(Q))
        else:
            a = rng.randrange(0, max(1, Rl - Q))
            q = mutate(rng, w[a:a + Q + 8])[:Q].ljust(Q, b"A")
        if kind == 2:
            w = w[: rng.randint(min(Rl, max(1, Q // 2)), Rl)]
        if kind == 3:
            w = bytes(((c | 0x20) if rng.random() < 0.3 else c) for c in w)
            q = bytes((ord("N") if rng.random() < 0.03 else c) for c in q)
        if kind == 4:
            q = bytes(((c | 0x20) if rng.random() < 0.2 else c) for c in q)
        out = R.sw_kernel(q, w, Q, Rl)
        cases.append(dict(q=q.decode("latin-1"), w=w.decode("latin-1"), Q=Q, R=Rl,
                          score=out["score"], start=out["start"], end=out["end"],
                          len=out["len"], qcons=out["qcons"].decode("latin-1"),
                          rcons=out["rcons"].decode("latin-1")))
    return cases


def messy_fasta(rng, n_seqs=4, total=30_000):
    out = []
    for r in range(n_seqs):
        n = total // n_seqs + rng.randint(-800, 800)
        s = bytearray(rng.choice(b"ACGT") for _ in range(n))
        for _ in range(10):
            a = rng.randrange(n)
            for i in range(a, min(n, a + rng.randint(1, 30))):
                s[i] = (s[i] | 0x20) if rng.random() < 0.7 else ord("N")
        out.append(b">seq%d desc\n" % r)
        width = rng.choice([50, 60, 61, 70])
        for i in range(0, n, width):
            out.append(bytes(s[i:i + width]) + b"\n")
    return b"".join(out)


def main():
    if not R.available():
        sys.exit("oracle/_ref is not built (needs the reference sources)")
    rng = random.Random(2024)
    json.dump(sw_pairs(rng), open(os.path.join(HERE, "sw_pairs.json"), "w"), indent=0)
    fa = messy_fasta(rng)
    look, rep, ri, rp = R.index(fa, 8, 6)
    nz = [[h, look[h], rep[h]] for h in range(len(look)) if rep[h] or look[h]]
    json.dump(dict(fasta=fa.decode(), k=8, thres=6, buckets=nz, ref_idx=ri, ref_pos=rp),
              open(os.path.join(HERE, "index_k8.json"), "w"))
    # pipeline: 3 sequences, reads from both strands, an odd read count
    seqs = [bytes(rng.choice(b"ACGT") for _ in range(n)) for n in (9000, 6000, 4000)]
    ref = b"".join(b">chr%d\n" % (i + 1) + b"\n".join(s[j:j + 60] for j in range(0, len(s), 60))
                   + b"\n" for i, s in enumerate(seqs))
    reads = []
    comp = bytes.maketrans(b"ACGT", b"TGCA")
    for i in range(53):
        s = seqs[rng.randrange(3)]
        a = rng.randrange(0, len(s) - 110)
        r = mutate(rng, s[a:a + 110], 0.02, 0.004)[:100].ljust(100, b"A")
        if i % 2:
            r = r.translate(comp)[::-1]
        if i % 11 == 5:
            r = bytes(rng.choice(b"ACGT") for _ in range(100))
        reads.append(b">r%d\n%s\n" % (i, r))
    reads = b"".join(reads)
    out = R.pipeline(ref, reads, DEVICE_MEM)
    open(os.path.join(HERE, "pipeline_ref.fa"), "wb").write(ref)
    open(os.path.join(HERE, "pipeline_reads.fa"), "wb").write(reads)
    open(os.path.join(HERE, "pipeline_out.txt"), "wb").write(out)
    json.dump(dict(device_mem=DEVICE_MEM), open(os.path.join(HERE, "pipeline_meta.json"), "w"))
    # SAM records (-f 1) of the same inputs (every record printed, so the
    # Phase-2 batch size does not change them)
    sam = R.pipeline(ref, reads, DEVICE_MEM, out_format=1)
    assert R.pipeline(ref, reads, SAM_SMALL_MEM, out_format=1) == sam
    open(os.path.join(HERE, "pipeline_out_sam.txt"), "wb").write(sam)
    # the reference CLI's GPU default Phase 1 (lt13 seed-and-extend) on the
    # same inputs, through the default records
    lt13 = R.pipeline(ref, reads, DEVICE_MEM, seeder=1)
    open(os.path.join(HERE, "pipeline_out_lt13.txt"), "wb").write(lt13)
    print("wrote fixtures:", len(out), "bytes of pipeline output,", len(sam), "of SAM output")


if __name__ == "__main__":
    main()
