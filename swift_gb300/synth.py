"""Seeded synthetic inputs with the shapes of the benchmark workloads.

No public dataset is involved: references are i.i.d. uniform ACGT (plus, for
the 50 Mbp workload, diverged copies of repeat units), reads are sampled from
forward-strand positions with substitutions and 1-3 bp indels and are exactly
``read_len`` bases long after mutation.

Workloads (all seeded with numpy PCG64; reference seed 0, reads seed 1):
  small  : 1 Mbp, 1 sequence; 10,000 reads x 100 bp; subs 0.01, indels 0.001
  scale  : 50 Mbp in 24 sequences with log-normal (sigma 0.8) lengths, 10 %
           built from copies of 500 distinct 300 bp units at 3 % divergence;
           1,000,000 reads x 100 bp with the small error model plus 5 %
           uniformly random reads
"""
from __future__ import annotations

import numpy as np

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def fasta_bytes(names, seqs, width: int = 60) -> bytes:
    out = []
    for name, s in zip(names, seqs):
        out.append(b">" + name.encode() + b"\n")
        s = np.asarray(s, dtype=np.uint8)
        n = len(s)
        full = n // width
        if full:
            body = np.empty((full, width + 1), dtype=np.uint8)
            body[:, :width] = s[: full * width].reshape(full, width)
            body[:, width] = ord("\n")
            out.append(body.tobytes())
        if n % width:
            out.append(s[full * width:].tobytes() + b"\n")
    return b"".join(out)


def make_reference(total_bp: int, n_seqs: int = 1, sigma: float = 0.0,
                   repeat_frac: float = 0.0, n_units: int = 500, unit_len: int = 300,
                   divergence: float = 0.03, seed: int = 0):
    """Returns (names, list of uint8 arrays)."""
    rng = _rng(seed)
    if n_seqs == 1 or sigma == 0.0:
        w = np.ones(n_seqs)
    else:
        w = rng.lognormal(0.0, sigma, n_seqs)
    lens = np.floor(w / w.sum() * total_bp).astype(np.int64)
    lens[0] += total_bp - lens.sum()
    cat = ACGT[rng.integers(0, 4, total_bp, dtype=np.uint8)]
    if repeat_frac > 0:
        units = ACGT[rng.integers(0, 4, (n_units, unit_len))]
        n_slots = total_bp // unit_len
        n_copies = int(round(repeat_frac * total_bp / unit_len))
        slots = rng.choice(n_slots, size=n_copies, replace=False)
        which = rng.integers(0, n_units, n_copies)
        copies = units[which].copy()
        mut = rng.random(copies.shape) < divergence
        shift = rng.integers(1, 4, copies.shape)
        code = np.searchsorted(ACGT, copies)
        copies = np.where(mut, ACGT[(code + shift) % 4], copies)
        idx = (slots[:, None] * unit_len + np.arange(unit_len)[None, :]).reshape(-1)
        cat[idx] = copies.reshape(-1)
    seqs, o = [], 0
    for L in lens:
        seqs.append(cat[o:o + L])
        o += L
    names = [f"chr{i + 1}" for i in range(n_seqs)]
    return names, seqs


def make_reads(seqs, n_reads: int, read_len: int = 100, sub_p: float = 0.01,
               indel_p: float = 0.001, random_frac: float = 0.0, seed: int = 1,
               len_range: tuple[int, int] | None = None):
    """Returns (names, list of bytes, origins (seq, pos) or (-1, -1))."""
    rng = _rng(seed)
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    cum = np.concatenate([[0], np.cumsum(lens)])
    if len_range is None:
        rl = np.full(n_reads, read_len, dtype=np.int64)
    else:
        rl = rng.integers(len_range[0], len_range[1] + 1, n_reads)
    pad = 16
    need = rl + pad
    # uniform positions over the concatenation, rejecting reads that run off
    # the end of their sequence
    pos = rng.integers(0, cum[-1], n_reads)
    sid = np.searchsorted(cum, pos, side="right") - 1
    off = pos - cum[sid]
    bad = off + need > lens[sid]
    while bad.any():
        pos[bad] = rng.integers(0, cum[-1], bad.sum())
        sid[bad] = np.searchsorted(cum, pos[bad], side="right") - 1
        off[bad] = pos[bad] - cum[sid[bad]]
        bad = off + need > lens[sid]
    is_rand = rng.random(n_reads) < random_frac
    maxl = int(need.max())
    cat = np.concatenate(seqs)
    src = cat[(pos[:, None] + np.arange(maxl)[None, :]).clip(0, len(cat) - 1)]
    # substitutions (to a different base)
    code = np.searchsorted(ACGT, src)
    sub = rng.random(src.shape) < sub_p
    src = np.where(sub, ACGT[(code + rng.integers(1, 4, src.shape)) % 4], src)
    out = []
    n_ind = rng.binomial(rl, indel_p)
    for r in range(n_reads):
        L = int(rl[r])
        if is_rand[r]:
            out.append(ACGT[rng.integers(0, 4, L)].tobytes())
            continue
        s = src[r]
        if n_ind[r] == 0:
            out.append(s[:L].tobytes())
            continue
        buf = bytearray(s.tobytes())
        for _ in range(int(n_ind[r])):
            at = int(rng.integers(0, L))
            size = int(rng.integers(1, 4))
            if rng.random() < 0.5:
                buf[at:at] = ACGT[rng.integers(0, 4, size)].tobytes()
            else:
                del buf[at:at + size]
        if len(buf) < L:
            buf += ACGT[rng.integers(0, 4, L - len(buf))].tobytes()
        out.append(bytes(buf[:L]))
    names = [f"r{i}" for i in range(n_reads)]
    origins = [(-1, -1) if is_rand[i] else (int(sid[i]), int(off[i])) for i in range(n_reads)]
    return names, out, origins


def paired_reads(seqs, n_pairs: int, read_len: int = 100, frag: tuple[int, int] = (200, 500),
                 sub_p: float = 0.01, seed: int = 1):
    """Paired-end reads: fragments of length U[frag] from uniform positions;
    mate 1 the fragment's first read_len bases, mate 2 the reverse complement
    of its last read_len bases, substitutions at sub_p; names r<i>/1 and
    r<i>/2.  Returns (reads FASTA 1, reads FASTA 2)."""
    rng = _rng(seed)
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    cum = np.concatenate([[0], np.cumsum(lens)])
    f = rng.integers(frag[0], frag[1] + 1, n_pairs)
    pos = rng.integers(0, cum[-1], n_pairs)
    sid = np.searchsorted(cum, pos, side="right") - 1
    off = pos - cum[sid]
    bad = off + f > lens[sid]
    while bad.any():
        pos[bad] = rng.integers(0, cum[-1], bad.sum())
        sid[bad] = np.searchsorted(cum, pos[bad], side="right") - 1
        off[bad] = pos[bad] - cum[sid[bad]]
        bad = off + f > lens[sid]
    cat = np.concatenate(seqs)
    L = read_len
    m1 = cat[pos[:, None] + np.arange(L)[None, :]]
    m2 = cat[(pos + f - L)[:, None] + np.arange(L)[None, :]]
    comp = np.zeros(256, np.uint8)
    for a, c in zip(b"ACGT", b"TGCA"):
        comp[a] = c
    m2 = comp[m2[:, ::-1]]
    for m in (m1, m2):
        code = np.searchsorted(ACGT, m)
        sub = rng.random(m.shape) < sub_p
        m[:] = np.where(sub, ACGT[(code + rng.integers(1, 4, m.shape)) % 4], m)

    def fasta(mat, mate):
        body = np.empty((n_pairs, L + 1), np.uint8)
        body[:, :L] = mat
        body[:, L] = ord("\n")
        rows = [b">r%d/%d\n" % (i, mate) + body[i].tobytes() for i in range(n_pairs)]
        return b"".join(rows)

    return fasta(m1, 1), fasta(m2, 2)


def reads_fasta(names, reads) -> bytes:
    parts = []
    for n, r in zip(names, reads):
        parts.append(b">" + n.encode() + b"\n" + r + b"\n")
    return b"".join(parts)


def pairs_workload(n_reads: int, seed: int = 1, max_regions: int = 64, flank: int = 64,
                   ref=None):
    """Batched Phase-2 workload of varying lengths: reads with L ~ U[36, 250]
    (1 % substitutions, 0.1 % indels), each against n ~ U{1..max_regions}
    regions: its true region and n - 1 decoys at uniform positions, each
    region [pos - flank, pos + L + flank) clipped to its sequence.  Returns
    (reference bytes, reads bytes, q_off, q_len, r_off, r_len) with offsets
    into the two byte strings (the reference without line breaks)."""
    if ref is None:
        _, seqs = make_reference(50_000_000, 24, sigma=0.8, repeat_frac=0.10, n_units=500,
                                 unit_len=300, divergence=0.03, seed=0)
    else:
        seqs = ref
    rng = _rng(seed + 100)
    _, reads, origins = make_reads(seqs, n_reads, sub_p=0.01, indel_p=0.001, seed=seed,
                                   len_range=(36, 250))
    lens = np.array([len(x) for x in seqs], dtype=np.int64)
    cum = np.concatenate([[0], np.cumsum(lens)])
    rl = np.array([len(r) for r in reads], dtype=np.int64)
    roff = np.concatenate([[0], np.cumsum(rl)[:-1]])
    n_reg = rng.integers(1, max_regions + 1, n_reads)
    read_of = np.repeat(np.arange(n_reads), n_reg)
    first = np.concatenate([[0], np.cumsum(n_reg)[:-1]])
    is_true = np.zeros(len(read_of), dtype=bool)
    is_true[first] = True
    pos = rng.integers(0, cum[-1], len(read_of))  # decoys: uniform
    tsid = np.array([o[0] for o in origins], dtype=np.int64)
    toff = np.array([o[1] for o in origins], dtype=np.int64)
    pos[first] = cum[tsid] + toff
    sid = np.searchsorted(cum, pos, side="right") - 1
    L = rl[read_of]
    lo = np.maximum(pos - flank, cum[sid])
    hi = np.minimum(pos + L + flank, cum[sid + 1])
    return (np.concatenate(seqs).tobytes(), b"".join(reads), roff[read_of], L.astype(np.int32),
            lo.astype(np.int64), (hi - lo).astype(np.int32))


def long_workload(n_queries: int = 20_000, seed: int = 1, ref_bp: int = 100_000_000):
    """Long-region Phase-2 workload: a uniform reference; queries of
    L ~ U[1000, 4000] bases (3 % substitutions, 0.5 % indels of 1-3 bases)
    from uniform positions, each against one region of length
    U[max(2000, L + 200), 8000] that contains the query's origin.  Returns
    (reference bytes, queries bytes, q_off, q_len, r_off, r_len)."""
    rng = _rng(seed)
    ref = ACGT[rng.integers(0, 4, ref_bp, dtype=np.uint8)]
    L = rng.integers(1000, 4001, n_queries)
    RL = np.array([int(rng.integers(max(2000, l + 200), 8001)) for l in L])
    pos = rng.integers(0, ref_bp - 8200, n_queries)
    qs = []
    for i in range(n_queries):
        s = ref[pos[i]:pos[i] + L[i]].copy()
        code = np.searchsorted(ACGT, s)
        sub = rng.random(L[i]) < 0.03
        s = np.where(sub, ACGT[(code + rng.integers(1, 4, L[i])) % 4], s)
        buf = bytearray(s.tobytes())
        for _ in range(int(rng.binomial(L[i], 0.005))):
            at = int(rng.integers(0, len(buf)))
            size = int(rng.integers(1, 4))
            if rng.random() < 0.5:
                buf[at:at] = ACGT[rng.integers(0, 4, size)].tobytes()
            else:
                del buf[at:at + size]
        while len(buf) < L[i]:
            buf += ACGT[rng.integers(0, 4, 1)].tobytes()
        qs.append(bytes(buf[:L[i]]))
    lead = np.array([int(rng.integers(0, RL[i] - L[i] + 1)) for i in range(n_queries)])
    r_off = np.clip(pos - lead, 0, ref_bp - RL)
    q_off = np.concatenate([[0], np.cumsum(L)[:-1]])
    return (ref.tobytes(), b"".join(qs), q_off.astype(np.int64), L.astype(np.int32),
            r_off.astype(np.int64), RL.astype(np.int32))


def workload(name: str, n_reads: int | None = None):
    """(reference FASTA, reads FASTA, description) of a named workload."""
    if name == "small":
        names, seqs = make_reference(1_000_000, 1, seed=0)
        n = n_reads or 10_000
        rn, rs, _ = make_reads(seqs, n, 100, 0.01, 0.001, 0.0, seed=1)
        desc = dict(workload="small", ref_bp=1_000_000, ref_seqs=1, reads=n, read_len=100)
    elif name == "scale":
        names, seqs = make_reference(50_000_000, 24, sigma=0.8, repeat_frac=0.10,
                                     n_units=500, unit_len=300, divergence=0.03, seed=0)
        n = n_reads or 1_000_000
        rn, rs, _ = make_reads(seqs, n, 100, 0.01, 0.001, 0.05, seed=1)
        desc = dict(workload="scale", ref_bp=50_000_000, ref_seqs=24, reads=n, read_len=100,
                    repeat_frac=0.10)
    else:
        raise ValueError(name)
    return fasta_bytes(names, seqs), reads_fasta(rn, rs), desc
