"""ctypes binding of oracle/_ref/libswift_ref.so: the reference's own code
(compiled from its sources by oracle/ref_harness) for validating the oracle.

TEST INFRASTRUCTURE ONLY.  Available only where the reference sources were
present at build time; callers skip when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libswift_ref.so")
TMP = os.path.join(HERE, "_ref", "tmp")

_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(LIB_PATH)
        f, i, p = C.c_float, C.c_int, C.c_void_p
        sw_args = [C.c_char_p, i, C.c_char_p, i, f, f, f, f, p, p, p, p, C.c_char_p, C.c_char_p]
        L.ref_sw_kernel.argtypes = sw_args
        L.ref_sw_cpu.argtypes = sw_args
        L.ref_index.argtypes = [C.c_char_p, i, i, p, p, p, p, p, p]
        L.ref_map_query.argtypes = [C.c_char_p, C.c_char_p, i, i, p, p, p]
        L.ref_best_hits.argtypes = [i, p, p, p, i, p, p, p]
        L.ref_pipeline.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                   C.c_longlong, i, i, f, f, f, f]
        L.ref_pipeline.restype = C.c_long
        L.ref_pipeline_fmt.argtypes = L.ref_pipeline.argtypes + [i, i]
        L.ref_pipeline_fmt.restype = C.c_long
        L.ref_pipeline_paired.argtypes = [C.c_char_p] * 5 + [C.c_longlong, i, f, f, f, f, i,
                                                             C.c_uint, C.c_uint]
        L.ref_pipeline_paired.restype = C.c_long
        _lib = L
    return _lib


def _sw(fn, q: bytes, r: bytes, Q=None, R=None, m=2, x=-1, o=-10, e=-1):
    Q = len(q) if Q is None else Q
    R = len(r) if R is None else R
    qb = q.ljust(Q, b"\0")[:Q]
    rb = r.ljust(R, b"\0")[:R]
    score, start, end, ln = C.c_float(), C.c_int(), C.c_int(), C.c_int()
    qc = C.create_string_buffer(Q + R + 2)
    rc = C.create_string_buffer(Q + R + 2)
    fn(qb, Q, rb, R, m, x, o, e, C.byref(score), C.byref(start), C.byref(end), C.byref(ln),
       qc, rc)
    n = max(ln.value, 0)
    return dict(score=score.value, start=start.value, end=end.value, len=ln.value,
                qcons=qc.raw[:n], rcons=rc.raw[:n])


def sw_kernel(q, r, Q=None, R=None, m=2, x=-1, o=-10, e=-1):
    """The reference's GPU kernel, run on CPU fibers (one per CUDA thread)."""
    return _sw(lib().ref_sw_kernel, q, r, Q, R, m, x, o, e)


def sw_cpu(q, r, Q=None, R=None, m=2, x=-1, o=-10, e=-1):
    """The reference's CPU Smith-Waterman."""
    return _sw(lib().ref_sw_cpu, q, r, Q, R, m, x, o, e)


def _tmp(name: str) -> str:
    os.makedirs(TMP, exist_ok=True)
    return os.path.join(TMP, name)


def index(fasta: bytes, k: int, thres: int):
    """lookupTable5Create: (lookup, repeats, ref_idx, ref_pos) as lists."""
    path = _tmp("index_ref.fa")
    open(path, "wb").write(fasta)
    nb, tot = C.c_int(), C.c_int()
    look, rep, ri, rp = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
    lib().ref_index(path.encode(), k, thres, C.byref(nb), C.byref(tot), C.byref(look),
                    C.byref(rep), C.byref(ri), C.byref(rp))
    n = nb.value
    t = tot.value + 1
    look_a = C.cast(look, C.POINTER(C.c_int))
    rep_a = C.cast(rep, C.POINTER(C.c_int))
    ri_a = C.cast(ri, C.POINTER(C.c_byte))
    rp_a = C.cast(rp, C.POINTER(C.c_int))
    return ([look_a[h] for h in range(n)], [rep_a[h] for h in range(n)],
            [ri_a[j] for j in range(t)], [rp_a[j] for j in range(t)])


def map_query(seq: bytes, rev: bytes, is_rev: int, max_hits: int = 3):
    """lookupTable5MapQry on the index of the last index() call (its maximum
    number of hits is the 3 the harness builds it with)."""
    ri = (C.c_byte * 8)()
    sh = (C.c_int * 8)()
    rp = (C.c_int * 8)()
    n = lib().ref_map_query(seq, rev, len(seq), is_rev, ri, sh, rp)
    return [(ri[h], sh[h], rp[h]) for h in range(n)]


def pipeline(ref: bytes, reads: bytes, device_mem: int, seed_len=12, thres=1000,
             m=2, x=-1, o=-10, e=-1, out_format=0, seeder=0) -> bytes:
    """The reference's pipeline file to file; out_format 1: SAM records;
    seeder 1: the lt13 seed-and-extend Phase 1 of search2Queries."""
    return pipeline_with_matches(ref, reads, device_mem, seed_len, thres, m, x, o, e,
                                 out_format, seeder)[0]


def _pipeline_in_process(rp, qp, op, mp, device_mem, seed_len, thres, m, x, o, e, out_format,
                         seeder):
    lib().ref_pipeline_fmt(rp.encode(), qp.encode(), op.encode(), mp.encode(), device_mem,
                           seed_len, thres, m, x, o, e, out_format, seeder)


def pipeline_with_matches(ref: bytes, reads: bytes, device_mem: int, seed_len=12, thres=1000,
                          m=2, x=-1, o=-10, e=-1, out_format=0, seeder=0):
    """(output bytes, Phase-1 records [(name, strand, ref_idx, shift, ref_pos)])."""
    rp, qp, op, mp = (_tmp(n) for n in ("p_ref.fa", "p_reads.fa", "p_out.txt", "p_match.txt"))
    open(rp, "wb").write(ref)
    open(qp, "wb").write(reads)
    args = (rp, qp, op, mp, device_mem, seed_len, thres, m, x, o, e, out_format, seeder)
    if seeder == 1:
        # lookupTable13Create keeps _maxRefPosComposite in a file-static that
        # it never resets: one reference per process, as in the reference
        import subprocess
        import sys
        code = ("import sys; sys.path.insert(0, %r); from oracle import ref as R; "
                "R._pipeline_in_process(*%r)" % (os.path.dirname(HERE), args))
        subprocess.run([sys.executable, "-c", code], check=True, capture_output=True)
    else:
        _pipeline_in_process(*args)
    recs = []
    for line in open(mp, "rb").read().splitlines():
        f = line.split(b"\t")
        recs.append((f[0].decode(), int(f[1]), int(f[2]), int(f[3]), int(f[4])))
    return open(op, "rb").read(), recs


def pipeline_paired(ref: bytes, reads1: bytes, reads2: bytes, device_mem: int, seed_len=12,
                    m=2, x=-1, o=-10, e=-1, out_format=0, min_frag=99, max_frag=600):
    """The reference's paired-end pipeline (-q/-q2) file to file:
    (output bytes, Phase-1 records [(id, name, rev, mate, ref_idx, shift, offset)])."""
    rp, q1, q2, op, mp = (_tmp(n) for n in ("pe_ref.fa", "pe_1.fa", "pe_2.fa", "pe_out.txt",
                                            "pe_match.txt"))
    open(rp, "wb").write(ref)
    open(q1, "wb").write(reads1)
    open(q2, "wb").write(reads2)
    lib().ref_pipeline_paired(rp.encode(), q1.encode(), q2.encode(), op.encode(), mp.encode(),
                              device_mem, seed_len, m, x, o, e, out_format, min_frag, max_frag)
    recs = []
    for line in open(mp, "rb").read().splitlines():
        f = line.split(b"\t")
        recs.append((int(f[0]), f[1].decode(), int(f[2]), int(f[3]), int(f[4]), int(f[5]),
                     int(f[6])))
    return open(op, "rb").read(), recs
