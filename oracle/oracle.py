"""ctypes binding of the CPU restatement in ``swift_oracle.c``.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke``
and the ``cpu_baseline`` leg of ``bench.py`` as the checker.  The product
never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libswift_oracle.so")


def build() -> str:
    subprocess.check_call(["make", "-s", "-C", HERE, "oracle"])
    return LIB_PATH


class Params(C.Structure):
    _fields_ = [
        ("seed_len", C.c_int),
        ("ignore_thres", C.c_int),
        ("max_hits", C.c_int),
        ("match", C.c_int),
        ("mismatch", C.c_int),
        ("gap_open", C.c_int),
        ("gap_ext", C.c_int),
        ("qry_len", C.c_int),
        ("device_mem", C.c_longlong),
        ("threads", C.c_int),
        ("out_format", C.c_int),
        ("seeder", C.c_int),
        ("max_read_len", C.c_int),
    ]


class Match(C.Structure):
    _fields_ = [
        ("slot_read", C.c_int32),
        ("strand", C.c_int32),
        ("ref_idx", C.c_int32),
        ("shift", C.c_int32),
        ("ref_pos", C.c_int32),
    ]


class Aln(C.Structure):
    _fields_ = [
        ("score", C.c_float),
        ("start", C.c_int32),
        ("end", C.c_int32),
        ("len", C.c_int32),
        ("cell_max", C.c_int32),
    ]


def default_params(**kw) -> Params:
    p = Params(12, 1000, 3, 2, -1, -10, -1, 0, 0, os.cpu_count() or 1, 0, 0, 0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.so_hash.argtypes = [C.c_char_p, C.c_int]
        L.so_index_build.argtypes = [C.c_char_p, C.c_size_t, C.c_int, C.c_int,
                                     C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]
        L.so_index_free.argtypes = [C.c_void_p]
        for f in ("so_index_num_buckets", "so_index_total", "so_index_num_refs"):
            getattr(L, f).argtypes = [C.c_void_p]
        for f in ("so_index_start", "so_index_repeats", "so_index_actual"):
            getattr(L, f).argtypes = [C.c_void_p, C.c_int]
        L.so_index_postings.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.so_index_buckets.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.so_best_hits.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                   C.c_void_p, C.c_void_p, C.c_void_p]
        L.so_map_query.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_int,
                                   C.c_void_p, C.c_void_p, C.c_void_p]
        L.so_revcomp.argtypes = [C.c_char_p, C.c_int, C.c_char_p]
        L.so_sw.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_int,
                            C.c_int, C.c_int, C.POINTER(Aln), C.c_char_p, C.c_char_p,
                            C.c_void_p]
        L.so_align.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t,
                               C.POINTER(Params), C.POINTER(C.c_void_p),
                               C.POINTER(C.c_size_t), C.c_char_p, C.c_size_t]
        L.so_phase1.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t,
                                C.POINTER(Params), C.POINTER(C.c_void_p),
                                C.POINTER(C.c_int), C.c_char_p, C.c_size_t]
        L.so_free.argtypes = [C.c_void_p]
        L.so_sw_batch.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_char_p, C.c_int, C.c_int,
                                  C.c_long, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_void_p]
        L.so_phase1_paired.argtypes = [C.c_char_p, C.c_size_t] * 3 + [
            C.POINTER(Params), C.POINTER(C.c_void_p), C.POINTER(C.c_long), C.c_char_p, C.c_size_t]
        L.so_align_paired.argtypes = [C.c_char_p, C.c_size_t] * 3 + [
            C.POINTER(Params), C.c_uint, C.c_uint, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t),
            C.c_char_p, C.c_size_t]
        L.so_lt13_map.argtypes = [C.c_char_p, C.c_size_t, C.c_int, C.c_int, C.c_char_p, C.c_int,
                                  C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
        L.so_session_create.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(Params),
                                        C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]
        L.so_session_align.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t,
                                       C.POINTER(C.c_void_p), C.POINTER(C.c_size_t),
                                       C.c_char_p, C.c_size_t]
        L.so_session_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def hash_kmer(s: bytes, k: int) -> int:
    return lib().so_hash(s, k)


def revcomp(s: bytes) -> bytes:
    out = C.create_string_buffer(len(s) + 1)
    lib().so_revcomp(s, len(s), out)
    return out.raw[: len(s)]


class Index:
    def __init__(self, fasta: bytes, k: int = 12, thres: int = 1000):
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = lib().so_index_build(fasta, len(fasta), k, thres, C.byref(h), err, 512)
        if rc != 0:
            raise OracleError(err.value.decode())
        self._h = h
        self.k = k

    def __del__(self):
        if getattr(self, "_h", None):
            lib().so_index_free(self._h)
            self._h = None

    @property
    def num_buckets(self) -> int:
        return lib().so_index_num_buckets(self._h)

    @property
    def total(self) -> int:
        return lib().so_index_total(self._h)

    def start(self, h: int) -> int:
        return lib().so_index_start(self._h, h)

    def repeats(self, h: int) -> int:
        return lib().so_index_repeats(self._h, h)

    def actual(self, h: int) -> int:
        return lib().so_index_actual(self._h, h)

    def postings(self):
        import numpy as np
        n = self.total + 1
        ri = np.zeros(n, dtype=np.int8)
        rp = np.zeros(n, dtype=np.int32)
        lib().so_index_postings(self._h, ri.ctypes.data, rp.ctypes.data)
        return ri, rp

    def buckets(self):
        """lookupTable[] and numRepeatsPerTuple[] of every bucket."""
        import numpy as np
        look = np.zeros(self.num_buckets, dtype=np.int32)
        rep = np.zeros(self.num_buckets, dtype=np.int32)
        lib().so_index_buckets(self._h, look.ctypes.data, rep.ctypes.data)
        return look, rep

    def map_query(self, seq: bytes, max_hits: int = 3):
        import numpy as np
        ri = np.zeros(max_hits, dtype=np.int8)
        sh = np.zeros(max_hits, dtype=np.int32)
        rp = np.zeros(max_hits, dtype=np.int32)
        n = lib().so_map_query(self._h, seq, len(seq), max_hits, ri.ctypes.data,
                               sh.ctypes.data, rp.ctypes.data)
        return [(int(ri[i]), int(sh[i]), int(rp[i])) for i in range(n)]


def best_hits(max_hits, ref_idx, shift, ref_pos):
    import numpy as np
    ri = np.ascontiguousarray(ref_idx, dtype=np.int8)
    sh = np.ascontiguousarray(shift, dtype=np.int32)
    rp = np.ascontiguousarray(ref_pos, dtype=np.int32)
    o_ri = np.zeros(max(max_hits, 1), dtype=np.int8)
    o_sh = np.zeros(max(max_hits, 1), dtype=np.int32)
    o_rp = np.zeros(max(max_hits, 1), dtype=np.int32)
    n = lib().so_best_hits(max_hits, ri.ctypes.data, sh.ctypes.data, rp.ctypes.data,
                           len(ri), o_ri.ctypes.data, o_sh.ctypes.data, o_rp.ctypes.data)
    return [(int(o_ri[i]), int(o_sh[i]), int(o_rp[i])) for i in range(n)]


def sw(q: bytes, r: bytes, Q: int | None = None, R: int | None = None,
       m=2, x=-1, o=-10, e=-1, want_dirs=False):
    """GPU-kernel Smith-Waterman semantics for one pair; q and r are padded
    with NUL bytes to Q and R."""
    import numpy as np
    Q = len(q) if Q is None else Q
    R = len(r) if R is None else R
    qb = q.ljust(Q, b"\0")[:Q]
    rb = r.ljust(R, b"\0")[:R]
    a = Aln()
    qc = C.create_string_buffer(Q + R + 2)
    rc = C.create_string_buffer(Q + R + 2)
    dirs = np.zeros((Q + 1) * (R + 1), dtype=np.uint8) if want_dirs else None
    lib().so_sw(qb, Q, rb, R, m, x, o, e, C.byref(a), qc, rc,
                dirs.ctypes.data if dirs is not None else None)
    n = a.len
    res = dict(score=a.score, start=a.start, end=a.end, len=a.len,
               cell_max=a.cell_max, qcons=qc.raw[:max(n, 0)], rcons=rc.raw[:max(n, 0)])
    if want_dirs:
        res["dirs"] = dirs.reshape(Q + 1, R + 1)
    return res


def sw_batch(qry: bytes, Q: int, ref: bytes, R: int, n: int, m=2, x=-1, o=-10, e=-1,
             threads: int | None = None):
    """so_sw over n pairs in the alignSequences layout (query i at i*(Q+1),
    window i at i*(R+1)) on host threads; returns (score, start, end, len)
    arrays."""
    import numpy as np
    out = (Aln * max(n, 1))()
    lib().so_sw_batch(qry, Q, Q + 1, ref, R, R + 1, n, m, x, o, e,
                      threads or os.cpu_count() or 1, out)
    a = np.ctypeslib.as_array(out).view(np.dtype([("score", "<f4"), ("start", "<i4"),
                                                   ("end", "<i4"), ("len", "<i4"),
                                                   ("cell_max", "<i4")]))[:n]
    return a["score"].copy(), a["start"].copy(), a["end"].copy(), a["len"].copy()


def align(ref: bytes, reads: bytes, params: Params | None = None) -> bytes:
    p = params or default_params()
    out = C.c_void_p()
    n = C.c_size_t()
    err = C.create_string_buffer(512)
    rc = lib().so_align(ref, len(ref), reads, len(reads), C.byref(p), C.byref(out),
                        C.byref(n), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    data = C.string_at(out, n.value)
    lib().so_free(out)
    return data


def phase1(ref: bytes, reads: bytes, params: Params | None = None):
    """Match-file records: list of (read, strand, ref_idx, shift, ref_pos)."""
    p = params or default_params()
    out = C.c_void_p()
    n = C.c_int()
    err = C.create_string_buffer(512)
    rc = lib().so_phase1(ref, len(ref), reads, len(reads), C.byref(p), C.byref(out),
                         C.byref(n), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    arr = C.cast(out, C.POINTER(Match))
    res = [(arr[i].slot_read, arr[i].strand, arr[i].ref_idx, arr[i].shift, arr[i].ref_pos)
           for i in range(n.value)]
    lib().so_free(out)
    return res


def lt13_map(ref: bytes, seq: bytes, k: int = 12, thres: int = 1000):
    """lt13 seed-and-extend hits of one query strand: [(ref_idx, ref_pos)]."""
    ri = (C.c_int32 * 3)()
    rp = (C.c_int32 * 3)()
    err = C.create_string_buffer(512)
    n = lib().so_lt13_map(ref, len(ref), k, thres, seq, len(seq), ri, rp, err, 512)
    if n < 0:
        raise OracleError(err.value.decode())
    return [(ri[i], rp[i]) for i in range(n)]


class Session:
    """Reference parsed and indexed once; align() runs Phase 1 + Phase 2."""

    def __init__(self, ref: bytes, params: Params | None = None):
        self.p = params or default_params()
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = lib().so_session_create(ref, len(ref), C.byref(self.p), C.byref(h), err, 512)
        if rc != 0:
            raise OracleError(err.value.decode())
        self._h = h

    def align(self, reads: bytes) -> bytes:
        out = C.c_void_p()
        n = C.c_size_t()
        err = C.create_string_buffer(512)
        rc = lib().so_session_align(self._h, reads, len(reads), C.byref(out), C.byref(n), err, 512)
        if rc != 0:
            raise OracleError(err.value.decode())
        data = C.string_at(out, n.value)
        lib().so_free(out)
        return data

    def __del__(self):
        if getattr(self, "_h", None):
            lib().so_session_free(self._h)
            self._h = None


def phase1_paired(ref: bytes, reads1: bytes, reads2: bytes, params: Params | None = None):
    """Paired-end Phase-1 records: (id, rev, mate, ref_idx, shift, offset, read)."""
    p = params or default_params()
    out = C.c_void_p()
    n = C.c_long()
    err = C.create_string_buffer(512)
    rc = lib().so_phase1_paired(ref, len(ref), reads1, len(reads1), reads2, len(reads2),
                                C.byref(p), C.byref(out), C.byref(n), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    a = C.cast(out, C.POINTER(C.c_int32))
    res = [tuple(a[7 * i + f] for f in range(7)) for i in range(n.value)]
    lib().so_free(out)
    return res


def align_paired(ref: bytes, reads1: bytes, reads2: bytes, params: Params | None = None,
                 min_frag: int = 99, max_frag: int = 600) -> bytes:
    """The paired-end pipeline's output (MIN/MAX_FRAG_SIZE defaults)."""
    p = params or default_params()
    out = C.c_void_p()
    n = C.c_size_t()
    err = C.create_string_buffer(512)
    rc = lib().so_align_paired(ref, len(ref), reads1, len(reads1), reads2, len(reads2),
                               C.byref(p), min_frag, max_frag, C.byref(out), C.byref(n), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    res = C.string_at(out, n.value)
    lib().so_free(out)
    return res
