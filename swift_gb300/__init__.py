"""Python binding of libswift_gb300.so, the GB300 SWIFT aligner hot path.

The library is the product: CUDA kernels for sm_103a behind the C ABI in
include/swift_gb300.h.  This module only loads it with ctypes.  There is no
CPU fallback: if the library cannot be loaded or no CUDA device is present,
every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libswift_gb300.so")
CLI_PATH = os.path.join(HERE, "swift")

SWIFT_OK = 0
ERRORS = {-1: "argument", -2: "input", -3: "cuda", -4: "memory", -5: "limit", -6: "device",
          -7: "cancelled"}
SERVE_STATES = {0: "queued", 1: "running", 2: "done", 3: "cancelled"}

# Exported C symbols (kept in step with include/swift_gb300.h).
EXPORTS = [
    "swift_params_default", "swift_ctx_create", "swift_ctx_destroy", "swift_last_error",
    "swift_ctx_info", "swift_ctx_set_sw_path", "swift_ctx_set_tuning",
    "swift_index_build", "swift_index_destroy", "swift_index_info", "swift_index_export",
    "swift_seed", "swift_seed_lt13", "swift_index_save", "swift_index_load",
    "swift_index_params", "swift_align_paired", "swift_align_paired_into", "swift_sw_batch", "swift_align", "swift_reads_upload",
    "swift_reads_destroy", "swift_align_resident", "swift_fetch_output",
    "swift_align_files", "swift_free", "swift_peak_dpx", "swift_align_into",
    "swift_sw_batch_noalloc", "swift_sw_pairs", "swift_server_create", "swift_server_submit",
    "swift_server_wait", "swift_server_destroy", "swift_server_poll", "swift_server_cancel",
]


class SwiftError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"swift error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("seed_len", C.c_int32), ("ignore_thres", C.c_int32), ("max_hits", C.c_int32),
        ("match", C.c_int32), ("mismatch", C.c_int32), ("gap_open", C.c_int32),
        ("gap_ext", C.c_int32), ("qry_len", C.c_int32), ("device_mem", C.c_int64),
        ("out_format", C.c_int32), ("seeder", C.c_int32), ("max_read_len", C.c_int32),
    ]


class Match(C.Structure):
    _fields_ = [("read", C.c_int32), ("strand", C.c_int32), ("ref_idx", C.c_int32),
                ("shift", C.c_int32), ("ref_pos", C.c_int32)]


class PairsStats(C.Structure):
    _fields_ = [("ms", C.c_double), ("pairs", C.c_int64), ("cells", C.c_int64),
                ("segments", C.c_int64), ("generic_pairs", C.c_int64), ("launches", C.c_int64),
                ("shape_lanes", C.c_int32 * 8), ("shape_rows", C.c_int32 * 8),
                ("tune_ms", C.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["shapes"] = {q: (self.shape_lanes[c], self.shape_rows[c])
                       for c, q in enumerate((32, 64, 104, 128, 208, 256, 320))
                       if self.shape_lanes[c]}
        del d["shape_lanes"], d["shape_rows"]
        return d


class RequestStats(C.Structure):
    _fields_ = [("queue_ms", C.c_double), ("run_ms", C.c_double), ("total_ms", C.c_double),
                ("device_ms", C.c_double), ("reads", C.c_int64), ("out_bytes", C.c_int64),
                ("wave_requests", C.c_int64), ("wave_reads", C.c_int64),
                ("parse_ms", C.c_double), ("wave_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [
        ("seed_ms", C.c_double), ("pairs_ms", C.c_double), ("sw_ms", C.c_double),
        ("select_ms", C.c_double), ("traceback_ms", C.c_double), ("format_ms", C.c_double),
        ("total_ms", C.c_double),
        ("reads", C.c_int64), ("records", C.c_int64), ("printed", C.c_int64),
        ("cells", C.c_int64), ("out_bytes", C.c_int64),
        ("seed_overflow_strands", C.c_int64), ("sw_generic_pairs", C.c_int64),
        ("launches", C.c_int64), ("host_parse_ms", C.c_double), ("h2d_ms", C.c_double),
        ("d2h_ms", C.c_double), ("traced_pairs", C.c_int64), ("bound_pruned", C.c_int64),
        ("retraced_pairs", C.c_int64), ("first_pass_ms", C.c_double),
        ("first_pass_cells", C.c_int64), ("first_pass_kind", C.c_int64),
        ("trace_ms", C.c_double), ("trace_cells", C.c_int64), ("lcs_kept", C.c_int64),
        ("seed_kernel_ms", C.c_double), ("seed_model_bytes", C.c_int64),
        ("sw_cells_computed", C.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    """Loads the in-tree library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SwiftError(-3, f"{LIB_PATH} is missing: run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        vp, i32, i64, sz = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t
        L.swift_params_default.argtypes = [C.POINTER(Params)]
        L.swift_params_default.restype = None
        L.swift_ctx_create.argtypes = [C.c_int, vp, C.POINTER(vp)]
        L.swift_ctx_destroy.argtypes = [vp]
        L.swift_last_error.argtypes = [vp]
        L.swift_last_error.restype = C.c_char_p
        L.swift_ctx_info.argtypes = [vp, C.POINTER(i64), C.POINTER(i32)]
        L.swift_ctx_set_sw_path.argtypes = [vp, i32]
        L.swift_ctx_set_tuning.argtypes = [vp, i32]
        L.swift_index_build.argtypes = [vp, C.c_char_p, sz, i32, i32, C.POINTER(vp)]
        L.swift_index_destroy.argtypes = [vp]
        L.swift_index_info.argtypes = [vp, vp, C.POINTER(i32), C.POINTER(i64), C.POINTER(i64)]
        L.swift_index_export.argtypes = [vp, vp, vp, vp, vp, vp]
        L.swift_seed.argtypes = [vp, vp, C.c_char_p, sz, i32, vp, i64, C.POINTER(i64)]
        L.swift_seed_lt13.argtypes = [vp, vp, C.c_char_p, sz, vp, i64, C.POINTER(i64)]
        L.swift_index_save.argtypes = [vp, vp, C.c_char_p]
        L.swift_index_load.argtypes = [vp, C.c_char_p, C.POINTER(vp)]
        L.swift_index_params.argtypes = [vp, vp, C.POINTER(i32), C.POINTER(i32)]
        L.swift_align_paired.argtypes = [vp, vp, C.c_char_p, sz, C.c_char_p, sz, C.POINTER(Params),
                                         C.c_uint32, C.c_uint32, C.POINTER(vp), C.POINTER(sz),
                                         vp]
        L.swift_align_paired_into.argtypes = [vp, vp, vp, sz, vp, sz, C.POINTER(Params),
                                              C.c_uint32, C.c_uint32, vp, sz, C.POINTER(sz), vp]
        f32 = C.c_float
        L.swift_sw_batch.argtypes = [vp, vp, vp, i32, i32, i64, f32, f32, f32, f32,
                                     vp, vp, vp, vp, vp, vp]
        L.swift_align.argtypes = [vp, vp, vp, sz, C.POINTER(Params), C.POINTER(vp),
                                  C.POINTER(sz), C.POINTER(Stats)]
        L.swift_sw_batch_noalloc.argtypes = L.swift_sw_batch.argtypes
        L.swift_server_create.argtypes = [i32, vp, C.POINTER(Params), i32, i64, C.POINTER(vp)]
        L.swift_server_submit.argtypes = [vp, C.c_char_p, sz, C.POINTER(i64)]
        L.swift_server_wait.argtypes = [vp, i64, C.POINTER(vp), C.POINTER(sz),
                                        C.POINTER(RequestStats), C.c_char_p, sz]
        L.swift_server_destroy.argtypes = [vp]
        L.swift_server_poll.argtypes = [vp, i64, C.POINTER(i32)]
        L.swift_server_cancel.argtypes = [vp, i64]
        L.swift_sw_pairs.argtypes = [vp, vp, vp, vp, vp, vp, vp, i64, i32, i32, i32, i32,
                                     vp, vp, vp, vp, vp, vp, i64, i32, C.POINTER(PairsStats)]
        L.swift_align_into.argtypes = [vp, vp, vp, sz, C.POINTER(Params), vp, sz, C.POINTER(sz),
                                       C.POINTER(Stats)]
        L.swift_reads_upload.argtypes = [vp, C.c_char_p, sz, C.POINTER(vp)]
        L.swift_reads_destroy.argtypes = [vp]
        L.swift_align_resident.argtypes = [vp, vp, vp, C.POINTER(Params), C.POINTER(sz),
                                           C.POINTER(Stats)]
        L.swift_fetch_output.argtypes = [vp, vp, sz]
        L.swift_align_files.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p,
                                        C.POINTER(Params)]
        L.swift_peak_dpx.argtypes = [vp, C.POINTER(C.c_double)]
        L.swift_free.argtypes = [vp]
        L.swift_free.restype = None
        _lib = L
    return _lib


def default_params(**kw) -> Params:
    p = Params()
    lib().swift_params_default(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Context:
    """A device context: one CUDA stream, one host thread at a time."""

    def __init__(self, device: int = 0, stream: int | None = None):
        h = C.c_void_p()
        rc = lib().swift_ctx_create(device, C.c_void_p(stream) if stream else None, C.byref(h))
        if rc != SWIFT_OK:
            raise SwiftError(rc, "context creation failed (is a CUDA device present?)")
        self._h = h

    def _check(self, rc):
        if rc != SWIFT_OK:
            raise SwiftError(rc, lib().swift_last_error(self._h).decode(errors="replace"))

    def info(self):
        mem, sms = C.c_int64(), C.c_int32()
        self._check(lib().swift_ctx_info(self._h, C.byref(mem), C.byref(sms)))
        return dict(total_mem=mem.value, sm_count=sms.value)

    def set_sw_path(self, path: int):
        """0: bounded selection (default); 1: generic kernel only; 2: exact score
        of every packed-path pair.  All give identical output."""
        self._check(lib().swift_ctx_set_sw_path(self._h, path))

    def set_tuning(self, mode: int):
        """swift_sw_pairs' packed shapes: 1 autotuned (default), 0 fixed
        defaults, k >= 2 the (k-2)-th candidate of every class."""
        self._check(lib().swift_ctx_set_tuning(self._h, mode))

    def peak_dpx_cells_per_s(self) -> float:
        v = C.c_double()
        self._check(lib().swift_peak_dpx(self._h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "_h", None):
            lib().swift_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    # -- index ---------------------------------------------------------------
    def index(self, ref_fasta: bytes, seed_len: int = 12, ignore_thres: int = 1000) -> "Index":
        return Index(self, ref_fasta, seed_len, ignore_thres)

    def reads(self, reads_fasta: bytes) -> "Reads":
        return Reads(self, reads_fasta)

    # -- Phase 1 ---------------------------------------------------------------
    def seed(self, index: "Index", reads_fasta: bytes, max_hits: int = 3):
        n = C.c_int64()
        self._check(lib().swift_seed(self._h, index._h, reads_fasta, len(reads_fasta), max_hits,
                                     None, 0, C.byref(n)))
        arr = (Match * max(n.value, 1))()
        self._check(lib().swift_seed(self._h, index._h, reads_fasta, len(reads_fasta), max_hits,
                                     arr, n.value, C.byref(n)))
        return [(m.read, m.strand, m.ref_idx, m.shift, m.ref_pos) for m in arr[: n.value]]

    def seed_lt13(self, index: "Index", reads_fasta: bytes):
        """lt13 seed-and-extend records (search2Queries)."""
        n = C.c_int64()
        self._check(lib().swift_seed_lt13(self._h, index._h, reads_fasta, len(reads_fasta),
                                          None, 0, C.byref(n)))
        arr = (Match * max(n.value, 1))()
        self._check(lib().swift_seed_lt13(self._h, index._h, reads_fasta, len(reads_fasta),
                                          arr, n.value, C.byref(n)))
        return [(m.read, m.strand, m.ref_idx, m.shift, m.ref_pos) for m in arr[: n.value]]

    # -- Phase 2 on explicit pairs (alignSequences) ------------------------------
    def sw_batch(self, queries, windows, Q: int, R: int, match=2, mismatch=-1, gap_open=-10,
                 gap_ext=-1):
        import numpy as np
        n = len(queries)
        q = np.zeros((n, Q + 1), dtype=np.uint8)
        w = np.zeros((n, R + 1), dtype=np.uint8)
        for i, (a, b) in enumerate(zip(queries, windows)):
            q[i, : min(len(a), Q)] = np.frombuffer(a[:Q], dtype=np.uint8)
            w[i, : min(len(b), R)] = np.frombuffer(b[:R], dtype=np.uint8)
        score = np.zeros(n, np.float32)
        start = np.zeros(n, np.int32)
        end = np.zeros(n, np.int32)
        ln = np.zeros(n, np.int32)
        qc = np.zeros((n, Q + R + 2), np.uint8)
        rc = np.zeros((n, Q + R + 2), np.uint8)
        self._check(lib().swift_sw_batch(
            self._h, q.ctypes.data, w.ctypes.data, Q, R, n, match, mismatch, gap_open, gap_ext,
            score.ctypes.data, start.ctypes.data, end.ctypes.data, ln.ctypes.data,
            qc.ctypes.data, rc.ctypes.data))
        out = []
        for i in range(n):
            L = int(ln[i])
            out.append(dict(score=float(score[i]), start=int(start[i]), end=int(end[i]), len=L,
                            qcons=bytes(qc[i, :max(L, 0)]), rcons=bytes(rc[i, :max(L, 0)])))
        return out

    def sw_batch_arrays(self, q, w, Q: int, R: int, match=2, mismatch=-1, gap_open=-10,
                        gap_ext=-1):
        """swift_sw_batch on host arrays already in its layout: q is n x (Q+1)
        and w n x (R+1) uint8.  Returns (score, start, end, len) arrays; the
        consensus strings stay in host buffers this call allocates."""
        import numpy as np
        n = q.shape[0]
        score = np.zeros(n, np.float32)
        start, end, ln = (np.zeros(n, np.int32) for _ in range(3))
        qc = np.zeros((n, Q + R + 2), np.uint8)
        rc = np.zeros((n, Q + R + 2), np.uint8)
        self._check(lib().swift_sw_batch(
            self._h, q.ctypes.data, w.ctypes.data, Q, R, n, match, mismatch, gap_open, gap_ext,
            score.ctypes.data, start.ctypes.data, end.ctypes.data, ln.ctypes.data,
            qc.ctypes.data, rc.ctypes.data))
        return score, start, end, ln

    def sw_pairs(self, qry: bytes, q_off, q_len, ref: bytes, r_off, r_len, match=2, mismatch=-1,
                 gap_open=-10, gap_ext=-1, mode=0, consensus=True):
        """Pairs of varying lengths (host buffers): pair i aligns
        qry[q_off[i]:q_off[i]+q_len[i]] against ref[r_off[i]:r_off[i]+r_len[i]].
        Returns (dict of numpy arrays, stats); consensus strings as lists of
        bytes when asked for."""
        import numpy as np
        q_off = np.ascontiguousarray(q_off, dtype=np.int64)
        r_off = np.ascontiguousarray(r_off, dtype=np.int64)
        q_len = np.ascontiguousarray(q_len, dtype=np.int32)
        r_len = np.ascontiguousarray(r_len, dtype=np.int32)
        n = len(q_len)
        qb = np.frombuffer(qry, dtype=np.uint8) if len(qry) else np.zeros(1, np.uint8)
        rb = np.frombuffer(ref, dtype=np.uint8) if len(ref) else np.zeros(1, np.uint8)
        out = {k: np.zeros(max(n, 1), np.int32) for k in ("score", "start", "end", "len")}
        cs = 0
        qc = rc = None
        if consensus and n:
            cs = (int((q_len + r_len).max()) + 2 + 3) & ~3
            qc = np.zeros((n, cs), np.uint8)
            rc = np.zeros((n, cs), np.uint8)
        st = PairsStats()
        self._check(lib().swift_sw_pairs(
            self._h, qb.ctypes.data, q_off.ctypes.data, q_len.ctypes.data, rb.ctypes.data,
            r_off.ctypes.data, r_len.ctypes.data, n, match, mismatch, gap_open, gap_ext,
            out["score"].ctypes.data, out["start"].ctypes.data, out["end"].ctypes.data,
            out["len"].ctypes.data, qc.ctypes.data if qc is not None else None,
            rc.ctypes.data if rc is not None else None, cs, mode, C.byref(st)))
        res = {k: v[:n] for k, v in out.items()}
        if qc is not None:
            res["qcons"] = [bytes(qc[i, :max(int(res["len"][i]), 0)]) for i in range(n)]
            res["rcons"] = [bytes(rc[i, :max(int(res["len"][i]), 0)]) for i in range(n)]
        return res, st.as_dict()

    # -- whole pipeline ----------------------------------------------------------
    def align(self, index: "Index", reads_fasta, params: Params | None = None,
              stats: bool = False, nbytes: int | None = None):
        """reads_fasta: bytes, or an integer host address (e.g. of pinned
        memory) with nbytes."""
        p = params or default_params(seed_len=index.seed_len, ignore_thres=index.ignore_thres)
        out = C.c_void_p()
        n = C.c_size_t()
        st = Stats()
        if isinstance(reads_fasta, int):
            ptr, ln = C.c_void_p(reads_fasta), nbytes
        else:
            ptr, ln = C.cast(C.c_char_p(reads_fasta), C.c_void_p), len(reads_fasta)
        self._check(lib().swift_align(self._h, index._h, ptr, ln,
                                      C.byref(p), C.byref(out), C.byref(n), C.byref(st)))
        data = C.string_at(out, n.value) if n.value else b""
        lib().swift_free(out)
        return (data, st.as_dict()) if stats else data

    def align_paired(self, index: "Index", reads1: bytes, reads2: bytes,
                     params: Params | None = None, min_frag: int = 99, max_frag: int = 600,
                     stats: bool = False):
        """Paired-end alignment (-q / -q2); the output text (and stats)."""
        p = params or default_params(seed_len=index.seed_len, ignore_thres=index.ignore_thres)
        out = C.c_void_p()
        n = C.c_size_t()
        st = Stats()
        self._check(lib().swift_align_paired(self._h, index._h, reads1, len(reads1), reads2,
                                             len(reads2), C.byref(p), min_frag, max_frag,
                                             C.byref(out), C.byref(n), C.byref(st)))
        text = C.string_at(out, n.value)
        lib().swift_free(out)
        return (text, st.as_dict()) if stats else text

    def align_paired_into(self, index: "Index", ptr1: int, len1: int, ptr2: int, len2: int,
                          out_ptr: int, cap: int, params: Params | None = None,
                          min_frag: int = 99, max_frag: int = 600):
        """Paired-end alignment with host buffers given by address (for
        example pinned memory); returns (bytes written, stats)."""
        p = params or default_params(seed_len=index.seed_len, ignore_thres=index.ignore_thres)
        n = C.c_size_t()
        st = Stats()
        self._check(lib().swift_align_paired_into(self._h, index._h, C.c_void_p(ptr1), len1,
                                                  C.c_void_p(ptr2), len2, C.byref(p), min_frag,
                                                  max_frag, C.c_void_p(out_ptr), cap, C.byref(n),
                                                  C.byref(st)))
        return n.value, st.as_dict()

    def align_into(self, index: "Index", reads_ptr: int, nbytes: int, out_ptr: int, cap: int,
                   params: Params | None = None):
        """Pipeline with host input and output buffers given by address (for
        example pinned memory); returns (bytes written, stats)."""
        p = params or default_params(seed_len=index.seed_len, ignore_thres=index.ignore_thres)
        n = C.c_size_t()
        st = Stats()
        self._check(lib().swift_align_into(self._h, index._h, C.c_void_p(reads_ptr), nbytes,
                                           C.byref(p), C.c_void_p(out_ptr), cap, C.byref(n),
                                           C.byref(st)))
        return n.value, st.as_dict()

    def align_resident(self, index: "Index", reads: "Reads", params: Params | None = None):
        p = params or default_params(seed_len=index.seed_len, ignore_thres=index.ignore_thres)
        n = C.c_size_t()
        st = Stats()
        self._check(lib().swift_align_resident(self._h, index._h, reads._h, C.byref(p),
                                               C.byref(n), C.byref(st)))
        return n.value, st.as_dict()

    def fetch_output(self, n: int) -> bytes:
        buf = C.create_string_buffer(max(n, 1))
        self._check(lib().swift_fetch_output(self._h, buf, n))
        return buf.raw[:n]

    def align_files(self, qry_path: str, ref_path: str, out_path: str,
                    params: Params | None = None):
        p = params or default_params()
        self._check(lib().swift_align_files(self._h, qry_path.encode(), ref_path.encode(),
                                            out_path.encode(), C.byref(p)))


class Server:
    """Serving loop over a resident index: submit reads, wait for records."""

    def __init__(self, index: "Index", device: int = 0, params: Params | None = None,
                 workers: int = 2, mem_budget: int = 0):
        self._index = index  # keeps the index alive
        p = params or default_params(seed_len=index.seed_len, ignore_thres=index.ignore_thres)
        h = C.c_void_p()
        rc = lib().swift_server_create(device, index._h, C.byref(p), workers, mem_budget,
                                       C.byref(h))
        if rc != SWIFT_OK:
            raise SwiftError(rc, "server creation failed")
        self._h = h

    def submit(self, reads_fasta: bytes) -> int:
        t = C.c_int64()
        rc = lib().swift_server_submit(self._h, reads_fasta, len(reads_fasta), C.byref(t))
        if rc != SWIFT_OK:
            raise SwiftError(rc, "submit failed")
        return t.value

    def poll(self, ticket: int) -> str:
        """'queued', 'running', 'done' or 'cancelled', without blocking."""
        st = C.c_int32()
        rc = lib().swift_server_poll(self._h, ticket, C.byref(st))
        if rc != SWIFT_OK:
            raise SwiftError(rc, "unknown ticket")
        return SERVE_STATES[st.value]

    def cancel(self, ticket: int) -> bool:
        """Cancels a request that has not started; False once it runs or is done."""
        rc = lib().swift_server_cancel(self._h, ticket)
        if rc == -5:
            return False
        if rc != SWIFT_OK:
            raise SwiftError(rc, "unknown ticket")
        return True

    def wait(self, ticket: int):
        """Returns (records bytes, stats dict); raises SwiftError for a failed request."""
        out, n, st = C.c_void_p(), C.c_size_t(), RequestStats()
        err = C.create_string_buffer(512)
        rc = lib().swift_server_wait(self._h, ticket, C.byref(out), C.byref(n), C.byref(st),
                                     err, 512)
        data = C.string_at(out, n.value) if out.value and n.value else b""
        if out.value:
            lib().swift_free(out)
        if rc != SWIFT_OK:
            raise SwiftError(rc, err.value.decode(errors="replace"))
        return data, st.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            lib().swift_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Index:
    """Device-resident reference (FASTA bytes, 2-bit codes) and SSAHA index."""

    def __init__(self, ctx: Context, ref_fasta: bytes | None, seed_len=12, ignore_thres=1000,
                 _handle=None):
        if _handle is None:
            h = C.c_void_p()
            ctx._check(lib().swift_index_build(ctx._h, ref_fasta, len(ref_fasta), seed_len,
                                               ignore_thres, C.byref(h)))
        else:
            h = _handle
            k, t = C.c_int32(), C.c_int32()
            ctx._check(lib().swift_index_params(ctx._h, h, C.byref(k), C.byref(t)))
            seed_len, ignore_thres = k.value, t.value
        self._h = h
        self.ctx = ctx
        self.seed_len = seed_len
        self.ignore_thres = ignore_thres

    @classmethod
    def load(cls, ctx: Context, path: str) -> "Index":
        """An index saved by Index.save, rebuilt on ctx's device."""
        h = C.c_void_p()
        ctx._check(lib().swift_index_load(ctx._h, path.encode(), C.byref(h)))
        return cls(ctx, None, _handle=h)

    def save(self, path: str):
        self.ctx._check(lib().swift_index_save(self.ctx._h, self._h, path.encode()))

    def info(self):
        nr, tot, nb = C.c_int32(), C.c_int64(), C.c_int64()
        self.ctx._check(lib().swift_index_info(self.ctx._h, self._h, C.byref(nr), C.byref(tot),
                                               C.byref(nb)))
        return dict(n_refs=nr.value, total=tot.value, n_buckets=nb.value)

    def export(self):
        import numpy as np
        inf = self.info()
        look = np.zeros(inf["n_buckets"], np.int32)
        rep = np.zeros(inf["n_buckets"], np.int32)
        ri = np.zeros(inf["total"] + 1, np.int8)
        rp = np.zeros(inf["total"] + 1, np.int32)
        self.ctx._check(lib().swift_index_export(self.ctx._h, self._h, look.ctypes.data,
                                                 rep.ctypes.data, ri.ctypes.data, rp.ctypes.data))
        return look, rep, ri, rp

    def close(self):
        if getattr(self, "_h", None):
            lib().swift_index_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Reads:
    """Reads parsed and resident on the device."""

    def __init__(self, ctx: Context, reads_fasta: bytes):
        h = C.c_void_p()
        ctx._check(lib().swift_reads_upload(ctx._h, reads_fasta, len(reads_fasta), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().swift_reads_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
