"""satsuma2_gb300 -- the satsuma2 cross-correlation hot path on one GB300.

The compute lives in ``libsatsuma2_gb300.so`` (hand-written sm_103a CUDA
behind the C ABI of ``include/satsuma2_xcorr.h``).  This module is a thin
ctypes binding of that ABI that mirrors the reference slave's per-pair
interface (HomologyByXCorr::Align / FilterMatches,
analysis/HomologyByXCorrSlave.cc:168-253): chunk pairs in, t_result records out,
with the slave's -cutoff / -cutoff_fast / -l / -t_chunk / -q_chunk /
-prob_table parameters.  There is no CPU path: if the library is missing or no
GPU is usable, every call raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsatsuma2_gb300.so")

XC_OK = 0
MAX_FFT_LEN = 32768   # longest FFT the library runs (XC_ERR_UNSUPPORTED beyond)
ERRORS = {-1: "XC_ERR_ARG", -2: "XC_ERR_CUDA", -3: "XC_ERR_NOMEM", -4: "XC_ERR_CAPACITY",
          -5: "XC_ERR_INPUT", -6: "XC_ERR_TIMEOUT", -7: "XC_ERR_UNSUPPORTED", -8: "XC_ERR_BUSY"}

# t_result (analysis/WorkQueue.h:23-33), 72 bytes.
RESULT_DTYPE = np.dtype([
    ("query_id", "<u8"), ("target_id", "<u8"), ("query_size", "<u8"),
    ("qstart", "<u8"), ("tstart", "<u8"), ("len", "<u8"),
    ("reverse", "u1"), ("_pad", "V7"), ("prob", "<f8"), ("ident", "<f8")])
assert RESULT_DTYPE.itemsize == 72

# Every entry point include/satsuma2_xcorr.h declares.
EXPORTS = ("xc_create", "xc_destroy", "xc_align_pairs", "xc_batch_upload", "xc_batch_run",
           "xc_batch_results", "xc_batch_free", "xc_batch_launches", "xc_batch_run_timed",
           "xc_transfer_stats", "xc_submit", "xc_wait", "xc_serving_stats", "xc_debug_pair",
           "xc_version", "xc_device_name", "xc_align_pair_noalloc", "xc_batch_offsets",
           "xc_batch_straddles", "xc_tune", "xc_apply_tuning")
STRAD_CAP = 16   # XC_STRAD_CAP: near-threshold lags listed per pair strand


class XCError(RuntimeError):
    def __init__(self, code, what):
        self.code = code
        super().__init__("%s: %s (%d)" % (what, ERRORS.get(code, "error"), code))


class Params(ctypes.Structure):
    """xc_params (include/satsuma2_xcorr.h)."""
    _fields_ = [("cutoff", ctypes.c_double), ("cutoff_fast", ctypes.c_double),
                ("min_prob", ctypes.c_double), ("target_total", ctypes.c_double),
                ("min_len", ctypes.c_int), ("t_chunk", ctypes.c_int), ("q_chunk", ctypes.c_int),
                ("fft_len", ctypes.c_int), ("use_prob_table", ctypes.c_int),
                ("prob_table_cutoff", ctypes.c_double), ("max_batch", ctypes.c_int),
                ("result_slots", ctypes.c_int)]


class Pair(ctypes.Structure):
    """xc_pair (include/satsuma2_xcorr.h)."""
    _fields_ = [("tseq", ctypes.c_char_p), ("tlen", ctypes.c_int), ("t_chunk_start", ctypes.c_int),
                ("target_id", ctypes.c_ulong), ("qseq", ctypes.c_char_p), ("qlen", ctypes.c_int),
                ("q_chunk_start", ctypes.c_int), ("query_id", ctypes.c_ulong),
                ("query_size", ctypes.c_ulong), ("fast", ctypes.c_int)]


# xc_pair as a numpy record (LP64 layout of the ctypes Pair above, 64 bytes):
# arrays of chunk pairs that point into caller-owned sequence buffers.
PAIR_DTYPE = np.dtype({"names": ["tseq", "tlen", "t_chunk_start", "target_id", "qseq", "qlen", "q_chunk_start",
                                 "query_id", "query_size", "fast"],
                       "formats": ["<u8", "<i4", "<i4", "<u8", "<u8", "<i4", "<i4", "<u8", "<u8", "<i4"],
                       "offsets": [0, 8, 12, 16, 24, 32, 36, 40, 48, 56], "itemsize": 64})

_lib = None


def load(path=LIB_PATH):
    """Loads the CUDA library; raises (never falls back) when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError("%s is not built: run satsuma2_gb300.build" % path)
    lib = ctypes.CDLL(path)
    vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
    lib.xc_create.argtypes = [ctypes.POINTER(Params), i, ctypes.POINTER(vp)]
    lib.xc_destroy.argtypes = [vp]
    lib.xc_align_pairs.argtypes = [vp, vp, sz, vp, sz, ctypes.POINTER(sz), vp]
    lib.xc_align_pair_noalloc.argtypes = [vp, vp, vp, sz, ctypes.POINTER(sz)]
    lib.xc_batch_upload.argtypes = [vp, vp, sz, ctypes.POINTER(vp)]
    lib.xc_batch_run.argtypes = [vp, vp, vp]
    lib.xc_batch_results.argtypes = [vp, vp, vp, sz, ctypes.POINTER(sz), vp]
    lib.xc_batch_free.argtypes = [vp, vp]
    lib.xc_batch_launches.argtypes = [vp, vp]
    lib.xc_batch_run_timed.argtypes = [vp, vp, vp, vp]
    lib.xc_batch_offsets.argtypes = [vp, vp, vp, sz, ctypes.POINTER(sz), vp]
    lib.xc_batch_straddles.argtypes = [vp, vp, vp, vp]
    lib.xc_transfer_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    lib.xc_submit.argtypes = [vp, vp, sz, ctypes.POINTER(ctypes.c_uint64)]
    lib.xc_wait.argtypes = [vp, ctypes.c_uint64, i, vp, sz, ctypes.POINTER(sz)]
    lib.xc_serving_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    lib.xc_debug_pair.argtypes = [vp, ctypes.POINTER(Pair), vp, vp, vp, vp, vp, vp, i, ctypes.POINTER(i)]
    lib.xc_tune.argtypes = [vp, ctypes.c_char_p, sz, ctypes.POINTER(sz)]
    lib.xc_apply_tuning.argtypes = [vp, ctypes.c_char_p]
    lib.xc_version.restype = ctypes.c_char_p
    lib.xc_device_name.argtypes = [vp, ctypes.c_char_p, sz]
    _lib = lib
    return lib


def _check(code, what):
    if code != XC_OK:
        raise XCError(code, what)


def make_pairs(items):
    """items: iterable of dicts or (t, q) tuples -> (ctypes array, keepalive).

    Dict keys: t, q, t_chunk_start, target_id, q_chunk_start, query_id,
    query_size, fast."""
    items = list(items)
    arr = (Pair * len(items))()
    keep = []
    for k, it in enumerate(items):
        if isinstance(it, tuple):
            it = {"t": it[0], "q": it[1]}
        t, q = bytes(it["t"]), bytes(it["q"])
        keep.append((t, q))
        arr[k] = Pair(t, len(t), it.get("t_chunk_start", 0), it.get("target_id", 0), q, len(q),
                      it.get("q_chunk_start", 0), it.get("query_id", 0),
                      it.get("query_size", len(q)), it.get("fast", 0))
    return arr, keep


def _pair_array(items):
    """items as a contiguous PAIR_DTYPE array if it is an array of chunk-pair
    records (PAIR_DTYPE, or a concatenation that lost its padding), else None."""
    if isinstance(items, np.ndarray) and items.dtype.names == PAIR_DTYPE.names:
        return np.ascontiguousarray(items.astype(PAIR_DTYPE, copy=False))
    return None


def block_pairs(tbuf, tchunks, qbuf, qchunks, tf, tt, qf, qt, target_id=0, query_id=0, fast=0):
    """The chunk pairs of one t_pair block (inclusive chunk ranges), query-major
    as HomologyByXCorr::align_target loops (HomologyByXCorrSlave.cc:281-299),
    as a PAIR_DTYPE array pointing into tbuf / qbuf (numpy uint8 arrays the
    caller keeps alive).  tchunks / qchunks: int arrays of (start, end) per
    chunk of one target and one query sequence."""
    tchunks = np.asarray(tchunks, np.int64)
    qchunks = np.asarray(qchunks, np.int64)
    ti = np.arange(tf, tt + 1)
    qi = np.arange(qf, qt + 1)
    T, Qg = np.meshgrid(ti, qi)          # query outer, target inner
    T, Qg = T.ravel(), Qg.ravel()
    out = np.zeros(len(T), PAIR_DTYPE)
    out["tseq"] = tbuf.ctypes.data + tchunks[T, 0]
    out["tlen"] = tchunks[T, 1] - tchunks[T, 0]
    out["t_chunk_start"] = tchunks[T, 0]
    out["target_id"] = target_id
    out["qseq"] = qbuf.ctypes.data + qchunks[Qg, 0]
    out["qlen"] = qchunks[Qg, 1] - qchunks[Qg, 0]
    out["q_chunk_start"] = qchunks[Qg, 0]
    out["query_id"] = query_id
    out["query_size"] = len(qbuf)
    out["fast"] = fast
    return out


class XCorr:
    """One GPU context of the chunk-pair cross-correlation path.

    Mirrors the slave's parameters (HomologyByXCorrSlave.cc:334-384).  min_prob
    defaults to 0.99, the threshold the slave actually applies (:76)."""

    def __init__(self, cutoff=1.8, cutoff_fast=2.9, min_prob=0.99, target_total=4096.0, min_len=0,
                 t_chunk=4096, q_chunk=4096, fft_len=0, prob_table=False, prob_table_cutoff=0.9999,
                 max_batch=4096, result_slots=64, device=0):
        self.lib = load()
        self.params = Params(cutoff, cutoff_fast, min_prob, target_total, min_len, t_chunk, q_chunk,
                             fft_len, 1 if prob_table else 0, prob_table_cutoff, max_batch, result_slots)
        self.ctx = ctypes.c_void_p()
        _check(self.lib.xc_create(ctypes.byref(self.params), device, ctypes.byref(self.ctx)), "xc_create")

    def close(self):
        if self.ctx:
            self.lib.xc_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def device_name(self):
        buf = ctypes.create_string_buffer(256)
        self.lib.xc_device_name(self.ctx, buf, 256)
        return buf.value.decode()

    def align(self, items, with_counts=False):
        """Runs chunk pairs (both strands) -> structured array of t_result
        records.  items as for make_pairs, or a PAIR_DTYPE array."""
        pa = _pair_array(items)
        if pa is not None:
            items = pa   # (kept alive for the call)
            arr, n = ctypes.c_void_p(items.ctypes.data), len(items)
        else:
            arr, keep = make_pairs(items)
            n = len(arr)
        cap = max(64, 16 * n)
        counts = np.zeros(n, np.uint64)
        while True:
            out = np.zeros(cap, RESULT_DTYPE)
            n_out = ctypes.c_size_t()
            r = self.lib.xc_align_pairs(self.ctx, arr, n, out.ctypes.data, cap, ctypes.byref(n_out),
                                        counts.ctypes.data)
            if r == -4 and n_out.value > cap:
                cap = n_out.value
                continue
            _check(r, "xc_align_pairs")
            res = out[:n_out.value].copy()
            return (res, counts) if with_counts else res

    def debug_pair(self, t, q, seg_cap=1 << 16, signals=True, **kw):
        """Stage outputs of one pair: signals, xc, offsets, raw segments per
        strand.  With signals=False no signals are written, and an A/C/G/T
        pair at FFT 8192 runs on the both-strands correlation kernel, as in
        xc_align_pairs; signal output runs it one CTA per strand."""
        arr, keep = make_pairs([dict(t=t, q=q, **kw)])
        Lmax = MAX_FFT_LEN
        sig = np.zeros(2 * 8 * Lmax if signals else 1, np.float32)
        xcv = np.zeros(2 * Lmax, np.float32)
        offs = np.zeros(2 * Lmax, np.int32)
        noffs = np.zeros(2, np.int32)
        segs = np.zeros(2 * seg_cap * 3, np.int32)
        nsegs = np.zeros(2, np.int32)
        L = ctypes.c_int()
        _check(self.lib.xc_debug_pair(self.ctx, arr, sig.ctypes.data if signals else None, xcv.ctypes.data,
                                      offs.ctypes.data,
                                      noffs.ctypes.data, segs.ctypes.data, nsegs.ctypes.data, seg_cap,
                                      ctypes.byref(L)), "xc_debug_pair")
        L = L.value
        sig = sig[:2 * 8 * L].reshape(2, 2, 4, L) if signals else None
        return {
            "L": L,
            "signals": sig,
            "xc": xcv[:2 * L].reshape(2, L),
            "offsets": [offs[s * L:s * L + noffs[s]].copy() for s in range(2)],
            "segments": [segs[s * seg_cap * 3:s * seg_cap * 3 + 3 * min(nsegs[s], seg_cap)].reshape(-1, 3).copy()
                         for s in range(2)],
        }

    # device-resident batches -------------------------------------------------
    def upload(self, items):
        """Packs and uploads chunk pairs (items as for align, or a PAIR_DTYPE
        array) as a device-resident batch."""
        pa = _pair_array(items)
        if pa is not None:
            items = pa   # (kept alive for the call)
            arr, n = ctypes.c_void_p(items.ctypes.data), len(items)
        else:
            arr, keep = make_pairs(items)
            n = len(arr)
        b = ctypes.c_void_p()
        _check(self.lib.xc_batch_upload(self.ctx, arr, n, ctypes.byref(b)), "xc_batch_upload")
        return Batch(self, b, n)

    # serving -------------------------------------------------------------------
    def submit(self, items):
        """Queues chunk pairs for the GPU; items as for align, the (array,
        keepalive) pair make_pairs returns (built ahead of time), or a
        PAIR_DTYPE array (block_pairs).  The library copies the sequences."""
        pa = _pair_array(items)
        if pa is not None:
            items = pa   # (kept alive for the call)
            arr, n = ctypes.c_void_p(items.ctypes.data), len(items)
        else:
            if isinstance(items, tuple) and len(items) == 2 and isinstance(items[0], ctypes.Array):
                arr, keep = items
            else:
                arr, keep = make_pairs(items)
            n = len(arr)
        t = ctypes.c_uint64()
        _check(self.lib.xc_submit(self.ctx, arr, n, ctypes.byref(t)), "xc_submit")
        return t.value

    def wait(self, ticket, timeout_ms=10000, cap=4096):
        while True:
            out = np.zeros(cap, RESULT_DTYPE)
            n_out = ctypes.c_size_t()
            r = self.lib.xc_wait(self.ctx, ticket, timeout_ms, out.ctypes.data, cap, ctypes.byref(n_out))
            if r == -4 and n_out.value > cap:
                cap = n_out.value
                continue
            _check(r, "xc_wait")
            return out[:n_out.value].copy()

    def tune(self):
        """Runs the autotuner (xc_tune) and returns its table (text)."""
        n = ctypes.c_size_t()
        buf = ctypes.create_string_buffer(8192)
        _check(self.lib.xc_tune(self.ctx, buf, len(buf), ctypes.byref(n)), "xc_tune")
        return buf.value.decode()

    def apply_tuning(self, table):
        _check(self.lib.xc_apply_tuning(self.ctx, table.encode()), "xc_apply_tuning")

    def transfer_stats(self):
        h, d = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self.lib.xc_transfer_stats(self.ctx, ctypes.byref(h), ctypes.byref(d)), "xc_transfer_stats")
        return h.value, d.value

    def serving_stats(self):
        p50, p99 = ctypes.c_double(), ctypes.c_double()
        c, p = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self.lib.xc_serving_stats(self.ctx, ctypes.byref(p50), ctypes.byref(p99), ctypes.byref(c),
                                         ctypes.byref(p)), "xc_serving_stats")
        return {"p50_ms": p50.value, "p99_ms": p99.value, "completed": c.value, "pairs": p.value}


class Batch:
    """A packed, device-resident batch (xc_batch_*)."""

    def __init__(self, xcorr, handle, n):
        self.x, self.h, self.n = xcorr, handle, n

    def run(self, stream=None):
        _check(self.x.lib.xc_batch_run(self.x.ctx, self.h, stream), "xc_batch_run")

    def run_timed(self, stream=None):
        """Runs once with stage events; returns [corr_ms, scan_ms, finalize_ms]."""
        ms = np.zeros(3, np.float32)
        _check(self.x.lib.xc_batch_run_timed(self.x.ctx, self.h, stream, ms.ctypes.data), "xc_batch_run_timed")
        return ms.tolist()

    def launches(self):
        return self.x.lib.xc_batch_launches(self.x.ctx, self.h)

    def results(self, with_counts=False):
        cap = max(64, 16 * self.n)
        counts = np.zeros(self.n, np.uint64)
        while True:
            out = np.zeros(cap, RESULT_DTYPE)
            n_out = ctypes.c_size_t()
            r = self.x.lib.xc_batch_results(self.x.ctx, self.h, out.ctypes.data, cap, ctypes.byref(n_out),
                                            counts.ctypes.data)
            if r == -4 and n_out.value > cap:
                cap = n_out.value
                continue
            _check(r, "xc_batch_results")
            res = out[:n_out.value].copy()
            return (res, counts) if with_counts else res

    def offsets(self):
        """FindTop offsets of the last run: list over pairs of [forward, reverse] int32 arrays."""
        counts = np.zeros(2 * self.n, np.int32)
        n_out = ctypes.c_size_t()
        _check(self.x.lib.xc_batch_offsets(self.x.ctx, self.h, None, 0, ctypes.byref(n_out), counts.ctypes.data),
               "xc_batch_offsets")
        offs = np.zeros(max(1, n_out.value), np.int32)
        _check(self.x.lib.xc_batch_offsets(self.x.ctx, self.h, offs.ctypes.data, len(offs), ctypes.byref(n_out),
                                           counts.ctypes.data), "xc_batch_offsets")
        out, o = [], 0
        for i in range(self.n):
            a = offs[o:o + counts[2 * i]].copy()
            o += counts[2 * i]
            b = offs[o:o + counts[2 * i + 1]].copy()
            o += counts[2 * i + 1]
            out.append([a, b])
        return out

    def straddles(self):
        """Near-threshold lags of the last run: (counts [n, 2], lags [n, 2, STRAD_CAP], -1 padded)."""
        counts = np.zeros(2 * self.n, np.int32)
        lags = np.zeros(2 * self.n * STRAD_CAP, np.int32)
        _check(self.x.lib.xc_batch_straddles(self.x.ctx, self.h, counts.ctypes.data, lags.ctypes.data),
               "xc_batch_straddles")
        return counts.reshape(self.n, 2), lags.reshape(self.n, 2, STRAD_CAP)

    def free(self):
        if self.h:
            self.x.lib.xc_batch_free(self.x.ctx, self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
