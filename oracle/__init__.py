"""TEST INFRASTRUCTURE ONLY: CPU oracles for the satsuma2 cross-correlation path.

Two libraries live here, both loaded through ctypes:

* ``liboracle.so`` -- ``xcorr_oracle.c``, a plain-C restatement of the
  reference algorithm (FP64 cross-correlation, exact FindTop / DoOne /
  GetMatchProbability / FilterMatches).  It builds anywhere gcc exists.
* ``_ref/libsatsuma_ref.so`` -- the reference's own sources, unmodified,
  compiled by ``build_ref.sh`` together with ``ref_harness.cc``.  The sources
  come from the reference tree, or from the copy ``install_ref.sh`` leaves in
  ``baseline/_ref/satsuma2`` (git-ignored), so the library can be rebuilt on a
  machine without the reference tree; tests that need it skip where neither
  exists.

Only ``tests/``, ``tests/golden/make_golden.py``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU baseline legs may import this package.  The product package
``satsuma2_gb300`` never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsatsuma_ref.so")
REF_SLAVE = os.path.join(HERE, "_ref", "HomologyByXCorrSlave")
# where install_ref.sh puts the reference sources (git-ignored; travels with the tree)
REF_INSTALL = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "satsuma2")

_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_u64 = ctypes.c_uint64

RESULT_DTYPE = np.dtype([
    ("query_id", "<u8"), ("target_id", "<u8"), ("query_size", "<u8"),
    ("qstart", "<u8"), ("tstart", "<u8"), ("len", "<u8"),
    ("reverse", "u1"), ("_pad", "V7"), ("prob", "<f8"), ("ident", "<f8")])
assert RESULT_DTYPE.itemsize == 72


def build(force=False):
    """Compiles xcorr_oracle.c into liboracle.so (seconds; -ffp-contract=off)."""
    src = os.path.join(HERE, "xcorr_oracle.c")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    tmp = ORACLE_SO + ".tmp.%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-ffp-contract=off",
                           "-o", tmp, src, "-lm", "-lpthread"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def install_ref(reference_root=None):
    """Copies the reference's CPU sources (unmodified) into baseline/_ref/satsuma2
    with install_ref.sh; no-op where the reference tree is absent.
    reference_root: None = install_ref.sh's default ($SATSUMA2_REFERENCE or the
    reference checkout of the build machine)."""
    args = ["sh", os.path.join(HERE, "install_ref.sh")]
    if reference_root:
        args.append(reference_root)
    subprocess.check_call(args, stdout=subprocess.DEVNULL)
    return REF_INSTALL if os.path.isdir(os.path.join(REF_INSTALL, "analysis")) else None


def build_ref(reference_root=None):
    """Builds _ref/ from a reference tree: reference_root, else
    $SATSUMA2_REFERENCE, else the installed copy in baseline/_ref/satsuma2.
    Returns the library path, or None when no tree is found.  The build is
    reused while no source is newer than the library."""
    root = reference_root or os.environ.get("SATSUMA2_REFERENCE") or REF_INSTALL
    if not os.path.isfile(os.path.join(root, "analysis", "CrossCorr.cc")):
        return None
    srcs = [os.path.join(HERE, "ref_harness.cc"), os.path.join(HERE, "build_ref.sh")]
    for d in ("analysis", "base", "util"):
        dd = os.path.join(root, d)
        srcs += [os.path.join(dd, f) for f in os.listdir(dd)]
    if (os.path.exists(REF_SO) and os.path.exists(REF_SLAVE)
            and os.path.getmtime(REF_SO) >= max(os.path.getmtime(f) for f in srcs)):
        return REF_SO
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), root], stdout=subprocess.DEVNULL)
    return REF_SO


class _OrcParams(ctypes.Structure):
    _fields_ = [("cutoff", _d), ("cutoff_fast", _d), ("min_prob", _d), ("target_total", _d),
                ("min_len", _i), ("t_chunk", _i), ("q_chunk", _i), ("fft_len", _i),
                ("probtable", _vp), ("probtable_cutoff", _d)]


class _OrcPair(ctypes.Structure):
    _fields_ = [("tseq", ctypes.c_char_p), ("tlen", _i), ("t_chunk_start", _i), ("target_id", _u64),
                ("qseq", ctypes.c_char_p), ("qlen", _i), ("q_chunk_start", _i), ("query_id", _u64),
                ("query_size", _u64), ("fast", _i)]


def _ptr(a):
    return a.ctypes.data_as(_vp)


class Oracle:
    """ctypes view of liboracle.so (the C restatement)."""

    def __init__(self):
        build()
        self.lib = lib = ctypes.CDLL(ORACLE_SO)
        lib.orc_init()
        lib.orc_signal.argtypes = [ctypes.c_char_p, _i, _i, _vp]
        lib.orc_rc.argtypes = [ctypes.c_char_p, _i, ctypes.c_char_p]
        lib.orc_xcorr64.argtypes = [ctypes.c_char_p, _i, ctypes.c_char_p, _i, _i, _vp]
        lib.orc_findtop.argtypes = [_vp, _i, _d, _vp, _i]
        lib.orc_findtop_f32.argtypes = [_vp, _i, _d, _vp, _i]
        lib.orc_thresholds.argtypes = [_vp, _i, _d, _vp]
        lib.orc_doone.argtypes = [ctypes.c_char_p, _i, ctypes.c_char_p, _i, _i, _vp, _i]
        lib.orc_match_prob.restype = _d
        lib.orc_match_prob.argtypes = [ctypes.c_char_p, ctypes.c_char_p, _i, _i, _i, _d, _vp]
        lib.orc_print_ident.restype = _d
        lib.orc_print_ident.argtypes = [ctypes.c_char_p, ctypes.c_char_p, _i, _i, _i]
        lib.orc_probtable_build.argtypes = [_d, _d, _vp, _i]
        lib.orc_probtable_prob.restype = _d
        lib.orc_probtable_prob.argtypes = [_vp, _d, ctypes.c_char_p, ctypes.c_char_p, _i, _i, _i, _vp]
        lib.orc_align_pair.argtypes = [ctypes.POINTER(_OrcParams), ctypes.POINTER(_OrcPair), _vp,
                                       _vp, _vp, _i,
                                       _vp, _i, _vp, _vp, _i, _vp, _vp, _i, _vp]
        lib.orc_align_batch.restype = ctypes.c_longlong
        lib.orc_align_batch.argtypes = [ctypes.POINTER(_OrcParams), ctypes.POINTER(_OrcPair), _i, _i]
        lib.orc_min_matches.restype = _i
        lib.orc_codec.argtypes = [_i, _vp]
        lib.orc_score.argtypes = [_i, _i]
        lib.orc_equal.restype = _d
        lib.orc_equal.argtypes = [_i, _i]

    def signal(self, seq, L):
        out = np.zeros(4 * L, np.float32)
        rc = self.lib.orc_signal(seq, len(seq), L, _ptr(out))
        if rc:
            raise ValueError("orc_signal: bad input")
        return out.reshape(4, L)

    def rc(self, seq):
        buf = ctypes.create_string_buffer(len(seq) + 1)
        self.lib.orc_rc(seq, len(seq), buf)
        return buf.raw[:len(seq)]

    def xcorr64(self, t, q, L):
        out = np.zeros(L, np.float64)
        if self.lib.orc_xcorr64(t, len(t), q, len(q), L, _ptr(out)):
            raise ValueError("orc_xcorr64: bad input")
        return out

    def findtop(self, xc, cutoff):
        xc = np.ascontiguousarray(xc)
        out = np.zeros(len(xc), np.int32)
        if xc.dtype == np.float32:
            n = self.lib.orc_findtop_f32(_ptr(xc), len(xc), cutoff, _ptr(out), len(xc))
        else:
            xc = xc.astype(np.float64)
            n = self.lib.orc_findtop(_ptr(xc), len(xc), cutoff, _ptr(out), len(xc))
        return out[:n].copy()

    def thresholds(self, xc, cutoff):
        xc = np.ascontiguousarray(xc, dtype=np.float64)
        thr = np.zeros(len(xc), np.float64)
        self.lib.orc_thresholds(_ptr(xc), len(xc), cutoff, _ptr(thr))
        return thr

    def doone(self, t, q, pos):
        cap = 1 << 14
        segs = np.zeros(3 * cap, np.int32)
        n = self.lib.orc_doone(t, len(t), q, len(q), pos, _ptr(segs), cap)
        return segs[:3 * n].reshape(n, 3).copy()

    def match_prob(self, t, q, ts, qs, length, target_total):
        ident = ctypes.c_double()
        p = self.lib.orc_match_prob(t, q, ts, qs, length, target_total, ctypes.byref(ident))
        return p, ident.value

    def print_ident(self, t, q, ts, qs, length):
        return self.lib.orc_print_ident(t, q, ts, qs, length)

    def probtable(self, target_size, cutoff, nthreads=8):
        tab = np.zeros(512 * 2048, np.float64)
        self.lib.orc_probtable_build(target_size, cutoff, _ptr(tab), nthreads)
        return tab

    @staticmethod
    def params(cutoff=1.8, cutoff_fast=2.9, min_prob=0.99, target_total=4096.0, min_len=0,
               t_chunk=4096, q_chunk=4096, fft_len=0, probtable=None, probtable_cutoff=0.0):
        return _OrcParams(cutoff, cutoff_fast, min_prob, target_total, min_len, t_chunk, q_chunk,
                          fft_len, probtable.ctypes.data if probtable is not None else None,
                          probtable_cutoff)

    @staticmethod
    def pair(t, q, t_chunk_start=0, target_id=0, q_chunk_start=0, query_id=0, query_size=None,
             fast=0):
        return _OrcPair(t, len(t), t_chunk_start, target_id, q, len(q), q_chunk_start, query_id,
                        len(q) if query_size is None else query_size, fast)

    def align_pair(self, params, pair, xc_in=None, offsets_in=None, want_detail=False):
        """Returns (results, detail) where detail has offsets/segments/xc per strand.
        offsets_in: optional [offsets_fwd, offsets_rc] to use instead of FindTop."""
        L = params.fft_len or 2 * params.t_chunk
        cap = 1 << 14
        res = np.zeros(cap, RESULT_DTYPE)
        offs = np.zeros(2 * L, np.int32)
        noffs = np.zeros(2, np.int32)
        scap = 1 << 16
        segs = np.zeros(2 * 3 * scap, np.int32)
        nsegs = np.zeros(2, np.int32)
        xco = np.zeros(2 * L, np.float64)
        xin = None
        if xc_in is not None:
            xin = np.ascontiguousarray(xc_in, dtype=np.float32).reshape(-1)
        oin = nin = None
        ocap = 0
        if offsets_in is not None:
            ocap = max(1, max(len(o) for o in offsets_in))
            oin = np.zeros(2 * ocap, np.int32)
            nin = np.array([len(offsets_in[0]), len(offsets_in[1])], np.int32)
            for s in range(2):
                oin[s * ocap:s * ocap + len(offsets_in[s])] = offsets_in[s]
        n = self.lib.orc_align_pair(ctypes.byref(params), ctypes.byref(pair),
                                    _ptr(xin) if xin is not None else None,
                                    _ptr(oin) if oin is not None else None,
                                    _ptr(nin) if nin is not None else None, ocap,
                                    _ptr(res), cap,
                                    _ptr(offs), _ptr(noffs), L, _ptr(segs), _ptr(nsegs), scap,
                                    _ptr(xco))
        if n < 0:
            raise ValueError("orc_align_pair: bad input")
        detail = None
        if want_detail:
            detail = {
                "offsets": [offs[s * L:s * L + noffs[s]].copy() for s in range(2)],
                "segments": [segs[s * 3 * scap:s * 3 * scap + 3 * nsegs[s]].reshape(-1, 3).copy()
                             for s in range(2)],
                "xc": xco.reshape(2, L).copy(),
            }
        return res[:n].copy(), detail

    def align_batch(self, params, pairs, nthreads):
        arr = (_OrcPair * len(pairs))(*pairs)
        return self.lib.orc_align_batch(ctypes.byref(params), arr, len(pairs), nthreads)


class Reference:
    """ctypes view of _ref/libsatsuma_ref.so (the reference's own code)."""

    def __init__(self):
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        self.lib = lib = ctypes.CDLL(REF_SO)
        lib.ref_signal.argtypes = [ctypes.c_char_p, _i, _i, _vp]
        lib.ref_rc.argtypes = [ctypes.c_char_p, _i, ctypes.c_char_p]
        lib.ref_xcorr.argtypes = [ctypes.c_char_p, _i, ctypes.c_char_p, _i, _i, _vp]
        lib.ref_findtop.argtypes = [_vp, _i, _d, _vp, _i]
        lib.ref_doone.argtypes = [ctypes.c_char_p, _i, ctypes.c_char_p, _i, _i, _vp, _i]
        lib.ref_match_prob.restype = _d
        lib.ref_match_prob.argtypes = [ctypes.c_char_p, _i, ctypes.c_char_p, _i, _i, _i, _i, _d, _vp]
        lib.ref_print_ident.restype = _d
        lib.ref_print_ident.argtypes = [ctypes.c_char_p, _i, ctypes.c_char_p, _i, _i, _i, _i]
        lib.ref_equal_amb.restype = _d
        lib.ref_equal_amb.argtypes = [_i, _i]
        lib.ref_equal.restype = _d
        lib.ref_equal.argtypes = [_i, _i]
        lib.ref_codec.argtypes = [_i, _vp]
        lib.ref_probtable_new.restype = _vp
        lib.ref_probtable_new.argtypes = [_d, _d]
        lib.ref_probtable_free.argtypes = [_vp]
        lib.ref_probtable_dump.argtypes = [_vp, _vp]
        lib.ref_probtable_prob.restype = _d
        lib.ref_probtable_prob.argtypes = [_vp, ctypes.c_char_p, _i, ctypes.c_char_p, _i, _i, _i, _i, _vp]
        lib.ref_align_pair.argtypes = [ctypes.c_char_p, _i, _i, ctypes.c_ulong,
                                       ctypes.c_char_p, _i, _i, ctypes.c_ulong, ctypes.c_ulong,
                                       _i, _d, _i, _d, _d, _i, _vp, _vp, _i,
                                       _vp, _vp, _i, _vp, _vp, _i, _vp]

    def signal(self, seq, L):
        out = np.zeros(4 * L, np.float32)
        self.lib.ref_signal(seq, len(seq), L, _ptr(out))
        return out.reshape(4, L)

    def rc(self, seq):
        buf = ctypes.create_string_buffer(len(seq) + 1)
        self.lib.ref_rc(seq, len(seq), buf)
        return buf.raw[:len(seq)]

    def xcorr(self, t, q, L):
        out = np.zeros(L, np.float32)
        self.lib.ref_xcorr(t, len(t), q, len(q), L, _ptr(out))
        return out

    def findtop(self, xc, cutoff):
        xc = np.ascontiguousarray(xc, dtype=np.float32)
        out = np.zeros(len(xc), np.int32)
        n = self.lib.ref_findtop(_ptr(xc), len(xc), cutoff, _ptr(out), len(xc))
        return out[:n].copy()

    def doone(self, t, q, pos):
        cap = 1 << 14
        segs = np.zeros(3 * cap, np.int32)
        n = self.lib.ref_doone(t, len(t), q, len(q), pos, _ptr(segs), cap)
        return segs[:3 * n].reshape(n, 3).copy()

    def match_prob(self, t, q, ts, qs, length, target_total):
        ident = ctypes.c_double()
        p = self.lib.ref_match_prob(t, len(t), q, len(q), ts, qs, length, target_total,
                                    ctypes.byref(ident))
        return p, ident.value

    def print_ident(self, t, q, ts, qs, length):
        return self.lib.ref_print_ident(t, len(t), q, len(q), ts, qs, length)

    def probtable(self, target_size, cutoff):
        h = self.lib.ref_probtable_new(target_size, cutoff)
        tab = np.zeros(512 * 2048, np.float64)
        self.lib.ref_probtable_dump(h, _ptr(tab))
        return h, tab

    def align_pair(self, t, q, fft_len, cutoff=1.8, min_len=0, min_prob=0.99, target_total=4096.0,
                   query_chunk=4096, t_chunk_start=0, target_id=0, q_chunk_start=0, query_id=0,
                   query_size=None, probtable=None, want_detail=False):
        L = fft_len
        cap = 1 << 14
        res = np.zeros(cap, RESULT_DTYPE)
        scap = 1 << 16
        qsz = len(q) if query_size is None else query_size
        if want_detail:
            offs = np.zeros(2 * L, np.int32)
            noffs = np.zeros(2, np.int32)
            segs = np.zeros(2 * 3 * scap, np.int32)
            nsegs = np.zeros(2, np.int32)
            xco = np.zeros(2 * L, np.float32)
            extra = (_ptr(offs), _ptr(noffs), L, _ptr(segs), _ptr(nsegs), scap, _ptr(xco))
        else:   # records only: the reference path without stage copies
            extra = (None, None, 0, None, None, 0, None)
        n = self.lib.ref_align_pair(t, len(t), t_chunk_start, target_id, q, len(q), q_chunk_start,
                                    query_id, qsz, L, cutoff, min_len, min_prob, target_total,
                                    query_chunk, probtable, _ptr(res), cap, *extra)
        detail = None
        if want_detail:
            detail = {
                "offsets": [offs[s * L:s * L + noffs[s]].copy() for s in range(2)],
                "segments": [segs[s * 3 * scap:s * 3 * scap + 3 * nsegs[s]].reshape(-1, 3).copy()
                             for s in range(2)],
                "xc": xco.reshape(2, L).copy(),
            }
        return res[:n].copy(), detail
