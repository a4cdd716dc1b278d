"""xc_align_pair_noalloc, the entry point for callers that cannot call
cudaMalloc: processes whose device memory belongs to another allocator (a
framework's caching allocator or a fixed arena holding the free HBM), and
latency-bound callers sharing the GPU, for whom cudaFree's device-wide
synchronisation is not acceptable.  It keeps the chunks and the kernels'
scratch in one static device array instead of allocating.

Checked through the C ABI against xc_align_pairs on the same pairs, two calls
in a row per pair (each call reuses the array the previous one left behind),
with the result tolerance the other GPU tests use, and against the oracle over
the FindTop offsets its kernels keep; at FFT 8192 and at the 16384 maximum,
and past the 1024-matches-per-strand limit.  This file sorts last so that a
run stopping at its first failure has run every other test first."""
import ctypes

import numpy as np
import pytest

import oracle
import satsuma2_gb300 as sg
from satsuma2_gb300 import workloads as W
from tests import parity

pytestmark = pytest.mark.gpu

TT = 4096.0 * 4096


def noalloc(x, item, cap=4096):
    """One call of xc_align_pair_noalloc -> (status, t_result records, n_out)."""
    arr, keep = sg.make_pairs([item])
    out = np.zeros(cap, sg.RESULT_DTYPE)
    n_out = ctypes.c_size_t()
    r = x.lib.xc_align_pair_noalloc(x.ctx, arr, out.ctypes.data, cap, ctypes.byref(n_out))
    return r, out[:n_out.value].copy() if r == sg.XC_OK else None, n_out.value


def pairs():
    rng = np.random.default_rng(31)
    t = W.random_bases(rng, 4096)
    items = [W.plain_pair(7)]
    items += [dict(t=a, q=b, t_chunk_start=8192, target_id=3, q_chunk_start=4096, query_id=5,
                   query_size=20000) for a, b in W.uniform_batch(3, seed=12)]
    items.append((t.tobytes(), W.revcomp(t).tobytes()))            # reverse-strand homology
    g = bytearray(W.plain_pair(8)[0])
    g[100:140] = b"N" * 40                                          # byte-table path
    items.append((bytes(g), W.plain_pair(8)[1]))
    items.append((W.random_bases(rng, 1500).tobytes(), W.random_bases(rng, 900).tobytes()))  # short
    # a 3001-base query (not a multiple of the 16-base window): the ragged-query kernel
    items.append((t.tobytes(), W.mutate(rng, t[500:3501], 0.9, indel_every=0).tobytes()))
    return items


def _as_dict(item):
    return item if isinstance(item, dict) else dict(t=item[0], q=item[1])


def _oracle_records(O, x, item, fft_len=0, q_chunk=4096):
    """The oracle's records over the offsets the library's kernels keep."""
    it = _as_dict(item)
    extra = {k: v for k, v in it.items() if k not in ("t", "q")}
    d = x.debug_pair(t=it["t"], q=it["q"], signals=False, **extra)
    P = O.params(target_total=TT, fft_len=fft_len, q_chunk=q_chunk)
    pr = O.pair(it["t"], it["q"], t_chunk_start=it.get("t_chunk_start", 0), target_id=it.get("target_id", 0),
                q_chunk_start=it.get("q_chunk_start", 0), query_id=it.get("query_id", 0),
                query_size=it.get("query_size"))
    want, _ = O.align_pair(P, pr, offsets_in=d["offsets"])
    return want


def test_noalloc_matches_align_pairs_twice_in_a_row():
    O = oracle.Oracle()
    x = sg.XCorr(target_total=TT)
    try:
        nonempty = 0
        for item in pairs():
            want = x.align([item])
            assert parity.same_results(_oracle_records(O, x, item), want, target_total=TT)
            for call in range(2):
                r, got, n = noalloc(x, item)
                assert r == sg.XC_OK, (call, r)
                assert n == len(want)
                assert parity.same_results(got, want, target_total=TT), call
            nonempty += len(want) > 0
        assert nonempty >= 3
    finally:
        x.close()


def test_noalloc_at_fft_16384():
    """The largest FFT length the static array holds: 8192-bp chunks."""
    O = oracle.Oracle()
    x = sg.XCorr(target_total=TT, t_chunk=8192, q_chunk=8192)
    try:
        rng = np.random.default_rng(77)
        t = W.random_bases(rng, 8192)
        core = W.mutate(rng, t[1000:7000], 0.85)
        q = np.concatenate([W.random_bases(rng, 1000), core, W.random_bases(rng, 8192 - 1000 - len(core))])[:8192]
        items = [(t.tobytes(), q.tobytes()), (t.tobytes(), W.revcomp(q).tobytes())]
        for item in items:
            want = x.align([item])
            assert len(want) > 0
            assert parity.same_results(_oracle_records(O, x, item, fft_len=16384, q_chunk=8192), want, target_total=TT)
            for call in range(2):
                r, got, n = noalloc(x, item)
                assert r == sg.XC_OK, (call, r)
                assert parity.same_results(got, want, target_total=TT), call
    finally:
        x.close()


def test_noalloc_reports_matches_beyond_its_slots():
    """min_prob 0 keeps every DoOne segment (thousands per pair): past 1024
    kept matches on a strand the call answers XC_ERR_CAPACITY with the number
    of matches found, and the next call in the array is clean."""
    x = sg.XCorr(target_total=TT, min_prob=0.0)
    try:
        item = W.plain_pair(7)
        want = x.align([item])
        assert (want["reverse"] == 0).sum() > 1024
        r, _, n = noalloc(x, item, cap=1 << 16)
        assert r == -4 and n == len(want)
        small = (W.random_bases(np.random.default_rng(3), 1500).tobytes(),
                 W.random_bases(np.random.default_rng(4), 900).tobytes())
        want2 = x.align([small])
        r, got, _ = noalloc(x, small)
        assert r == sg.XC_OK and parity.same_results(got, want2, target_total=TT)
    finally:
        x.close()


def test_noalloc_rejects_sizes_beyond_its_limits():
    x = sg.XCorr(target_total=TT)
    try:
        item = W.plain_pair(7)
        want = x.align([item])
        assert len(want) > 1
        r, _, n = noalloc(x, item, cap=1)                     # output too small
        assert r == -4 and n == len(want)
        r, got, _ = noalloc(x, item)                          # and the next call is clean
        assert r == sg.XC_OK and parity.same_results(got, want, target_total=TT)
    finally:
        x.close()
    x = sg.XCorr(target_total=TT, fft_len=32768)              # beyond the 16384 maximum
    try:
        r, _, _ = noalloc(x, W.plain_pair(7))
        assert r == -7
    finally:
        x.close()
