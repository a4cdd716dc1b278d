"""xc_align_pair_noalloc, the entry point for callers that cannot call
cudaMalloc: processes whose device memory belongs to another allocator (a
framework's caching allocator or a fixed arena holding the free HBM), and
latency-bound callers sharing the GPU, for whom cudaFree's device-wide
synchronisation is not acceptable.  It keeps the chunks and the kernels'
scratch in one static device array instead of allocating.

Checked through the C ABI against xc_align_pairs on the same pairs, two calls
in a row per pair (each call reuses the array the previous one left behind),
with the result tolerance the other GPU tests use.  This file sorts last so
that a run stopping at its first failure has run every other test first."""
import ctypes

import numpy as np
import pytest

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
    return items


def test_noalloc_matches_align_pairs_twice_in_a_row():
    x = sg.XCorr(target_total=TT)
    try:
        nonempty = 0
        for item in pairs():
            want = x.align([item])
            for call in range(2):
                r, got, n = noalloc(x, item)
                assert r == sg.XC_OK, (call, r)
                assert n == len(want)
                assert parity.same_results(got, want, target_total=TT), call
            nonempty += len(want) > 0
        assert nonempty >= 3
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
