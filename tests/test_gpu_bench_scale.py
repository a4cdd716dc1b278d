"""Parity at benchmark scale: the device batches the benchmark times, checked
whole against the oracle.

For each configuration the batch is uploaded and run as bench.py runs it
(xc_batch_run), and its records (xc_batch_results), FindTop offsets
(xc_batch_offsets) and near-threshold lags (xc_batch_straddles) are read back:

* offsets equal the FP64 oracle's (exact FindTop on the FP64 correlation)
  except "straddles", lags whose FP64 value lies within the band around the
  FP64 threshold; the number of such differences is bounded and every one of
  them is in the library's own near-threshold list;
* records equal the oracle's over the GPU's own offsets (coordinates, strands
  and identity bit-exact; prob to libm level);
* the correlation is within 1e-3 of FP64 (relative to the peak) on a sample.

Configurations: the 4096-pair uniform batch (seed 42, the benchmark's), 2000
pairs of the uneven-length batch (FFT 1024-8192), four 24x24 grid blocks of
the genome workload (2304 pairs with chunk coordinates, through the spectra
path) and 200 pairs of 16384 bp at FFT 32768.  With SATSUMA2_PARITY_REPORT=<path> the figures are written there
as JSON (profiles/parity_bench_configs.json is that file from a GB300 run)."""
import json
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle
from satsuma2_gb300 import workloads as W
from tests import parity

pytestmark = pytest.mark.gpu

XC_TOL = 1e-3
SEED = 42
_REPORT = {}


@pytest.fixture(scope="module")
def O():
    return oracle.Oracle()


def _check_batch(O, x, items, L_of, P, target_total, cutoff=1.8, n_xc_sample=48, upload=None, pair_of=None,
                 launches=None):
    """items: (t, q) byte pairs; upload: what to upload instead (a chunk-pair
    array of the same pairs); pair_of(k): oracle pair fields of pair k
    (chunk coordinates) besides t and q; launches: the batch's kernel count."""
    b = x.upload(items if upload is None else upload)
    if launches is not None:
        assert b.launches() == launches
    b.run()
    res, counts = b.results(with_counts=True)
    offs = b.offsets()
    near_cnt, near_lags = b.straddles()
    starts = np.concatenate([[0], np.cumsum(counts.astype(np.int64))])

    def one(k):
        t, q = items[k]
        L = L_of(t, q)
        rcq = O.rc(q)
        diff_n, not_listed = 0, 0
        for s, qq in enumerate((q, rcq)):
            xc64 = O.xcorr64(t, qq, L)
            thr = O.thresholds(xc64, cutoff)
            rel = parity.STRADDLE_REL_OSC if L > 16384 else parity.STRADDLE_REL
            band = rel * max(1.0, float(np.abs(xc64).max()))
            band_set = set(np.nonzero(np.abs(xc64 - thr) <= band)[0].tolist())
            diff = parity.compare_offsets(offs[k][s], np.nonzero(xc64 > thr)[0], band_set)
            diff_n += len(diff)
            if diff and near_cnt[k, s] <= near_lags.shape[2]:
                not_listed += len(diff - set(near_lags[k, s][:near_cnt[k, s]].tolist()))
        want, _ = O.align_pair(P(L), O.pair(t, q, **(pair_of(k) if pair_of else {})), offsets_in=offs[k])
        mine = res[starts[k]:starts[k + 1]]
        ok = parity.same_results(mine, want, target_total=target_total)
        return diff_n, not_listed, ok

    with ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        out = list(ex.map(one, range(len(items))))
    bad = [k for k, o in enumerate(out) if not o[2]]
    assert not bad, "records differ from the oracle at pairs %s" % bad[:10]
    n_diff = sum(o[0] for o in out)
    assert sum(o[1] for o in out) == 0, "an offset difference is missing from the near-threshold list"
    # the correlation itself, on a sample (debug output runs the same kernel)
    err = 0.0
    for k in range(0, len(items), max(1, len(items) // n_xc_sample)):
        t, q = items[k]
        d = x.debug_pair(t=t, q=q, signals=False)
        for s, qq in enumerate((q, O.rc(q))):
            xc64 = O.xcorr64(t, qq, d["L"])
            err = max(err, float(np.abs(d["xc"][s].astype(np.float64) - xc64).max())
                      / max(1.0, float(np.abs(xc64).max())))
    assert err <= XC_TOL, err
    b.free()
    return {"pairs": len(items), "records": int(len(res)), "offsets": int(sum(len(o[0]) + len(o[1]) for o in offs)),
            "offsets_differing_from_fp64": int(n_diff), "near_threshold_lags": int(near_cnt.sum()),
            "xc_err_max_vs_fp64": err, "xc_err_sampled_pairs": len(range(0, len(items), max(1, len(items) // n_xc_sample)))}


def _report(name, fig):
    _REPORT[name] = fig
    path = os.environ.get("SATSUMA2_PARITY_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(_REPORT, f, indent=1, sort_keys=True)


def test_uniform_4096_bench_batch_vs_oracle(O):
    import satsuma2_gb300 as sg
    items = W.uniform_batch(4096, seed=SEED)
    TT = 4096.0 * 4096
    x = sg.XCorr(target_total=TT)
    fig = _check_batch(O, x, items, lambda t, q: 8192, lambda L: O.params(target_total=TT), TT)
    x.close()
    # FP32 against FP64 parts only within ~1e-6 of the peak: a handful of lags
    assert fig["offsets_differing_from_fp64"] <= max(8, fig["pairs"] // 100), fig
    _report("uniform_4096x4096_fft8192", fig)


def test_uneven_2000_vs_oracle(O):
    import satsuma2_gb300 as sg
    items = W.uneven_batch(2000, seed=SEED)
    TT = float(sum(len(t) for t, _ in items))
    x = sg.XCorr(fft_len=-1, target_total=TT)
    fig = _check_batch(O, x, items, lambda t, q: W.uneven_fft_len(len(t), len(q)),
                       lambda L: O.params(target_total=TT, fft_len=L), TT)
    x.close()
    assert fig["offsets_differing_from_fp64"] <= max(8, fig["pairs"] // 100), fig
    _report("uneven_2000_fft1024_8192", fig)


def test_grid_blocks_vs_oracle(O):
    """Config 3: the first four 24x24 blocks of the genome workload in
    grid-search order, uploaded as chunk-pair arrays into the genome buffers
    (chunks shared within a block: the spectra path), records with their
    chunk coordinates and reverse-strand query positions."""
    import satsuma2_gb300 as sg
    t, q, (src, _) = W.serving_genomes(seed=SEED, with_map=True)
    tb, qb = np.frombuffer(t, np.uint8), np.frombuffer(q, np.uint8)
    tc = np.array(W.chunk_starts(len(t), 4096, 1024), np.int64)
    qc = np.array(W.chunk_starts(len(q), 4096, 0), np.int64)
    blocks = W.grid_search_blocks(src, len(tc), len(qc))[:4]
    arr = np.concatenate([sg.block_pairs(tb, tc, qb, qc, *blk) for blk in blocks])
    base_t, base_q = tb.ctypes.data, qb.ctypes.data
    items = [(t[a - base_t:a - base_t + lt], q[c - base_q:c - base_q + lq])
             for a, lt, c, lq in zip(arr["tseq"].tolist(), arr["tlen"].tolist(), arr["qseq"].tolist(),
                                     arr["qlen"].tolist())]

    def pair_of(k):
        return {"t_chunk_start": int(arr["t_chunk_start"][k]), "q_chunk_start": int(arr["q_chunk_start"][k]),
                "query_size": int(arr["query_size"][k])}

    TT = float(len(t))
    x = sg.XCorr(target_total=TT)
    # spectra kernel, correlation from spectra, hand-back, scan, two finalize kernels
    fig = _check_batch(O, x, items, lambda t, q: 8192, lambda L: O.params(target_total=TT), TT,
                       upload=arr, pair_of=pair_of, launches=6)
    x.close()
    assert fig["offsets_differing_from_fp64"] <= max(8, fig["pairs"] // 100), fig
    _report("grid_blocks_4x576_fft8192_spectra", fig)


def test_large_200_fft32768_vs_oracle(O):
    import satsuma2_gb300 as sg
    items = W.large_batch(200, seed=SEED)
    TT = 16384.0 * 200
    x = sg.XCorr(t_chunk=16384, q_chunk=16384, target_total=TT)
    fig = _check_batch(O, x, items, lambda t, q: 32768,
                       lambda L: O.params(target_total=TT, fft_len=32768, q_chunk=16384), TT, n_xc_sample=24)
    x.close()
    assert fig["offsets_differing_from_fp64"] <= max(8, fig["pairs"] // 10), fig
    _report("large_200_16384bp_fft32768", fig)
