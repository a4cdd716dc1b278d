"""Parity helpers shared by the tests: golden fixture access and the match-set
comparison contract.

Contract (per chunk pair and strand):
* FindTop offsets equal the reference's except "straddles": indices whose FP64
  correlation lies within ``band`` of the FP64 threshold (there the FP32
  rounding of either implementation decides);
* DoOne segments and t_result records that come from offsets both sides kept
  are identical; the probability may differ by a few ulp (GPU erf/exp vs
  glibc), everything else is bit-exact.
"""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STRADDLE_REL = 2e-5      # band = STRADDLE_REL * max|xc| (FP32 errors measured ~2e-7)
# At FFT 32768 FFTReal switches to its float rotation oscillator for the passes
# beyond 12 (FFTReal.h:78): the reference's own FP32 error grows to ~1.5e-4 of
# the peak (~0.08 absolute near the FindTop threshold), so the band widens there.
STRADDLE_REL_OSC = 3e-4
PROB_RTOL = 1e-12


def load_cases():
    z = np.load(os.path.join(GOLDEN, "cases.npz"), allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    out = []
    for m in meta:
        k = m["index"]
        p = "c%d_" % k
        c = dict(m)
        c["t"] = z[p + "t"].tobytes()
        c["q"] = z[p + "q"].tobytes()
        c["ref_offsets"] = [z[p + "off0"], z[p + "off1"]]
        c["ref_segments"] = [z[p + "seg0"], z[p + "seg1"]]
        c["ref_results"] = z[p + "res"]
        out.append(c)
    return out


def load_slave_e2e():
    z = np.load(os.path.join(GOLDEN, "slave_e2e.npz"), allow_pickle=False)
    d = {k: z[k] for k in z.files}
    d["meta"] = json.loads(str(z["meta"]))
    return d


def load_slave_e2e_probtable():
    """The reference slave's records with -prob_table over the first
    meta["n_blocks"] blocks of slave_e2e.npz (sequences and blocks from there)."""
    d = load_slave_e2e()
    z = np.load(os.path.join(GOLDEN, "slave_e2e_probtable.npz"), allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    d["results"] = z["results"]
    d["meta"] = meta
    d["blocks"] = np.concatenate([d["blocks"][:meta["n_blocks"]], d["blocks"][-1:]])
    return d


def slave_items(d):
    """The chunk pairs of the golden run's real blocks, block by block
    (query-major, target-minor, as align_target loops)."""
    tseqs = [d["tg0"].tobytes(), d["tg1"].tobytes(), d["sentinel"].tobytes()]
    qseqs = [d["qg0"].tobytes(), d["qg1"].tobytes(), d["qg2"].tobytes(), d["sentinel"].tobytes()]
    items = []
    for (tf, tt, qf, qt) in d["blocks"][:-1]:
        for qi in range(qf, qt + 1):
            for ti in range(tf, tt + 1):
                ts, tst, ten = d["tchunks"][ti]
                qs, qst, qen = d["qchunks"][qi]
                items.append(dict(t=tseqs[ts][tst:ten], q=qseqs[qs][qst:qen], t_chunk_start=int(tst),
                                  target_id=int(ts), q_chunk_start=int(qst), query_id=int(qs),
                                  query_size=len(qseqs[qs])))
    return items


def result_offsets(res, case):
    """(strand, FindTop index) of each t_result record of one chunk pair."""
    L = case["L"]
    out = []
    for r in res:
        ts = int(np.int64(r["tstart"])) - case["t_chunk_start"]
        qs = int(np.int64(r["qstart"]))
        if r["reverse"]:
            qs = qs - case["query_size"] + case["q_chunk_start"] + case["query_chunk"]
        else:
            qs = qs - case["q_chunk_start"]
        out.append((int(r["reverse"]), qs - ts + L // 2))
    return out


def straddles(O, case, strand_q, strand):
    """Set of offset indices within the straddle band of the FP64 threshold."""
    xc64 = O.xcorr64(case["t"], strand_q, case["L"])
    cutoff = case["cutoff"]
    thr = O.thresholds(xc64, cutoff)
    rel = STRADDLE_REL_OSC if case["L"] > 16384 else STRADDLE_REL
    band = rel * max(1.0, float(np.abs(xc64).max()))
    return set(np.nonzero(np.abs(xc64 - thr) <= band)[0].tolist()), xc64


def compare_offsets(got, ref, band_set):
    """Returns the symmetric difference, asserting it lies in band_set."""
    diff = set(np.asarray(got).tolist()) ^ set(np.asarray(ref).tolist())
    bad = diff - band_set
    assert not bad, "offsets differ outside the straddle band: %s" % sorted(bad)[:20]
    return diff


def prob_tolerance(target_total):
    """Absolute prob tolerance between two libms.

    The reference forms cdf = 0.5*(1 + erf(z)) with z far below zero, so
    1 + erf(z) = 2*expect/targetTotal is tiny and one ulp of erf (2^-52 near
    -1) becomes a relative error of ulp*targetTotal/(2*expect) in expect, i.e.
    an absolute error of about ulp*targetTotal/2 in expect and in prob =
    exp(-expect).  Allow 16 such ulps."""
    return 16.0 * 2.0 ** -52 * max(1.0, float(target_total))


def same_results(a, b, prob_rtol=PROB_RTOL, target_total=1.0):
    """Exact equality of t_result arrays except libm-level prob differences."""
    if len(a) != len(b):
        return False
    for f in ("query_id", "target_id", "query_size", "qstart", "tstart", "len", "reverse"):
        if not np.array_equal(a[f], b[f]):
            return False
    if not np.array_equal(a["ident"].view(np.uint64), b["ident"].view(np.uint64)):
        return False
    pa, pb = a["prob"], b["prob"]
    both_nan = np.isnan(pa) & np.isnan(pb)
    tol = np.maximum(prob_rtol * np.maximum(np.abs(pa), np.abs(pb)), prob_tolerance(target_total))
    ok = both_nan | (np.abs(pa - pb) <= tol)
    return bool(np.all(ok))


def drop_offsets(res, case, dropped):
    """Results whose (strand, offset) is not in dropped."""
    keep = [i for i, so in enumerate(result_offsets(res, case)) if so not in dropped]
    return res[keep]
