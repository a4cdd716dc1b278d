"""CPU tests: the oracle (oracle/xcorr_oracle.c) against the golden vectors the
reference produced (tests/golden/), and against the reference library itself
when it is present in this container."""
import hashlib
import os

import numpy as np
import pytest

import oracle
from tests import parity
from satsuma2_gb300 import workloads as W

CASES = parity.load_cases()


@pytest.fixture(scope="module")
def O():
    return oracle.Oracle()


def sha1(a):
    return hashlib.sha1(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_min_matches(O):
    # (int)(45 * 0.42 * 100) in double (CrossCorr.cc:675)
    assert O.lib.orc_min_matches() == 1889


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_signals_bit_exact(O, case):
    rcq = O.rc(case["q"])
    for k, s in enumerate((case["t"], case["q"], rcq)):
        sig = O.signal(s, case["L"])
        assert [sha1(sig[c]) for c in range(4)] == case["signal_sha1"][k]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_offsets_within_straddle(O, case):
    rcq = O.rc(case["q"])
    for s, qq in enumerate((case["q"], rcq)):
        band, xc64 = parity.straddles(O, case, qq, s)
        got = O.findtop(xc64, case["cutoff"])
        parity.compare_offsets(got, case["ref_offsets"][s], band)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_segments_exact(O, case):
    rcq = O.rc(case["q"])
    L = case["L"]
    for s, qq in enumerate((case["q"], rcq)):
        segs = [O.doone(case["t"], qq, int(i) - L // 2) for i in case["ref_offsets"][s]]
        got = np.concatenate(segs) if segs else np.zeros((0, 3), np.int32)
        assert np.array_equal(got.reshape(-1, 3), case["ref_segments"][s].reshape(-1, 3))


_TABLES = {}


def _params(O, case):
    pt = None
    if case["probtable"]:
        key = (case["target_total"], case["probtable_cutoff"])
        if key not in _TABLES:
            _TABLES[key] = O.probtable(*key)
        pt = _TABLES[key]
        sha = hashlib.sha1(pt.tobytes()).hexdigest()
        assert sha is not None
    return O.params(cutoff=case["cutoff"], min_prob=case["min_prob"], target_total=case["target_total"],
                    min_len=case["min_len"], q_chunk=case["query_chunk"], fft_len=case["L"],
                    probtable=pt, probtable_cutoff=case["probtable_cutoff"])


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_results_exact_given_offsets(O, case):
    P = _params(O, case)
    pr = O.pair(case["t"], case["q"], t_chunk_start=case["t_chunk_start"], target_id=case["target_id"],
                q_chunk_start=case["q_chunk_start"], query_id=case["query_id"],
                query_size=case["query_size"])
    res, _ = O.align_pair(P, pr, offsets_in=case["ref_offsets"])
    assert parity.same_results(res, case["ref_results"], prob_rtol=1e-12)


def test_probtable_matches_reference_table(O):
    z = np.load(os.path.join(parity.GOLDEN, "cases.npz"))
    for c in CASES:
        if c["probtable"]:
            key = "probtable_sha1_%d" % c["index"]
            tab = _TABLES.get((c["target_total"], c["probtable_cutoff"]))
            if tab is None:
                tab = O.probtable(c["target_total"], c["probtable_cutoff"])
            # Row 0 is never filled by the reference (dumped as -1): same here.
            assert hashlib.sha1(tab.tobytes()).hexdigest() == str(z[key])


def test_slave_end_to_end(O):
    """The oracle reproduces the unmodified reference slave's t_result stream."""
    d = parity.load_slave_e2e()
    m = d["meta"]
    tseqs = [d["tg0"].tobytes(), d["tg1"].tobytes(), d["sentinel"].tobytes()]
    qseqs = [d["qg0"].tobytes(), d["qg1"].tobytes(), d["qg2"].tobytes(), d["sentinel"].tobytes()]
    P = O.params(cutoff=m["cutoff"], min_prob=m["min_prob_effective"], target_total=m["target_total"],
                 t_chunk=m["t_chunk"], q_chunk=m["q_chunk"])
    out = []
    for (tf, tt, qf, qt) in d["blocks"][:-1]:
        for qi in range(qf, qt + 1):
            for ti in range(tf, tt + 1):
                ts, tst, ten = d["tchunks"][ti]
                qs, qst, qen = d["qchunks"][qi]
                pr = O.pair(tseqs[ts][tst:ten], qseqs[qs][qst:qen], t_chunk_start=int(tst), target_id=int(ts),
                            q_chunk_start=int(qst), query_id=int(qs), query_size=len(qseqs[qs]))
                res, _ = O.align_pair(P, pr)
                out.append(res)
    got = np.concatenate(out)
    assert parity.same_results(got, d["results"], prob_rtol=1e-12)


def test_slave_end_to_end_probtable(O):
    """The oracle reproduces the reference slave's -prob_table stream."""
    d = parity.load_slave_e2e_probtable()
    m = d["meta"]
    pt = O.probtable(m["target_total"], m["prob_table_cutoff"])
    P = O.params(cutoff=m["cutoff"], min_prob=m["min_prob_effective"], target_total=m["target_total"],
                 t_chunk=m["t_chunk"], q_chunk=m["q_chunk"], probtable=pt,
                 probtable_cutoff=m["prob_table_cutoff"])
    out = []
    for it in parity.slave_items(d):
        pr = O.pair(it["t"], it["q"], t_chunk_start=it["t_chunk_start"], target_id=it["target_id"],
                    q_chunk_start=it["q_chunk_start"], query_id=it["query_id"], query_size=it["query_size"])
        res, _ = O.align_pair(P, pr)
        out.append(res)
    got = np.concatenate(out)
    assert len(got) > 50000
    assert parity.same_results(got, d["results"], prob_rtol=0.0)


def test_workloads_deterministic():
    a = W.uniform_batch(4, seed=3)
    b = W.uniform_batch(4, seed=3)
    assert a == b
    assert all(len(t) == 4096 and len(q) == 4096 for t, q in a)
    u = W.uneven_batch(50, seed=1)
    assert all(300 <= len(t) <= 4096 and 300 <= len(q) <= 4096 for t, q in u)
    assert {W.uneven_fft_len(len(t), len(q)) for t, q in u} <= {1024, 2048, 4096, 8192}
    t, q = W.plain_pair(42)
    assert len(t) == len(q) == 4096
    assert W.chunk_starts(6144, 4096, 1024)[-1] == (6144, 6144)   # empty last chunk


@pytest.mark.skipif(not os.path.exists(oracle.REF_SO), reason="reference library not built here")
def test_oracle_vs_reference_random(O):
    R = oracle.Reference()
    rng = np.random.default_rng(123)
    for trial in range(6):
        L = [2048, 4096, 8192][trial % 3]
        tl = int(rng.integers(1, L // 2 + 1))
        ql = int(rng.integers(1, L // 2 + 1))
        letters = np.frombuffer(b"ACGTACGTACGTNKRYB-", np.uint8)
        t = letters[rng.integers(0, len(letters), tl)].tobytes()
        q = letters[rng.integers(0, len(letters), ql)].tobytes()
        for s in (t, q, O.rc(q)):
            assert np.array_equal(O.signal(s, L).view(np.uint32), R.signal(s, L).view(np.uint32))
        rr, rd = R.align_pair(t, q, L, want_detail=True)
        P = O.params(fft_len=L)
        ro, _ = O.align_pair(P, O.pair(t, q), offsets_in=rd["offsets"])
        assert parity.same_results(ro, rr, prob_rtol=0.0)
