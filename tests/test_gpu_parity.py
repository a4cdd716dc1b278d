"""GPU parity tests: the CUDA path through the C ABI against the reference's
golden vectors (tests/golden/) and the oracle, on the same seeded inputs.

Bars (see tests/parity.py): signals bit-exact; correlation within 1e-3 of the
FP64 oracle (relative to its peak); FindTop offsets equal except straddles;
DoOne segments exact; t_result records exact except ulp-level prob."""
import hashlib
import threading

import numpy as np
import pytest

import oracle
from tests import parity
from satsuma2_gb300 import workloads as W

pytestmark = pytest.mark.gpu

CASES = parity.load_cases()
XC_TOL = 1e-3


@pytest.fixture(scope="module")
def O():
    return oracle.Oracle()


_CTX = {}


def ctx_for(case):
    import satsuma2_gb300 as sg
    from satsuma2_gb300 import build
    key = (case["cutoff"], case["min_prob"], case["target_total"], case["min_len"], case["query_chunk"],
           case["L"], case["probtable"], case["probtable_cutoff"])
    if key not in _CTX:
        build.build()
        _CTX[key] = sg.XCorr(cutoff=case["cutoff"], min_prob=case["min_prob"], target_total=case["target_total"],
                             min_len=case["min_len"], q_chunk=case["query_chunk"], fft_len=case["L"],
                             prob_table=bool(case["probtable"]), prob_table_cutoff=case["probtable_cutoff"])
    return _CTX[key]


def pair_item(case):
    return dict(t=case["t"], q=case["q"], t_chunk_start=case["t_chunk_start"], target_id=case["target_id"],
                q_chunk_start=case["q_chunk_start"], query_id=case["query_id"], query_size=case["query_size"])


SUPPORTED = CASES


def sha1(a):
    return hashlib.sha1(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("case", SUPPORTED, ids=[c["name"] for c in SUPPORTED])
def test_stages_match_reference(O, case):
    x = ctx_for(case)
    d = x.debug_pair(**pair_item(case))
    L = case["L"]
    assert d["L"] == L
    rcq = O.rc(case["q"])
    # signals: strand 0 holds target + query, strand 1 target + RC query
    assert [sha1(d["signals"][0, 0, c]) for c in range(4)] == case["signal_sha1"][0]
    assert [sha1(d["signals"][0, 1, c]) for c in range(4)] == case["signal_sha1"][1]
    assert [sha1(d["signals"][1, 1, c]) for c in range(4)] == case["signal_sha1"][2]
    # correlation, offsets and segments from both correlation kernels: with
    # signal output one CTA per strand, without it (A/C/G/T pairs at FFT 8192)
    # the both-strands kernel that xc_align_pairs runs
    for dd in (d, x.debug_pair(signals=False, **pair_item(case))):
        for s, qq in enumerate((case["q"], rcq)):
            band, xc64 = parity.straddles(O, case, qq, s)
            scale = max(1.0, float(np.abs(xc64).max()))
            err = float(np.abs(dd["xc"][s].astype(np.float64) - xc64).max()) / scale
            assert err <= XC_TOL, err
            parity.compare_offsets(dd["offsets"][s], case["ref_offsets"][s], band)
            # DoOne segments over the GPU's own offsets: exact
            want = [O.doone(case["t"], qq, int(i) - L // 2) for i in dd["offsets"][s]]
            want = np.concatenate(want) if want else np.zeros((0, 3), np.int32)
            assert np.array_equal(dd["segments"][s].reshape(-1, 3), want.reshape(-1, 3))


@pytest.mark.parametrize("case", SUPPORTED, ids=[c["name"] for c in SUPPORTED])
def test_results_match_reference(O, case):
    x = ctx_for(case)
    res = x.align([pair_item(case)])
    d = x.debug_pair(signals=False, **pair_item(case))   # the kernel align ran
    rcq = O.rc(case["q"])
    dropped = set()
    for s, qq in enumerate((case["q"], rcq)):
        band, _ = parity.straddles(O, case, qq, s)
        for i in parity.compare_offsets(d["offsets"][s], case["ref_offsets"][s], band):
            dropped.add((s, i))
    ref = case["ref_results"]
    assert parity.same_results(parity.drop_offsets(res, case, dropped), parity.drop_offsets(ref, case, dropped),
                               target_total=case["target_total"])
    # and exactly the oracle's records over the GPU's own offsets
    pt = None
    if case["probtable"]:
        pt = O.probtable(case["target_total"], case["probtable_cutoff"])
    P = O.params(cutoff=case["cutoff"], min_prob=case["min_prob"], target_total=case["target_total"],
                 min_len=case["min_len"], q_chunk=case["query_chunk"], fft_len=case["L"], probtable=pt,
                 probtable_cutoff=case["probtable_cutoff"])
    pr = O.pair(case["t"], case["q"], t_chunk_start=case["t_chunk_start"], target_id=case["target_id"],
                q_chunk_start=case["q_chunk_start"], query_id=case["query_id"], query_size=case["query_size"])
    want, _ = O.align_pair(P, pr, offsets_in=d["offsets"])
    assert parity.same_results(res, want, target_total=case["target_total"])


def test_fft_beyond_32768_unsupported():
    import satsuma2_gb300 as sg
    x = sg.XCorr(fft_len=65536, target_total=4096.0)
    with pytest.raises(sg.XCError) as e:
        x.align([W.plain_pair(3)])
    assert e.value.code == -7
    x.close()


def test_fft32768_batch_vs_oracle(O):
    """Config-4-shaped pairs (16384 bp, microsatellites, skewed GC) at FFT
    32768, several in one launch: records equal the oracle's over the GPU's
    own offsets, and the offsets equal the FP64 oracle's except straddles."""
    import satsuma2_gb300 as sg
    items = W.large_batch(6, seed=11)
    TT = 16384.0 * 6
    x = sg.XCorr(fft_len=32768, t_chunk=16384, q_chunk=16384, target_total=TT)
    res, counts = x.align(items, with_counts=True)
    P = O.params(target_total=TT, fft_len=32768, q_chunk=16384)
    o = 0
    for k, (t, q) in enumerate(items):
        got = res[o:o + int(counts[k])]
        o += int(counts[k])
        d = x.debug_pair(t=t, q=q, signals=False)
        case = dict(t=t, L=32768, cutoff=1.8)
        for s, qq in enumerate((q, O.rc(q))):
            band, xc64 = parity.straddles(O, case, qq, s)
            err = float(np.abs(d["xc"][s].astype(np.float64) - xc64).max()) / max(1.0, float(np.abs(xc64).max()))
            assert err <= XC_TOL, err
            thr = O.thresholds(xc64, 1.8)
            parity.compare_offsets(d["offsets"][s], np.nonzero(xc64 > thr)[0], band)
        want, _ = O.align_pair(P, O.pair(t, q), offsets_in=d["offsets"])
        assert parity.same_results(got, want, target_total=TT)
    x.close()


def test_rejects_non_ascii():
    import satsuma2_gb300 as sg
    x = ctx_for(CASES[0])
    t = bytearray(b"ACGT" * 500)
    t[100] = 0xC3
    with pytest.raises(sg.XCError) as e:
        x.align([(bytes(t), b"ACGT" * 300)])
    assert e.value.code == -5
    # a query of 1201 bases (not a multiple of the 16-base window) goes to the
    # ragged-query kernel, which finds the byte itself; alone, and beside
    # pairs that stay valid
    q = bytearray(b"ACGT" * 300 + b"A")
    q[1190] = 0xC3
    ok = (b"ACGT" * 500, b"ACGT" * 300 + b"C")
    for items in ([(b"ACGT" * 500, bytes(q))], [ok, (b"ACGT" * 500, bytes(q)), ok]):
        with pytest.raises(sg.XCError) as e:
            x.align(items)
        assert e.value.code == -5
    assert len(x.align([ok, ok])) >= 0


def test_batch_equals_single_pairs(O):
    """Many pairs in one launch (bucketed by FFT length) = one pair per call."""
    import satsuma2_gb300 as sg
    x = sg.XCorr(fft_len=-1, target_total=4096.0 * 64)
    items = W.uneven_batch(48, seed=9) + W.uniform_batch(16, seed=21)
    res, counts = x.align(items, with_counts=True)
    o = 0
    for k, it in enumerate(items):
        single = x.align([it])
        got = res[o:o + int(counts[k])]
        o += int(counts[k])
        assert parity.same_results(got, single)
    x.close()


def test_split_scan_small_batch_vs_oracle(O):
    """Batches smaller than a wave split each strand's scan over several CTAs
    that each order the strand's diagonals by length themselves.  With the
    envelope off (FFT 2048) a pair keeps hundreds of offsets, many per length
    bucket, so the CTAs must agree on that order exactly: every pair's records
    equal the oracle's over the GPU's offsets, on three runs of the batch."""
    import satsuma2_gb300 as sg
    items = [it for it in W.uneven_batch(1600, seed=23) if W.uneven_fft_len(len(it[0]), len(it[1])) == 2048][:40]
    assert len(items) >= 20
    TT = float(sum(len(t) for t, _ in items))
    x = sg.XCorr(fft_len=-1, target_total=TT)
    P = O.params(target_total=TT, fft_len=2048)
    b = x.upload(items)
    want = None
    for run in range(3):
        b.run()
        res, counts = b.results(with_counts=True)
        if want is None:
            offs = b.offsets()
            o = 0
            for k, (t, q) in enumerate(items):
                got = res[o:o + int(counts[k])]
                o += int(counts[k])
                ref, _ = O.align_pair(P, O.pair(t, q), offsets_in=offs[k])
                assert parity.same_results(got, ref, target_total=TT), k
            want = res
        else:
            assert parity.same_results(res, want, target_total=TT), run
    b.free()
    x.close()


def test_uniform_batch_vs_oracle(O):
    import satsuma2_gb300 as sg
    items = W.uniform_batch(32, seed=5)
    x = sg.XCorr(target_total=4096.0 * 4096)
    res, counts = x.align(items, with_counts=True)
    P = O.params(target_total=4096.0 * 4096)
    o = 0
    for k, (t, q) in enumerate(items):
        got = res[o:o + int(counts[k])]
        o += int(counts[k])
        d = x.debug_pair(t=t, q=q, signals=False)
        want, _ = O.align_pair(P, O.pair(t, q), offsets_in=d["offsets"])
        assert parity.same_results(got, want, target_total=4096.0 * 4096)
    x.close()


def test_device_batch_replay_is_stable():
    import satsuma2_gb300 as sg
    items = W.uniform_batch(64, seed=33)
    x = sg.XCorr(target_total=4096.0 * 4096)
    ref = x.align(items)
    b = x.upload(items)
    assert b.launches() >= 4
    for _ in range(3):
        b.run()
        assert parity.same_results(b.results(), ref)
    b.free()
    x.close()


def _slave_stream_check(O, d, prob_table):
    """The CUDA path reproduces the unmodified reference slave's output stream.

    The oracle reproduces that stream exactly on the CPU (test_oracle), so it
    splits the stream per chunk pair; records from offsets where the GPU's
    FP32 FindTop and the FP64 oracle disagree inside the straddle band are set
    aside on both sides.  Returns the number of (strand, offset) set aside."""
    import satsuma2_gb300 as sg
    m = d["meta"]
    pt = O.probtable(m["target_total"], m["prob_table_cutoff"]) if prob_table else None
    x = sg.XCorr(cutoff=m["cutoff"], min_prob=m["min_prob_effective"], target_total=m["target_total"],
                 t_chunk=m["t_chunk"], q_chunk=m["q_chunk"], prob_table=prob_table,
                 prob_table_cutoff=m.get("prob_table_cutoff", 0.9999))
    P = O.params(cutoff=m["cutoff"], min_prob=m["min_prob_effective"], target_total=m["target_total"],
                 t_chunk=m["t_chunk"], q_chunk=m["q_chunk"], probtable=pt,
                 probtable_cutoff=m.get("prob_table_cutoff", 0.0))
    items = parity.slave_items(d)
    got, counts = x.align(items, with_counts=True)
    slave = d["results"]
    og = os_ = 0
    n_dropped = 0
    for k, it in enumerate(items):
        pr = O.pair(it["t"], it["q"], t_chunk_start=it["t_chunk_start"], target_id=it["target_id"],
                    q_chunk_start=it["q_chunk_start"], query_id=it["query_id"], query_size=it["query_size"])
        want, det = O.align_pair(P, pr, want_detail=True)
        mine = got[og:og + int(counts[k])]
        theirs = slave[os_:os_ + len(want)]
        og += int(counts[k])
        os_ += len(want)
        assert parity.same_results(theirs, want, target_total=m["target_total"]), "oracle no longer splits the slave stream at pair %d" % k
        case = dict(L=8192, t_chunk_start=it["t_chunk_start"], q_chunk_start=it["q_chunk_start"],
                    query_size=it["query_size"], query_chunk=m["q_chunk"], cutoff=m["cutoff"], t=it["t"])
        dbg = x.debug_pair(signals=False, **it)
        dropped = set()
        for s, qq in enumerate((it["q"], O.rc(it["q"]))):
            band, _ = parity.straddles(O, case, qq, s)
            for i in parity.compare_offsets(dbg["offsets"][s], det["offsets"][s], band):
                dropped.add((s, i))
        n_dropped += len(dropped)
        a = parity.drop_offsets(mine, case, dropped)
        b = parity.drop_offsets(theirs, case, dropped)
        assert parity.same_results(a, b, target_total=m["target_total"]), "pair %d:\nGPU %s\nslave %s" % (
            k, a[["qstart", "tstart", "len", "reverse", "prob", "ident"]],
            b[["qstart", "tstart", "len", "reverse", "prob", "ident"]])
    assert og == len(got) and os_ == len(slave)
    x.close()
    return n_dropped, len(items)


def test_slave_end_to_end(O):
    n_dropped, n_pairs = _slave_stream_check(O, parity.load_slave_e2e(), prob_table=False)
    assert n_dropped <= max(2, n_pairs // 10)   # straddling offsets are rare


def test_slave_end_to_end_probtable(O):
    """-prob_table: thousands of records per pair (a small targetTotal makes
    most DoOne segments pass the table), far past the result slots."""
    n_dropped, n_pairs = _slave_stream_check(O, parity.load_slave_e2e_probtable(), prob_table=True)
    assert n_dropped <= max(2, n_pairs // 10)


def _block_items(tchunks, qchunks, tf, qf, n=24):
    """One n x n grid block of chunk pairs, query-major as align_target loops."""
    return [dict(t=tchunks[ti], q=qchunks[qi], t_chunk_start=3072 * ti, target_id=0,
                 q_chunk_start=4096 * qi, query_id=0, query_size=4096 * len(qchunks))
            for qi in range(qf, qf + n) for ti in range(tf, tf + n)]


def test_spectra_path_matches_pair_kernel(O, monkeypatch):
    """Grid blocks of chunk pairs share their chunks: the spectra path
    (spec_kernel once per distinct chunk, then the pair kernel from stored
    spectra) and the both-strands kernel form each pair's sums by different
    FP32 operations (the four channels as two packed pairs, against the
    basis A - T, C - G, A + T with the two sequences' A + T in one
    transform).  Their FindTop offsets agree except at lags that one of them
    lists as near its threshold; where a pair's offsets agree its records
    are identical; the records of both equal the oracle's over their own
    offsets.  The chunks include an N run (handed back to the per-strand
    kernel), an empty chunk and a short last query chunk whose length is not
    a multiple of the entropy window."""
    import satsuma2_gb300 as sg
    rng = np.random.default_rng(93)
    t = W.random_bases(rng, 3072 * 12 + 1024)
    q = W.mutate(rng, t[2000:3072 * 12], 0.85)
    q = np.concatenate([q, W.random_bases(rng, 4096 * 9 + 2001 - len(q))]) if len(q) < 4096 * 9 + 2001 else q[:4096 * 9 + 2001]
    q[4096 * 2 + 100:4096 * 2 + 300] = ord("N")
    tc = np.array(W.chunk_starts(len(t), 4096, 1024), np.int64)
    qc = np.array(W.chunk_starts(len(q), 4096, 0), np.int64)
    qc = np.concatenate([qc, [[len(q), len(q)]]])          # an empty chunk
    blocks = [sg.block_pairs(t, tc, q, qc, 0, len(tc) - 1, 0, len(qc) - 1)]
    items = blocks[0]
    TT = float(len(t))
    x_on = sg.XCorr(target_total=TT)
    monkeypatch.setenv("SATSUMA2_GB300_SPECTRA", "0")
    x_off = sg.XCorr(target_total=TT)
    monkeypatch.delenv("SATSUMA2_GB300_SPECTRA")
    b_on, b_off = x_on.upload(items), x_off.upload(items)
    assert b_on.launches() == b_off.launches() + 1           # the spectra kernel
    b_on.run()
    b_off.run()
    r_on, c_on = b_on.results(with_counts=True)
    r_off, c_off = b_off.results(with_counts=True)
    o_on, o_off = b_on.offsets(), b_off.offsets()
    n_on, l_on = b_on.straddles()
    n_off, l_off = b_off.straddles()
    s_on = np.concatenate([[0], np.cumsum(c_on.astype(np.int64))])
    s_off = np.concatenate([[0], np.cumsum(c_off.astype(np.int64))])
    n_diff = n_same = 0
    for k in range(len(items)):
        same = True
        for s2 in range(2):
            d = set(o_on[k][s2].tolist()) ^ set(o_off[k][s2].tolist())
            if d:
                same = False
                n_diff += len(d)
                assert n_on[k, s2] <= sg.STRAD_CAP and n_off[k, s2] <= sg.STRAD_CAP
                near = set(l_on[k, s2][:n_on[k, s2]].tolist()) | set(l_off[k, s2][:n_off[k, s2]].tolist())
                assert d <= near, (k, s2, sorted(d - near))
        if same:
            n_same += 1
            assert parity.same_results(r_on[s_on[k]:s_on[k + 1]], r_off[s_off[k]:s_off[k + 1]], prob_rtol=0.0,
                                       target_total=0.0), k
    assert n_diff <= 4 and n_same >= len(items) - 4, (n_diff, n_same)
    assert len(r_on) > 0
    P = O.params(target_total=TT)
    tb, qb = t.tobytes(), q.tobytes()
    for k in range(0, len(items), 7):
        it = items[k]
        ts, qs = int(it["t_chunk_start"]), int(it["q_chunk_start"])
        pr = O.pair(tb[ts:ts + int(it["tlen"])], qb[qs:qs + int(it["qlen"])], t_chunk_start=ts, q_chunk_start=qs,
                    query_size=len(qb))
        for o, r, st in ((o_on, r_on, s_on), (o_off, r_off, s_off)):
            want, _ = O.align_pair(P, pr, offsets_in=o[k])
            assert parity.same_results(r[st[k]:st[k + 1]], want, target_total=TT), k
    b_on.free()
    b_off.free()
    x_on.close()
    x_off.close()


def test_serving_probtable_blocks_overflow_vs_oracle(O):
    """Serving in -prob_table mode: three 576-pair grid blocks plus a batch of
    tandem-repeat pairs, submitted together.  At hundreds of records per pair
    the slot batches overflow their device result pool; the scheduler grows
    it and runs the batch again.  Every request's records equal
    xc_align_pairs', and the oracle's over the GPU's own offsets."""
    import satsuma2_gb300 as sg
    from concurrent.futures import ThreadPoolExecutor
    rng = np.random.default_rng(61)
    genome = W.random_bases(rng, 3072 * 40 + 1024)
    tchunks = [genome[3072 * i:3072 * i + 4096].tobytes() for i in range(40)]
    qg = W.mutate(rng, genome[:4096 * 30], 0.85)
    qchunks = [qg[4096 * i:4096 * i + 4096].tobytes() for i in range(len(qg) // 4096)]
    blocks = [_block_items(tchunks, qchunks, 0, 0), _block_items(tchunks, qchunks, 8, 2),
              _block_items(tchunks, qchunks, 16, 4)]
    reps = []
    for k in range(64):
        t = W.random_bases(rng, 4096)
        rep = W.tandem_repeat(rng, int(rng.integers(200, 1200)), 1, 6)
        p = int(rng.integers(0, 4096 - len(rep)))
        t[p:p + len(rep)] = rep
        q = W.random_bases(rng, 4096)
        p2 = int(rng.integers(0, 4096 - len(rep)))
        q[p2:p2 + len(rep)] = W.mutate(rng, rep, 0.97, indel_every=0)
        reps.append((t.tobytes(), q.tobytes()))
    reqs = blocks + [reps]
    TT = 4096.0 * 64
    x = sg.XCorr(target_total=TT, prob_table=True, prob_table_cutoff=0.9999, max_batch=4096)
    tickets = [x.submit(r) for r in reqs]
    served = [x.wait(tk, timeout_ms=300000) for tk in tickets]
    pt = O.probtable(TT, 0.9999)
    P = O.params(target_total=TT, probtable=pt, probtable_cutoff=0.9999)
    total = 0
    for r, got in zip(reqs, served):
        want, counts = x.align(r, with_counts=True)
        assert parity.same_results(got, want, target_total=TT)
        total += len(got)
        offs = [x.debug_pair(signals=False, **(it if isinstance(it, dict) else dict(t=it[0], q=it[1])))["offsets"]
                for it in r]

        def one(k):
            it = r[k] if isinstance(r[k], dict) else dict(t=r[k][0], q=r[k][1])
            pr = O.pair(it["t"], it["q"], t_chunk_start=it.get("t_chunk_start", 0),
                        q_chunk_start=it.get("q_chunk_start", 0), query_size=it.get("query_size"))
            return O.align_pair(P, pr, offsets_in=offs[k])[0]
        with ThreadPoolExecutor(16) as ex:
            oracle_recs = list(ex.map(one, range(len(r))))
        o = 0
        for k in range(len(r)):
            mine = want[o:o + int(counts[k])]
            o += int(counts[k])
            assert parity.same_results(mine, oracle_recs[k], target_total=TT), k
    assert total > 3 * 65536   # well past one batch's initial overflow pool
    x.close()


def test_serving_same_alone_and_in_mix():
    """Continuous batching: each request's results equal its standalone run."""
    import satsuma2_gb300 as sg
    x = sg.XCorr(target_total=4096.0 * 4096, max_batch=96)
    pool = W.uniform_batch(96, seed=44)
    reqs = [pool[i:i + 1 + (i % 5)] for i in range(0, 90, 6)]
    alone = [x.align(r) for r in reqs]
    tickets = [None] * len(reqs)

    def worker(k):
        tickets[k] = x.submit(reqs[k])

    th = [threading.Thread(target=worker, args=(k,)) for k in range(len(reqs))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for k, tk in enumerate(tickets):
        got = x.wait(tk, timeout_ms=60000)
        assert parity.same_results(got, alone[k])
    st = x.serving_stats()
    assert st["completed"] >= len(reqs)
    x.close()


def test_wait_times_out_and_keeps_ticket():
    import satsuma2_gb300 as sg
    x = sg.XCorr(target_total=4096.0 * 4096)
    items = W.uniform_batch(512, seed=45)
    tk = x.submit(items)
    try:
        x.wait(tk, timeout_ms=0)
        timed_out = False
    except sg.XCError as e:
        assert e.code == -6
        timed_out = True
    res = x.wait(tk, timeout_ms=120000)
    assert len(res) >= 0
    assert timed_out or len(res) >= 0
    x.close()


def test_edge_chunks_match_oracle(O):
    """Empty chunks (the slave clears all-N chunks to length 0), very short
    ones, odd lengths, a chunk of N only and one of IUPAC letters, in one
    batch: every pair's records equal the oracle's over the GPU's offsets."""
    import satsuma2_gb300 as sg
    rng = np.random.default_rng(44)
    full = W.random_bases(rng, 4096).tobytes()
    items = [
        (b"", full), (full, b""), (b"", b""),
        (full[:5], full[:7]), (full[:45], full[:46]), (full[:47], full[:47]),
        (full[:1023], full[:1025]), (full[:1024], full[:3001]), (full[3:3004], full[:4096]),
        (b"", full[:2001]), (full[:2001], b""),
        (b"N" * 4096, full), (full[:2000] + b"RYKMSWBDHVN" * 50 + full[2550:4096], full),
    ]
    TT = 4096.0 * 16
    x = sg.XCorr(target_total=TT)
    res, counts = x.align(items, with_counts=True)
    P = O.params(target_total=TT)
    o = 0
    for k, (t, q) in enumerate(items):
        got = res[o:o + int(counts[k])]
        o += int(counts[k])
        d = x.debug_pair(t=t, q=q, signals=False)
        want, _ = O.align_pair(P, O.pair(t, q), offsets_in=d["offsets"])
        assert parity.same_results(got, want, target_total=TT), k
    x.close()


def _mixed_items(rng):
    """A/C/G/T pairs (both-strands kernel) interleaved with pairs it hands
    back to the per-strand kernel: an N run, IUPAC letters, query lengths
    that are not a multiple of the 16-base entropy window."""
    items = []
    for k in range(48):
        t = W.random_bases(rng, 4096).tobytes()
        q = bytearray(t[500:3500] + W.random_bases(rng, 1096).tobytes())
        for i in rng.choice(len(q), 300, replace=False):
            q[i] = b"ACGT"[rng.integers(4)]
        q = bytes(q)
        kind = k % 4
        if kind == 1:
            q = q[:2000] + b"N" * 100 + q[2100:]
        elif kind == 2:
            q = q[:4096 - 7]
        elif kind == 3:
            t = t[:1500] + b"RYKM" * 10 + t[1540:]
        items.append((t, q))
    return items


def test_mixed_batch_both_kernels_vs_oracle(O):
    """One launch where the both-strands kernel hands every fourth pair or
    so back to the per-strand kernel: each pair's records equal the oracle's
    over the GPU's own offsets."""
    import satsuma2_gb300 as sg
    rng = np.random.default_rng(71)
    items = _mixed_items(rng)
    TT = 4096.0 * 48
    x = sg.XCorr(target_total=TT)
    res, counts = x.align(items, with_counts=True)
    P = O.params(target_total=TT)
    o = 0
    n_rec = 0
    for k, (t, q) in enumerate(items):
        got = res[o:o + int(counts[k])]
        o += int(counts[k])
        n_rec += len(got)
        d = x.debug_pair(t=t, q=q, signals=False)
        want, _ = O.align_pair(P, O.pair(t, q), offsets_in=d["offsets"])
        assert parity.same_results(got, want, target_total=TT), k
    assert n_rec > 48
    x.close()


def test_ragged_query_kernel_vs_oracle(O, monkeypatch):
    """A/C/G/T pairs whose query is at least 1024 bases and not a multiple of
    the 16-base entropy window, so that the reverse complement's windows do
    not line up with the forward query's: the both-strands kernel hands them
    on to corr_rcq_kernel, one more launch.  Their offsets agree with the
    oracle's FP64 correlation and with the per-strand kernel's except inside
    the straddle band, and every pair's records equal the oracle's over the
    batch's own offsets.  Aligned pairs (a 4096-base and a 1008-base query),
    short targets (all window weights 1) and a ragged query holding an N
    (the per-strand kernel's) share the launch."""
    import satsuma2_gb300 as sg
    rng = np.random.default_rng(61)
    qlens = [1025, 1031, 1039, 1503, 2047, 2049, 3001, 3333, 4081, 4089, 4095, 4096, 1008]
    items = []
    for k, ql in enumerate(qlens * 2):
        t = W.random_bases(rng, 4096 if k % 3 else 4091)
        a = int(rng.integers(0, 4096 - 1000))
        seg = W.mutate(rng, t[a:a + min(ql, len(t) - a)], 0.85, indel_every=0)
        q = np.concatenate([seg, W.random_bases(rng, ql - len(seg))])
        q = W.revcomp(q) if k % 2 else q
        items.append((t.tobytes(), q.tobytes()))
    for tl, ql in ((700, 2047), (1023, 3001)):
        t = W.random_bases(rng, tl)
        q = np.concatenate([W.mutate(rng, t, 0.9, indel_every=0), W.random_bases(rng, ql - tl)])
        items.append((t.tobytes(), q.tobytes()))
    t, q = items[5]
    items.append((t, q[:1000] + b"N" + q[1001:]))
    TT = 4096.0 * len(items)
    x2 = sg.XCorr(target_total=TT)
    monkeypatch.setenv("SATSUMA2_GB300_PAIR_KERNEL", "0")
    x1 = sg.XCorr(target_total=TT)
    monkeypatch.delenv("SATSUMA2_GB300_PAIR_KERNEL")
    b = x2.upload(items)
    # both-strands kernel, ragged-query kernel, hand-back, scan, two finalize kernels
    assert b.launches() == 6
    b.run()
    res, counts = b.results(with_counts=True)
    offs = b.offsets()
    P = O.params(target_total=TT)
    o = 0
    n_rec = [0, 0]
    for k, (t, q) in enumerate(items):
        got = res[o:o + int(counts[k])]
        o += int(counts[k])
        n_rec[k % 2] += len(got)
        want, _ = O.align_pair(P, O.pair(t, q), offsets_in=offs[k])
        assert parity.same_results(got, want, target_total=TT), k
        d1 = x1.debug_pair(t=t, q=q, signals=False)
        _, det = O.align_pair(P, O.pair(t, q), want_detail=True)
        case = dict(L=8192, cutoff=1.8, t=t)
        for s, qq in enumerate((q, O.rc(q))):
            band, _ = parity.straddles(O, case, qq, s)
            parity.compare_offsets(offs[k][s], det["offsets"][s], band)
            parity.compare_offsets(offs[k][s], d1["offsets"][s], band)
    assert min(n_rec) > 0   # records on both strands' seeds
    b.free()
    x1.close()
    x2.close()
    assert [len(q) % 16 != 0 for _, q in items[-3:]] == [True, True, True]


def test_strand_kernel_switch_vs_oracle(O, monkeypatch):
    """SATSUMA2_GB300_PAIR_KERNEL=0 at context creation runs every pair one
    CTA per strand; its records equal the oracle's over its own offsets, and
    the offsets agree with the both-strands kernel's except inside the
    straddle band."""
    import satsuma2_gb300 as sg
    items = W.uniform_batch(24, seed=9)
    TT = 4096.0 * 4096
    x2 = sg.XCorr(target_total=TT)
    monkeypatch.setenv("SATSUMA2_GB300_PAIR_KERNEL", "0")
    x1 = sg.XCorr(target_total=TT)
    monkeypatch.delenv("SATSUMA2_GB300_PAIR_KERNEL")
    res, counts = x1.align(items, with_counts=True)
    P = O.params(target_total=TT)
    o = 0
    for k, (t, q) in enumerate(items):
        got = res[o:o + int(counts[k])]
        o += int(counts[k])
        d1 = x1.debug_pair(t=t, q=q, signals=False)
        want, _ = O.align_pair(P, O.pair(t, q), offsets_in=d1["offsets"])
        assert parity.same_results(got, want, target_total=TT), k
        d2 = x2.debug_pair(t=t, q=q, signals=False)
        case = dict(L=8192, cutoff=1.8, t=t)
        for s, qq in enumerate((q, O.rc(q))):
            band, _ = parity.straddles(O, case, qq, s)
            parity.compare_offsets(d2["offsets"][s], d1["offsets"][s], band)
            xa, xb = d1["xc"][s].astype(np.float64), d2["xc"][s].astype(np.float64)
            assert np.abs(xa - xb).max() <= 1e-4 * max(1.0, np.abs(xa).max())
    x1.close()
    x2.close()


def _oscillating_pair():
    """Target periodic in 64 bp; the query equals it exactly where a bit
    pattern e is 1, so every diagonal at a multiple of 64 has equality bits e
    (shifted).  e keeps the 46-wide window count at 18/19, flipping about ten
    times per 32-check word, so those diagonals carry ~10 DoOne segments per
    word where random ones carry ~1."""
    n = 4096
    rng = np.random.default_rng(38)
    e = np.zeros(n, np.int64)
    e[rng.choice(46, 19, replace=False)] = 1
    W = int(e[:46].sum())
    for c in range(46, n):
        base = W - e[c - 46]
        e[c] = 1 if W < 19 else 0
        W = base + e[c]
    acgt = np.frombuffer(b"ACGT", np.uint8)
    rng2 = np.random.default_rng(5)
    t = np.tile(acgt[rng2.integers(0, 4, 64)], n // 64)
    code = {65: 0, 67: 1, 71: 2, 84: 3}
    q = t.copy()
    for i in np.nonzero(e == 0)[0]:
        q[i] = acgt[(code[int(t[i])] + int(rng2.integers(1, 4))) % 4]
    return t.tobytes(), q.tobytes()


def test_scan_queue_overflow_vs_oracle(O):
    """Sub-ranges of up to 1280 marked words, ~10 segments each on the
    oscillating diagonals, against a queue of 2048 segment descriptors: the
    items that do not fit run their segments in place after the barrier.  All
    raw DoOne segments equal the oracle's on the GPU's offsets, and so do the
    records."""
    import satsuma2_gb300 as sg
    t, q = _oscillating_pair()
    TT = 4096.0 * 64
    x = sg.XCorr(target_total=TT)
    d = x.debug_pair(t=t, q=q, signals=False, seg_cap=1 << 19)
    total = 0
    for s, qq in enumerate((q, O.rc(q))):
        want = [O.doone(t, qq, int(i) - 4096) for i in d["offsets"][s]]
        want = np.concatenate(want) if want else np.zeros((0, 3), np.int32)
        total += len(want)
        assert np.array_equal(d["segments"][s].reshape(-1, 3), want.reshape(-1, 3)), s
    assert total > 20 * 2048   # far more segments than a sub-range's queue holds
    res = x.align([(t, q)])
    P = O.params(target_total=TT)
    want, _ = O.align_pair(P, O.pair(t, q), offsets_in=d["offsets"])
    assert parity.same_results(res, want, target_total=TT)
    x.close()


def test_randomized_batch_vs_oracle(O):
    """A seeded mix in one batch: lengths spread over the FFT buckets (many
    queries not a multiple of the 16-base window), homology on either
    strand, N runs, IUPAC letters, tandem repeats and empty chunks; every
    pair's records equal the oracle's over the GPU's own offsets, and the
    same items one at a time give the same records."""
    import satsuma2_gb300 as sg
    rng = np.random.default_rng(2024)
    items = []
    for k in range(96):
        tl = int(rng.integers(0, 4097)) if k % 11 else 0
        ql = int(rng.integers(300, 4097)) if k % 13 else 0
        t = W.random_bases(rng, tl, gc=float(rng.uniform(0.35, 0.6)))
        if tl > 600 and ql > 600 and k % 4:
            a = int(rng.integers(0, tl - 500))
            n = min(ql, tl - a)
            q = W.mutate(rng, t[a:a + n], float(rng.uniform(0.75, 0.95)), indel_every=400)[:ql]
            q = np.concatenate([q, W.random_bases(rng, ql - len(q))]) if len(q) < ql else q
            if k % 3 == 0:
                q = W.revcomp(q)
        else:
            q = W.random_bases(rng, ql)
        t, q = bytearray(t.tobytes()), bytearray(q.tobytes())
        if k % 7 == 0 and len(q) > 300:
            i = int(rng.integers(0, len(q) - 200))
            q[i:i + 150] = b"N" * 150
        if k % 9 == 0 and len(t) > 300:
            i = int(rng.integers(0, len(t) - 100))
            t[i:i + 40] = b"RYKMSWBDHV" * 4
        if k % 5 == 0 and len(t) > 400 and len(q) > 400:
            unit = bytes(b"ACGT"[j] for j in rng.integers(0, 4, int(rng.integers(2, 7))))
            rep = (unit * 100)[:200]
            i, j = int(rng.integers(0, len(t) - 200)), int(rng.integers(0, len(q) - 200))
            t[i:i + 200] = rep
            q[j:j + 200] = rep
        items.append((bytes(t), bytes(q)))
    assert sum(1 for _, q in items if len(q) >= 1024 and len(q) % 16) > 20
    TT = float(sum(len(t) for t, _ in items)) + 1.0
    x = sg.XCorr(fft_len=-1, target_total=TT)
    res, counts = x.align(items, with_counts=True)
    P = O.params(target_total=TT, fft_len=0)
    o = 0
    n_rec = 0
    for k, (t, q) in enumerate(items):
        got = res[o:o + int(counts[k])]
        o += int(counts[k])
        n_rec += len(got)
        d = x.debug_pair(t=t, q=q, signals=False)
        Pk = O.params(target_total=TT, fft_len=d["L"])
        want, _ = O.align_pair(Pk, O.pair(t, q), offsets_in=d["offsets"])
        assert parity.same_results(got, want, target_total=TT), k
        if k % 8 == 0:
            assert parity.same_results(x.align([(t, q)]), got, target_total=TT), k
    assert n_rec > 50
    x.close()
