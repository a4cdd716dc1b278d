"""Generates the golden fixtures for the cross-correlation path from the
reference itself (run in a container that has the reference tree).

* ``cases.npz``     -- per-stage outputs of the reference library
  (oracle/_ref/libsatsuma_ref.so, the reference sources compiled in place) for
  seeded chunk pairs covering the edge cases of the path: the plain 4096x4096
  pair, homologous / reverse-complemented / unrelated pairs, identical
  sequences, short chunks (<1024 bp, entropy weight 1), FFT lengths 1024-32768
  (envelope disabled at L<=2048), IUPAC / N / '-' / unknown letters, empty and
  all-N chunks, the fast cutoff, a minimum length filter, the reverse-strand
  coordinate mapping of a short last query chunk, and the probability-table
  mode.  Stored per case: inputs, parameters, SHA-1 of every signal channel,
  FindTop offsets and DoOne segments per strand, t_result records.
* ``slave_e2e.npz`` -- t_result records produced by the unmodified reference
  slave binary (oracle/_ref/HomologyByXCorrSlave) over a small genome pair,
  driven through its TCP protocol (analysis/WorkQueue.cc:93-166 master side)
  by a fake master in this script.
* ``slave_e2e_probtable.npz`` -- the same genome pair with the slave's
  ``-prob_table -min_prob 0.9999`` (ProbTable lookups instead of erf/exp,
  HomologyByXCorrSlave.cc:186-199, 413-421) over the first two blocks of
  ``slave_e2e.npz`` (``n_blocks``): the records only; the sequences and blocks
  are those of ``slave_e2e.npz``.

Usage: python tests/golden/make_golden.py [cases|slave|probtable ...]
(all three by default; builds oracle/_ref first)
"""
import hashlib
import json
import os
import socket
import struct
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from satsuma2_gb300 import workloads as W  # noqa: E402

SEED = 42


def sha1(a):
    return hashlib.sha1(np.ascontiguousarray(a).tobytes()).hexdigest()


def iupac_seq(rng, n, frac=0.08):
    s = W.random_bases(rng, n)
    letters = np.frombuffer(b"NKMRYSWBVHDX-Z", np.uint8)
    m = rng.random(n) < frac
    s[m] = letters[rng.integers(0, len(letters), int(m.sum()))]
    if n > 600:
        p = int(rng.integers(0, n - 300))
        s[p:p + 200] = ord("N")
    return s


def build_cases():
    rng = np.random.default_rng(SEED)
    cases = []

    def add(name, t, q, L, **kw):
        c = dict(name=name, t=bytes(t), q=bytes(q), L=L, cutoff=1.8, min_prob=0.99,
                 target_total=4096.0, min_len=0, query_chunk=4096, t_chunk_start=0, target_id=0,
                 q_chunk_start=0, query_id=0, query_size=len(q), probtable=0,
                 probtable_cutoff=0.0)
        c.update(kw)
        cases.append(c)

    t, q = W.plain_pair(SEED)
    add("plain_pair_p099", t, q, 8192)
    add("plain_pair_p099999", t, q, 8192, min_prob=0.99999)
    for i, (t, q) in enumerate(W.uniform_batch(8, seed=7)):
        add("uniform_%d" % i, t, q, 8192, target_total=4096.0 * 4096)
    t = W.random_bases(rng, 4096).tobytes()
    add("identical", t, t, 8192)
    t, q = W.uniform_batch(2, seed=11)[1]
    add("fast_cutoff", t, q, 8192, cutoff=2.9)
    t = W.random_bases(rng, 800)
    add("short_chunks", t, W.mutate(rng, t[100:700], 0.9), 8192)
    t = W.random_bases(rng, 700)
    add("L2048_no_envelope", t, np.concatenate([W.random_bases(rng, 300), W.mutate(rng, t, 0.85)]),
        2048)
    t = W.random_bases(rng, 400)
    add("L1024", t, np.concatenate([W.mutate(rng, t[50:], 0.9), W.random_bases(rng, 150)]), 1024)
    t = W.random_bases(rng, 1500)
    add("L4096_partial_windows", t,
        np.concatenate([W.random_bases(rng, 333), W.mutate(rng, t[200:1400], 0.8),
                        W.random_bases(rng, 470)]), 4096)
    t = iupac_seq(rng, 4096)
    q = iupac_seq(rng, 3000)
    q[1000:2500] = W.mutate(rng, t[1500:3000], 0.9, indel_every=0)
    add("iupac_letters", t, q, 8192)
    add("all_N_query", W.random_bases(rng, 4096), b"N" * 4096, 8192)
    add("empty_query", W.random_bases(rng, 4096), b"", 8192)
    add("empty_target", b"", W.random_bases(rng, 4096), 8192)
    t = W.random_bases(rng, 4096)
    rep = W.tandem_repeat(rng, 300, 2, 6)
    t[1000:1300] = rep
    q = W.random_bases(rng, 4096)
    q[2000:2300] = W.mutate(rng, rep, 0.95, indel_every=0)
    add("tandem_repeats", t, q, 8192)
    for i, (t, q) in enumerate(W.uneven_batch(6, seed=5)):
        add("uneven_%d" % i, t, q, W.uneven_fft_len(len(t), len(q)))
    t, q = W.uniform_batch(3, seed=13)[2]
    add("min_len_100", t, q, 8192, min_len=100)
    t = W.random_bases(rng, 4096)
    q = W.mutate(rng, W.revcomp(t[1000:2808]), 0.9, indel_every=0)
    add("rc_short_last_query_chunk", t, q, 8192, t_chunk_start=3072, target_id=3,
        q_chunk_start=8192, query_id=1, query_size=8192 + len(q))
    t, q = W.uniform_batch(4, seed=17)[3]
    add("probtable_mode", t, q, 8192, probtable=1, probtable_cutoff=0.9999,
        target_total=4096.0 * 64)
    t, q = W.large_batch(1, seed=19)[0]
    add("large_L32768", t, q, 32768, target_total=16384.0 * 2000)
    return cases


def run_cases(R, O):
    out = {}
    meta = []
    tables = {}
    for k, c in enumerate(build_cases()):
        L = c["L"]
        pt = None
        if c["probtable"]:
            key = (c["target_total"], c["probtable_cutoff"])
            if key not in tables:
                tables[key] = R.probtable(*key)
            pt = tables[key][0]
            out["probtable_sha1_%d" % k] = np.array(sha1(tables[key][1]))
        t0 = time.time()
        res, det = R.align_pair(c["t"], c["q"], L, cutoff=c["cutoff"], min_len=c["min_len"],
                                min_prob=c["min_prob"], target_total=c["target_total"],
                                query_chunk=c["query_chunk"], t_chunk_start=c["t_chunk_start"],
                                target_id=c["target_id"], q_chunk_start=c["q_chunk_start"],
                                query_id=c["query_id"], query_size=c["query_size"],
                                probtable=pt, want_detail=True)
        dt = time.time() - t0
        rcq = R.rc(c["q"])
        sig = []
        for s in (c["t"], c["q"], rcq):
            x = R.signal(s, L)
            sig.append([sha1(x[ch]) for ch in range(4)])
        xc64 = [O.xcorr64(c["t"], c["q"], L), O.xcorr64(c["t"], rcq, L)]
        scale = max(1.0, max(float(np.abs(x).max()) for x in xc64))
        ref_err = max(float(np.abs(det["xc"][s].astype(np.float64) - xc64[s]).max())
                      for s in range(2)) / scale
        p = "c%d_" % k
        out[p + "t"] = np.frombuffer(c["t"], np.uint8)
        out[p + "q"] = np.frombuffer(c["q"], np.uint8)
        for s in range(2):
            out[p + "off%d" % s] = det["offsets"][s]
            out[p + "seg%d" % s] = det["segments"][s]
        out[p + "res"] = res
        m = {k2: v for k2, v in c.items() if k2 not in ("t", "q")}
        m.update(index=k, signal_sha1=sig, ref_xc_err_vs_fp64=ref_err, xc_scale=scale,
                 n_results=int(len(res)), ref_ms=dt * 1e3,
                 n_offsets=[int(len(det["offsets"][s])) for s in range(2)],
                 n_segments=[int(len(det["segments"][s])) for s in range(2)])
        meta.append(m)
        print("%-28s L=%-5d offs=%s segs=%s res=%d err=%.2e" % (
            c["name"], L, m["n_offsets"], m["n_segments"], len(res), ref_err))
    for h in tables.values():
        R.lib.ref_probtable_free(h[0])
    out["meta"] = np.array(json.dumps(meta))
    return out


# --------------------------------------------------------------------------
# End-to-end: the unmodified reference slave behind a fake master
# --------------------------------------------------------------------------
T_PAIR = struct.Struct("<iiii?xxxiB3x")   # t_pair, analysis/WorkQueue.h:17-22 (28 bytes)
assert T_PAIR.size == 28


def write_fasta(path, seqs):
    with open(path, "w") as f:
        for name, s in seqs:
            f.write(">%s\n" % name)
            for i in range(0, len(s), 80):
                f.write(s[i:i + 80].decode() + "\n")


def recv_exact(conn, n):
    buf = b""
    while len(buf) < n:
        chunk = conn.recv(n - len(buf))
        if not chunk:
            raise ConnectionError("slave closed")
        buf += chunk
    return buf


def slave_e2e(prob_table=False):
    rng = np.random.default_rng(SEED + 1)
    tg = [W.random_bases(rng, 20000), W.random_bases(rng, 9000)]
    qg = [W.mutate(rng, tg[0][2000:15000], 0.85),
          W.revcomp(W.mutate(rng, tg[1][1000:8000], 0.88)),
          W.random_bases(rng, 3000)]
    sentinel = W.random_bases(rng, 4096)
    targets = [("t%d" % i, s.tobytes()) for i, s in enumerate(tg)] + [("sentinel", sentinel.tobytes())]
    queries = [("q%d" % i, s.tobytes()) for i, s in enumerate(qg)] + [("sentinel", sentinel.tobytes())]
    tchunks = []
    for si, (_, s) in enumerate(targets):
        for (st, en) in W.chunk_starts(len(s), 4096, 1024):
            tchunks.append((si, st, en))
    qchunks = []
    for si, (_, s) in enumerate(queries):
        for (st, en) in W.chunk_starts(len(s), 4096, 0):
            qchunks.append((si, st, en))
    n_t_real = sum(1 for c in tchunks if c[0] < len(tg))
    n_q_real = sum(1 for c in qchunks if c[0] < len(qg))
    sent_t = n_t_real          # first sentinel target chunk
    sent_q = n_q_real          # first sentinel query chunk
    # t_pair blocks over all real chunk pairs, in 4x3 blocks, then the sentinel pair.
    blocks = []
    for qf in range(0, n_q_real, 3):
        for tf in range(0, n_t_real, 4):
            blocks.append((tf, min(tf + 3, n_t_real - 1), qf, min(qf + 2, n_q_real - 1), False))
    # -prob_table keeps thousands of records per pair here: the first two
    # blocks (homologous chunks) keep that fixture small
    n_blocks = 2 if prob_table else len(blocks)
    blocks = blocks[:n_blocks]
    blocks.append((sent_t, sent_t, sent_q, sent_q, False))
    tmp = tempfile.mkdtemp(prefix="satsuma_e2e_")
    write_fasta(os.path.join(tmp, "t.fa"), targets)
    write_fasta(os.path.join(tmp, "q.fa"), queries)
    srv = socket.socket(socket.AF_INET, socket.SOCK_STREAM)
    srv.setsockopt(socket.SOL_SOCKET, socket.SO_REUSEADDR, 1)
    srv.bind(("127.0.0.1", 0))
    srv.listen(16)
    port = srv.getsockname()[1]
    extra = ["-prob_table", "-min_prob", "0.9999"] if prob_table else []
    proc = subprocess.Popen([oracle.REF_SLAVE, "-master", "127.0.0.1", "-port", str(port),
                             "-sid", "1", "-p", "1", "-q", "q.fa", "-t", "t.fa"] + extra, cwd=tmp,
                            stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    results = []
    pending = list(blocks)
    done = False
    srv.settimeout(120)
    try:
        while True:
            conn, _ = srv.accept()
            with conn:
                recv_exact(conn, 4)                       # slave id
                cnt = struct.unpack("<I", recv_exact(conn, 4))[0]
                data = recv_exact(conn, 72 * cnt) if cnt else b""
                recs = np.frombuffer(data, oracle.RESULT_DTYPE).copy()
                results.append(recs)
                if len(recs) and np.any(recs["target_id"] == len(tg)):
                    done = True
                if done:
                    conn.sendall(struct.pack("<i", -1))
                    break
                if pending:
                    b = pending.pop(0)
                    conn.sendall(struct.pack("<i", 1) + T_PAIR.pack(b[0], b[1], b[2], b[3], b[4], 1, 0))
                else:
                    conn.sendall(struct.pack("<i", 0))
                    time.sleep(0.05)
    finally:
        srv.close()
        try:
            proc.wait(timeout=30)
        except subprocess.TimeoutExpired:
            proc.kill()
    allres = np.concatenate(results) if results else np.zeros(0, oracle.RESULT_DTYPE)
    allres = allres[allres["target_id"] < len(tg)]
    target_total = float(sum(len(s) for _, s in targets))
    if prob_table:
        print("slave e2e, -prob_table: %d blocks, %d results" % (len(blocks), len(allres)))
        return {"results": allres,
                "meta": np.array(json.dumps(dict(target_total=target_total, t_chunk=4096, q_chunk=4096,
                                                 cutoff=1.8, min_prob_effective=0.99, prob_table=1,
                                                 prob_table_cutoff=0.9999, n_blocks=n_blocks,
                                                 n_real_targets=len(tg), n_real_queries=len(qg))))}
    out = {
        "tg0": tg[0], "tg1": tg[1], "qg0": qg[0], "qg1": qg[1], "qg2": qg[2],
        "sentinel": sentinel,
        "tchunks": np.array(tchunks, np.int64), "qchunks": np.array(qchunks, np.int64),
        "blocks": np.array([b[:4] for b in blocks], np.int64),
        "results": allres,
        "meta": np.array(json.dumps(dict(target_total=target_total, t_chunk=4096, q_chunk=4096,
                                         cutoff=1.8, min_prob_effective=0.99,
                                         n_real_targets=len(tg), n_real_queries=len(qg)))),
    }
    print("slave e2e: %d blocks, %d results" % (len(blocks), len(allres)))
    return out


def main():
    what = set(sys.argv[1:]) or {"cases", "slave", "probtable"}
    oracle.install_ref()
    oracle.build_ref()
    R = oracle.Reference()
    O = oracle.Oracle()
    if "cases" in what:
        np.savez_compressed(os.path.join(HERE, "cases.npz"), **run_cases(R, O))
    if "slave" in what:
        np.savez_compressed(os.path.join(HERE, "slave_e2e.npz"), **slave_e2e())
    if "probtable" in what:
        np.savez_compressed(os.path.join(HERE, "slave_e2e_probtable.npz"), **slave_e2e(prob_table=True))


if __name__ == "__main__":
    main()
