"""The drop-in slave (satsuma2_gb300/satsuma2_slave) behind a fake master
speaking the reference's TCP protocol (HomologyByXCorrSlave.cc:447-526;
t_pair / t_result, WorkQueue.h:17-33).

The master serves the t_pair blocks of the reference-slave golden run
(tests/golden/slave_e2e.npz: same FASTA records, same 4096-bp chunking), then
a sentinel block, and answers -1 once the sentinel's records are in.  With one
worker the slave's record stream must equal, record for record and in order,
what xc_align_pairs gives for the same chunk pairs taken block by block
(query-major, target-minor); test_slave_end_to_end holds those records to the
unmodified reference slave's stream.  With three workers blocks finish out of
order, so the records are compared as a sorted set."""
import os
import socket
import struct
import subprocess
import tempfile
import time

import numpy as np
import pytest

import satsuma2_gb300 as sg
from satsuma2_gb300 import build
from tests import parity

pytestmark = pytest.mark.gpu

T_PAIR = struct.Struct("<iiii?xxxiB3x")
SLAVE = os.path.join(os.path.dirname(sg.__file__), "satsuma2_slave")


def write_fasta(path, seqs):
    with open(path, "w") as f:
        for name, s in seqs:
            f.write(">%s some description\n" % name)
            for i in range(0, len(s), 70):
                f.write(s[i:i + 70].decode().lower() + "\n")   # the slave uppercases


def recv_exact(conn, n):
    buf = b""
    while len(buf) < n:
        chunk = conn.recv(n - len(buf))
        if not chunk:
            raise ConnectionError("slave closed")
        buf += chunk
    return buf


def run_slave(d, threads, expected, extra=()):
    """Serves every golden block to the slave; returns its records (sentinel
    records removed) in arrival order."""
    tg = [d["tg0"], d["tg1"], d["sentinel"]]
    qg = [d["qg0"], d["qg1"], d["qg2"], d["sentinel"]]
    tmp = tempfile.mkdtemp(prefix="slave_gb300_")
    write_fasta(os.path.join(tmp, "t.fa"), [("t%d" % i, s.tobytes()) for i, s in enumerate(tg)])
    write_fasta(os.path.join(tmp, "q.fa"), [("q%d" % i, s.tobytes()) for i, s in enumerate(qg)])
    srv = socket.socket(socket.AF_INET, socket.SOCK_STREAM)
    srv.setsockopt(socket.SOL_SOCKET, socket.SO_REUSEADDR, 1)
    srv.bind(("127.0.0.1", 0))
    srv.listen(16)
    srv.settimeout(60)
    port = srv.getsockname()[1]
    proc = subprocess.Popen([SLAVE, "-master", "127.0.0.1", "-port", str(port), "-sid", "7", "-p", str(threads),
                             "-q", "q.fa", "-t", "t.fa"] + list(extra), cwd=tmp, stdout=subprocess.PIPE,
                            stderr=subprocess.STDOUT)
    n_real_t = d["meta"]["n_real_targets"]
    pending = [tuple(int(v) for v in b) for b in d["blocks"]]
    got = []
    sentinel_seen = False
    deadline = time.time() + 120
    try:
        while time.time() < deadline:
            conn, _ = srv.accept()
            with conn:
                assert struct.unpack("<i", recv_exact(conn, 4))[0] == 7
                cnt = struct.unpack("<I", recv_exact(conn, 4))[0]
                recs = np.frombuffer(recv_exact(conn, 72 * cnt), sg.RESULT_DTYPE).copy() if cnt else \
                    np.zeros(0, sg.RESULT_DTYPE)
                sentinel_seen |= bool(np.any(recs["target_id"] == n_real_t))
                got.append(recs[recs["target_id"] < n_real_t])
                n_got = sum(len(g) for g in got)
                if sentinel_seen and n_got >= expected:
                    conn.sendall(struct.pack("<i", -1))
                    break
                if pending:
                    tf, tt, qf, qt = pending.pop(0)
                    conn.sendall(struct.pack("<i", 1) + T_PAIR.pack(tf, tt, qf, qt, False, 7, 0))
                else:
                    conn.sendall(struct.pack("<i", 0))
                    time.sleep(0.02)
        else:
            raise AssertionError("slave did not finish")
        out, _ = proc.communicate(timeout=60)
    finally:
        srv.close()
        if proc.poll() is None:
            proc.kill()
    assert proc.returncode == 0, out.decode()[-2000:]
    return np.concatenate(got) if got else np.zeros(0, sg.RESULT_DTYPE)


def expected_stream(d, prob_table=False):
    """xc_align_pairs over every chunk pair of the blocks, block by block."""
    m = d["meta"]
    x = sg.XCorr(cutoff=m["cutoff"], min_prob=m["min_prob_effective"], target_total=m["target_total"],
                 t_chunk=m["t_chunk"], q_chunk=m["q_chunk"], prob_table=prob_table,
                 prob_table_cutoff=m.get("prob_table_cutoff", 0.9999))
    want = x.align(parity.slave_items(d))
    x.close()
    return want, m["target_total"]


def sort_key(r):
    return np.lexsort((r["len"], r["reverse"], r["qstart"], r["tstart"], r["query_id"], r["target_id"]))


@pytest.fixture(scope="module")
def golden():
    build.build()
    assert os.path.exists(SLAVE), "the slave executable is not built"
    d = parity.load_slave_e2e()
    want, tt = expected_stream(d)
    assert len(want) > 20
    return d, want, tt


def test_slave_stream_one_worker(golden):
    d, want, tt = golden
    got = run_slave(d, 1, len(want))
    assert parity.same_results(got, want, target_total=tt)


def test_slave_three_workers(golden):
    d, want, tt = golden
    got = run_slave(d, 3, len(want))
    assert parity.same_results(got[sort_key(got)], want[sort_key(want)], target_total=tt)


def test_slave_stream_probtable():
    """-prob_table -min_prob 0.9999: the table replaces erf/exp and thousands
    of records per pair come back (tests/golden/slave_e2e_probtable.npz holds
    the reference slave's records for the same blocks; test_gpu_parity holds
    xc_align_pairs to them)."""
    build.build()
    d = parity.load_slave_e2e_probtable()
    want, tt = expected_stream(d, prob_table=True)
    assert len(want) > 50000
    got = run_slave(d, 2, len(want), extra=("-prob_table", "-min_prob", "0.9999"))
    assert parity.same_results(got[sort_key(got)], want[sort_key(want)], target_total=tt)
