"""CPU model of the scan kernel's floors (xc_scan.cu, run_hits_floor in
xc_runtime.cu).  Phase AB: a run of r passing checks inside one 32-check
word makes a segment of r + 45 bases whose equal-base count the kernel takes
from the word's equality bits; below the floor for r no G+C composition lets
the segment pass the probability screen.  Pass 1: a screened word whose edge
blocks fail and whose inner positions hold fewer equal bases than the least
floor stays unmarked; with the floors on, pass 1 marks by exactly those two
tests, without the eight-block screen (a superset of the screened marks).  Restated here in double and checked against the
oracle: every segment the floor drops has a match probability below
min_prob (so it never makes a record), and every word of a record-making
segment stays marked, for the screen settings of the uniform, genome and
strict workloads and with a min_len."""
import math

import numpy as np
import pytest

import oracle
from satsuma2_gb300 import workloads as W


def screen_z(min_prob, target_total):
    """The kernel's screen threshold (xc_runtime.cu screen_z), rounded to FP32."""
    r = -math.log(min_prob) / target_total * 1.01 + 4.5e-16
    lo, hi = -60.0, 60.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if 0.5 * math.erfc(-mid / math.sqrt(2.0)) <= r:
            lo = mid
        else:
            hi = mid
    return float(np.float32(hi + 0.02))


def floors(sz, min_len):
    """Least equal-base count per run length r = 1..32 (index r - 1)."""
    out = [0] * 32
    if not (sz < 0) or not math.isfinite(sz):
        return out
    for r in range(1, 33):
        n = r + 45
        fh = n + 1
        for h in range(1, n + 1):
            m = 1.0 - h / n
            p = (1.0 - m * m) / 4.0
            z = 0.0 if p * n >= h else (p * n - h) / math.sqrt(p * (1.0 - p) * n)
            if z <= sz + 1e-6:
                fh = h
                break
        out[r - 1] = 255 if n < min_len else min(fh, 255)
    return out


def _dropped(O, t, q, pos, fl):
    """The oracle's DoOne segments on one diagonal that the floor drops."""
    ta, qa = np.frombuffer(t, np.uint8), np.frombuffer(q, np.uint8)
    out = []
    for s0, _, ln in O.doone(t, q, pos):
        a, b = s0 + 45, s0 + ln - 1          # first and last passing check
        if (a >> 5) != (b >> 5):
            continue                          # not inside one word: kept
        r = b - a + 1
        eq = ta[s0:s0 + ln] == qa[s0 + pos:s0 + pos + ln]
        if int(eq.sum()) < fl[r - 1]:
            out.append((s0, ln))
    return out


@pytest.fixture(scope="module")
def O():
    return oracle.Oracle()


@pytest.mark.parametrize("min_prob,target_total,min_len", [
    (0.99, 4096.0 ** 2, 0),        # uniform 4096-pair workload
    (0.99, 2.0e7, 0),              # 20 Mb genome
    (0.99999, 4096.0 ** 2, 0),     # strict setting
    (0.99, 4096.0 ** 2, 60),       # with a minimum length
])
def test_floor_drops_no_record(O, min_prob, target_total, min_len):
    fl = floors(screen_z(min_prob, target_total), min_len)
    body = [f for r, f in enumerate(fl, 1) if r + 45 >= min_len]
    assert min(fl) > 19 and body == sorted(body)   # above the window minimum, nondecreasing
    assert all(f == 255 for r, f in enumerate(fl, 1) if r + 45 < min_len)
    items = W.uniform_batch(6, seed=17)
    P = O.params(target_total=target_total, min_prob=min_prob, min_len=min_len)
    n_seg = n_drop = 0
    for t, q in items:
        _, det = O.align_pair(P, O.pair(t, q), want_detail=True)
        for s, qq in enumerate((q, O.rc(q))):
            for off in det["offsets"][s]:
                pos = int(off) - 4096
                n_seg += len(O.doone(t, qq, pos))
                for s0, ln in _dropped(O, t, qq, pos, fl):
                    n_drop += 1
                    if ln < min_len:
                        continue
                    p, _ = O.match_prob(t, qq, s0, s0 + pos, ln, target_total)
                    assert p < min_prob, (s0, ln, p)
    assert n_drop > (3 * n_seg) // 4   # most segments are short noise runs


def test_floor_off_when_screen_keeps_all():
    assert floors(float("inf"), 0) == [0] * 32
    assert floors(0.5, 0) == [0] * 32


def _words_model(eq, w, F):
    """(screened, marked, marked_by_floor) of word w of a diagonal, positions
    out of range counted unequal: screened when some 4-check block's
    49-position span holds >= 19 equal bases; marked (the screened form) when
    screened and, besides, block 0 or block 7 passes or the 69 positions under
    checks 4..27 hold >= F equal bases; marked_by_floor (pass 1's form with
    the floors on) when block 0 or block 7 passes or those 69 positions hold
    >= F equal bases."""
    def cnt(lo, hi):   # equal bases at positions lo..hi
        lo, hi = max(lo, 0), min(hi, len(eq) - 1)
        return int(eq[lo:hi + 1].sum()) if hi >= lo else 0
    c = 32 * w
    blocks = [cnt(c + 4 * b - 45, c + 4 * b + 3) >= 19 for b in range(8)]
    screened = any(blocks)
    edge = blocks[0] or blocks[7]
    floor = cnt(c - 41, c + 27) >= F
    return screened, screened and (edge or floor), edge or floor


@pytest.mark.parametrize("min_prob,target_total", [(0.99, 4096.0 ** 2), (0.99999, 2.0e7)])
def test_word_floor_keeps_record_words(O, min_prob, target_total):
    """Pass 1 leaves a word unmarked when its edge blocks fail and the
    positions under its inner checks hold fewer equal bases than the least
    run floor: every word holding a check of a segment that makes a record
    stays marked, in both forms, and the marks stay a small share of the
    words (the floor form marks every word the screened form marks)."""
    fl = floors(screen_z(min_prob, target_total), 0)
    F = min(fl)
    items = W.uniform_batch(4, seed=29)
    P = O.params(target_total=target_total, min_prob=min_prob)
    n_words = n_screened = n_marked = n_floor = n_rec = 0
    for t, q in items:
        _, det = O.align_pair(P, O.pair(t, q), want_detail=True)
        ta = np.frombuffer(t, np.uint8)
        for s, qq in enumerate((q, O.rc(q))):
            qa = np.frombuffer(qq, np.uint8)
            for off in det["offsets"][s][::4]:
                pos = int(off) - 4096
                eq = np.zeros(len(ta), bool)
                lo, hi = max(0, -pos), min(len(ta), len(qa) - pos)
                if hi > lo:
                    eq[lo:hi] = ta[lo:hi] == qa[lo + pos:hi + pos]
                marks = {}
                for w in range(len(ta) // 32 + 1):
                    sc, mk, mf = _words_model(eq, w, F)
                    assert mf or not mk
                    n_words += 1
                    n_screened += sc
                    n_marked += mk
                    n_floor += mf
                    marks[w] = mk
                for s0, _, ln in O.doone(t, qq, pos):
                    p, _ = O.match_prob(t, qq, s0, s0 + pos, ln, target_total)
                    if p < min_prob:
                        continue
                    n_rec += 1
                    for w in range((s0 + 45) >> 5, ((s0 + ln - 1) >> 5) + 1):
                        assert marks[w], (pos, s0, ln, w)
    assert n_rec > 0
    assert n_marked < 0.8 * n_screened, (n_marked, n_screened)
    assert n_floor < 0.1 * n_words, (n_floor, n_words)
