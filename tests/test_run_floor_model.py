"""CPU model of the scan kernel's floor on in-word runs (xc_scan.cu phase AB,
run_hits_floor in xc_runtime.cu): a run of r passing checks inside one
32-check word makes a segment of r + 45 bases whose equal-base count is at
most window(b)'s count plus r - 1; below the floor for r no G+C composition
lets the segment pass the probability screen.  Restated here in double and
checked against the oracle: every segment the floor drops has a match
probability below min_prob (so it never makes a record), for the screen
settings of the uniform, genome and strict workloads and with a min_len."""
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
        wb = int(eq[ln - 46:].sum())
        assert int(eq.sum()) <= wb + r - 1    # the bound itself
        if wb + r - 1 < fl[r - 1]:
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
    assert n_drop > n_seg // 2   # most segments are short noise runs


def test_floor_off_when_screen_keeps_all():
    assert floors(float("inf"), 0) == [0] * 32
    assert floors(0.5, 0) == [0] * 32
