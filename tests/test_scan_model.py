"""CPU model of the scan kernel's bitplane DoOne (xc_scan.cu): 2-bit planes,
32-position equality words, the branch-free block screen (pass 1) and the
sparse exact pass with run tracking (pass 2), restated with Python integers
and checked against the oracle's DoOne on the same diagonals -- segments and
their equal-base counts exactly."""
import numpy as np
import pytest

import oracle
from satsuma2_gb300 import workloads as W

MIN_HITS = 19
M32 = 0xFFFFFFFF


def popc(x):
    return bin(x).count("1")


def lowmask(n):
    return M32 if n >= 32 else (1 << n) - 1


def planes(seq, nwords, pad=0):
    codes = [((b >> 1) ^ (b >> 2)) & 3 for b in seq]
    b0 = [0] * (nwords + pad)
    b1 = [0] * (nwords + pad)
    for i, c in enumerate(codes):
        w = i // 32 + pad
        b0[w] |= (c & 1) << (i & 31)
        b1[w] |= (c >> 1) << (i & 31)
    return b0, b1


def model_doone(t, q, pos):
    """Returns [(tstart, qstart, len, equal_bases)] as the kernel emits them."""
    T, Q = len(t), len(q)
    TW = max(T, Q) // 32 + 2
    tb0, tb1 = planes(t, TW + 2)
    qb0, qb1 = planes(q, TW + 8, pad=2)
    i0 = max(0, -pos)
    iend = min(T - 1, Q - pos)
    cfirst, clast = i0 + 46, iend - 1
    if clast < cfirst:
        return []

    def fs(lo, hi, sh):
        return ((hi << 32 | lo) >> sh) & M32

    def eword(w):
        if w < 0:
            return 0
        qo = 32 * w + pos + 64
        qw, sh = qo >> 5, qo & 31
        q0 = fs(qb0[qw], qb0[qw + 1], sh)
        q1 = fs(qb1[qw], qb1[qw + 1], sh)
        return ~((tb0[w] ^ q0) | (tb1[w] ^ q1)) & M32

    def validmask(w):
        lo, hi = max(cfirst - 32 * w, 0), min(clast - 32 * w, 31)
        return (M32 >> (31 - hi)) & (M32 << lo) & M32

    wfirst, wlast = cfirst >> 5, clast >> 5
    # pass 1
    flags = {}
    e2, e1 = eword(wfirst - 2), eword(wfirst - 1)
    for w in range(wfirst, wlast + 1):
        e0 = eword(w)
        U = (e1 << 32) | e2
        vm = validmask(w)
        f = 0
        for sb in range(4):
            a = 8 * sb + 19
            c53 = popc(U >> a) + popc(e0 & lowmask(a - 11))
            if c53 >= MIN_HITS and (vm >> (8 * sb)) & 0xFF:
                f |= 1 << sb
        if f:
            flags[w] = f
        e2, e1 = e1, e0
    # pass 2
    out = []
    opened, start, runcnt, accpos, lastw = False, 0, 0, 0, -4
    e2 = e1 = e0 = 0
    for w in sorted(flags):
        f = flags[w]
        if opened and w != lastw + 1:
            out.append((start, 32 * (lastw + 1), runcnt))
            opened = False
        if w == lastw + 1:
            e2, e1, e0 = e1, e0, eword(w)
        elif w == lastw + 2:
            e2, e1, e0 = e0, eword(w - 1), eword(w)
        else:
            e2, e1, e0 = eword(w - 2), eword(w - 1), eword(w)
        lastw = w
        U = (e1 << 32) | e2
        vm = validmask(w)
        g = 0
        for sb in range(4):
            if not (f >> sb) & 1:
                continue
            for u in range(8 * sb, 8 * sb + 8):
                wc = popc(U >> (u + 19)) + popc(e0 & lowmask(u + 1))
                if wc >= MIN_HITS:
                    g |= 1 << u
        g &= vm
        prev = ((g << 1) | (1 if opened else 0)) & M32
        rise = g & ~prev & M32
        fall = ~g & prev & vm & M32
        for u in range(32):
            if (rise >> u) & 1:
                start = 32 * w + u - 45
                runcnt = popc(U >> (u + 19)) + popc(e0 & lowmask(u + 1))
                accpos = u + 1
                opened = True
            elif (fall >> u) & 1:
                runcnt += popc(e0 & lowmask(u) & ~lowmask(accpos) & M32)
                out.append((start, 32 * w + u, runcnt))
                opened = False
        if opened:
            if w == wlast:
                ue = iend - 32 * w
                out.append((start, iend, runcnt + popc(e0 & lowmask(ue) & ~lowmask(accpos) & M32)))
                opened = False
            else:
                runcnt += popc(e0 & ~lowmask(accpos) & M32)
                accpos = 0
    if opened:
        out.append((start, 32 * (lastw + 1), runcnt))
    return [(s, s + pos, e - s, m) for s, e, m in out]


def equal_bases(t, q, s, pos, ln):
    return sum(1 for i in range(ln) if t[s + i] == q[s + pos + i])


@pytest.fixture(scope="module")
def O():
    return oracle.Oracle()


def test_model_matches_oracle_doone(O):
    rng = np.random.default_rng(77)
    cases = W.uniform_batch(6, seed=8) + [W.plain_pair(3)]
    t = W.random_bases(rng, 4096)
    cases.append((t.tobytes(), t.tobytes()))                      # identical: one long run
    cases.append((t.tobytes(), W.tandem_repeat(rng, 4096, 2, 3).tobytes()))
    for t, q in cases:
        offs = O.findtop(O.xcorr64(t, q, 8192), 1.8)
        extra = rng.integers(-4095, 4096, size=20)
        for i in list(offs[:40]) + [int(x) + 4096 for x in extra]:
            pos = int(i) - 4096
            got = model_doone(t, q, pos)
            want = O.doone(t, q, pos)
            assert [g[:3] for g in got] == [tuple(x) for x in want.tolist()], pos
            for s, qs, ln, m in got:
                assert m == equal_bases(t, q, s, pos, ln)


def model_doone_items(t, q, pos, icap=4096):
    """Pass 2 as the item kernel does it: every flagged 8-check block is an
    item (contiguous per diagonal, in block order); phase A gives each item
    its 8 exact window bits, phase B finds rises and falls from the previous
    item's last bit and takes a fall's run start from the same item or by
    looking back over the items before it.  Items are processed in
    sub-ranges of icap with the last item of one sub-range carried into the
    next.  Returns segments sorted by start (the kernel queues them unordered)."""
    T, Q = len(t), len(q)
    TW = max(T, Q) // 32 + 2
    tb0, tb1 = planes(t, TW + 2)
    qb0, qb1 = planes(q, TW + 8, pad=2)
    i0 = max(0, -pos)
    iend = min(T - 1, Q - pos)
    cfirst, clast = i0 + 46, iend - 1
    if clast < cfirst:
        return []

    def fs(lo, hi, sh):
        return ((hi << 32 | lo) >> sh) & M32

    def eword(w):
        if w < 0:
            return 0
        qo = 32 * w + pos + 64
        qw, sh = qo >> 5, qo & 31
        return ~((tb0[w] ^ fs(qb0[qw], qb0[qw + 1], sh)) | (tb1[w] ^ fs(qb1[qw], qb1[qw + 1], sh))) & M32

    def vmask(w):
        lo, hi = max(cfirst - 32 * w, 0), min(clast - 32 * w, 31)
        return (M32 >> (31 - hi)) & (M32 << lo) & M32

    wfirst, wlast = cfirst >> 5, clast >> 5
    flagged = set()
    for w in range(wfirst, wlast + 1):
        e2, e1, e0 = eword(w - 2), eword(w - 1), eword(w)
        U = (e1 << 32) | e2
        vm = vmask(w)
        for sb in range(4):
            a = 8 * sb + 19
            if popc(U >> a) + popc(e0 & lowmask(a - 11)) >= MIN_HITS and (vm >> (8 * sb)) & 0xFF:
                flagged.add(4 * (w - wfirst) + sb)
    blks = sorted(flagged)
    # phase A
    G = []
    for blk in blks:
        w, sb = wfirst + (blk >> 2), blk & 3
        e2, e1, e0 = eword(w - 2), eword(w - 1), eword(w)
        U = (e1 << 32) | e2
        g = 0
        for u in range(8):
            c = 8 * sb + u
            if popc(U >> (c + 19)) + popc(e0 & lowmask(c + 1)) >= MIN_HITS:
                g |= 1 << u
        G.append(g & (vmask(w) >> (8 * sb)) & 0xFF)

    def rise_of(i, pbit):
        return G[i] & ~(((G[i] << 1) | pbit) & 0xFF) & 0xFF

    segs = []
    carry = None   # (blk, G, open-run start) of the previous sub-range's last item
    for g0 in range(0, len(blks), icap):
        g1 = min(len(blks), g0 + icap)

        def pbit_of(i):
            if i > g0:
                return (G[i - 1] >> 7) if blks[i - 1] == blks[i] - 1 else 0
            if carry is not None and carry[0] == blks[i] - 1:
                return carry[1] >> 7
            return 0

        def run_start(i, u):
            """Check position where the run holding bit u-1 of item i began."""
            rb = rise_of(i, pbit_of(i)) & lowmask(u)
            while not rb:
                i -= 1
                if i < g0:
                    return carry[2]
                rb = rise_of(i, pbit_of(i))
            return 32 * (wfirst + (blks[i] >> 2)) + 8 * (blks[i] & 3) + rb.bit_length() - 1

        for i in range(g0, g1):
            blk, g = blks[i], G[i]
            w, sb = wfirst + (blk >> 2), blk & 3
            c0 = 32 * w + 8 * sb
            vm8 = (vmask(w) >> (8 * sb)) & 0xFF
            hi = min(clast - c0, 7)
            prev = ((g << 1) | pbit_of(i)) & 0xFF
            fall = ~g & prev & vm8 & 0xFF
            for u in range(8):
                if (fall >> u) & 1:
                    segs.append((run_start(i, u) - 45, c0 + u))
            if (g >> hi) & 1:
                if c0 + hi == clast:
                    segs.append((run_start(i, hi + 1) - 45, iend))
                elif blk + 1 not in flagged:
                    segs.append((run_start(i, 8) - 45, c0 + 8))
        last = g1 - 1
        carry = (blks[last], G[last], run_start(last, 8) if (G[last] >> 7) & 1 else -1)
    segs.sort()
    return [(s, s + pos, e - s, equal_bases(t, q, s, pos, e - s)) for s, e in segs]


@pytest.mark.parametrize("icap", [4096, 7, 1])
def test_item_model_matches_oracle_doone(O, icap):
    rng = np.random.default_rng(79)
    cases = W.uniform_batch(4, seed=10) + [W.plain_pair(5)]
    t = W.random_bases(rng, 4096)
    cases.append((t.tobytes(), t.tobytes()))
    cases.append((t.tobytes(), W.tandem_repeat(rng, 4096, 2, 3).tobytes()))
    for t, q in cases:
        offs = O.findtop(O.xcorr64(t, q, 8192), 1.8)
        extra = rng.integers(-4095, 4096, size=10)
        for i in list(offs[:20]) + [int(x) + 4096 for x in extra]:
            pos = int(i) - 4096
            got = model_doone_items(t, q, pos, icap)
            want = O.doone(t, q, pos)
            assert [g[:3] for g in got] == [tuple(x) for x in want.tolist()], (pos, icap)


def model_doone_words(t, q, pos, icap=4096):
    """Pass 2 with one item per marked word (its 4-bit block mask from the
    screen): phase A gives the item the exact bits of its marked blocks
    (unmarked blocks hold no passing check), phase B finds falls and closing
    ends against the previous word's bit 31, phase C takes each run start
    from the same word or by looking back over adjacent items.  Sub-ranges
    of icap items carry the last item into the next.  Returns segments sorted
    by start."""
    T, Q = len(t), len(q)
    TW = max(T, Q) // 32 + 2
    tb0, tb1 = planes(t, TW + 2)
    qb0, qb1 = planes(q, TW + 8, pad=2)
    i0 = max(0, -pos)
    iend = min(T - 1, Q - pos)
    cfirst, clast = i0 + 46, iend - 1
    if clast < cfirst:
        return []

    def fs(lo, hi, sh):
        return ((hi << 32 | lo) >> sh) & M32

    def eword(w):
        if w < 0:
            return 0
        qo = 32 * w + pos + 64
        qw, sh = qo >> 5, qo & 31
        return ~((tb0[w] ^ fs(qb0[qw], qb0[qw + 1], sh)) | (tb1[w] ^ fs(qb1[qw], qb1[qw + 1], sh))) & M32

    def vmask(w):
        lo, hi = max(cfirst - 32 * w, 0), min(clast - 32 * w, 31)
        return (M32 >> (31 - hi)) & (M32 << lo) & M32

    wfirst, wlast = cfirst >> 5, clast >> 5
    marked = {}
    for w in range(wfirst, wlast + 1):
        e2, e1, e0 = eword(w - 2), eword(w - 1), eword(w)
        U = (e1 << 32) | e2
        vm = vmask(w)
        f = 0
        for sb in range(4):
            a = 8 * sb + 19
            if popc(U >> a) + popc(e0 & lowmask(a - 11)) >= MIN_HITS and (vm >> (8 * sb)) & 0xFF:
                f |= 1 << sb
        if f:
            marked[w] = f
    words = sorted(marked)
    # phase A
    G = []
    for w in words:
        e2, e1, e0 = eword(w - 2), eword(w - 1), eword(w)
        U = (e1 << 32) | e2
        g = 0
        for sb in range(4):
            if not (marked[w] >> sb) & 1:
                continue
            for u in range(8 * sb, 8 * sb + 8):
                if popc(U >> (u + 19)) + popc(e0 & lowmask(u + 1)) >= MIN_HITS:
                    g |= 1 << u
        G.append(g & vmask(w))

    segs = []
    carry = None   # (word, G, open-run start) of the previous sub-range's last item
    for g0 in range(0, len(words), icap):
        g1 = min(len(words), g0 + icap)

        def pbit_of(i):
            if i > g0:
                return (G[i - 1] >> 31) if words[i - 1] == words[i] - 1 else 0
            if carry is not None and carry[0] == words[i] - 1:
                return carry[1] >> 31
            return 0

        def rise_of(i):
            return G[i] & ~(((G[i] << 1) | pbit_of(i)) & M32) & M32

        def run_start(i, u):
            rb = rise_of(i) & lowmask(u)
            while not rb:
                i -= 1
                if i < g0:
                    return carry[2]
                rb = rise_of(i)
            return 32 * words[i] + rb.bit_length() - 1

        for i in range(g0, g1):
            w, g = words[i], G[i]
            vm = vmask(w)
            hi = min(clast - 32 * w, 31)
            fall = ~g & (((g << 1) | pbit_of(i)) & M32) & vm & M32
            for u in range(32):
                if (fall >> u) & 1:
                    segs.append((run_start(i, u) - 45, 32 * w + u))
            if (g >> hi) & 1:
                if 32 * w + hi == clast:
                    segs.append((run_start(i, hi + 1) - 45, iend))
                elif w + 1 not in marked:
                    segs.append((run_start(i, 32) - 45, 32 * w + 32))
        last = g1 - 1
        carry = (words[last], G[last], run_start(last, 32) if (G[last] >> 31) & 1 else -1)
    segs.sort()
    return [(s, s + pos, e - s, equal_bases(t, q, s, pos, e - s)) for s, e in segs]


@pytest.mark.parametrize("icap", [4096, 5, 1])
def test_word_model_matches_oracle_doone(O, icap):
    rng = np.random.default_rng(80)
    cases = W.uniform_batch(4, seed=13) + [W.plain_pair(6)]
    t = W.random_bases(rng, 4096)
    cases.append((t.tobytes(), t.tobytes()))
    cases.append((t.tobytes(), W.tandem_repeat(rng, 4096, 2, 3).tobytes()))
    for t, q in cases:
        offs = O.findtop(O.xcorr64(t, q, 8192), 1.8)
        extra = rng.integers(-4095, 4096, size=10)
        for i in list(offs[:20]) + [int(x) + 4096 for x in extra]:
            pos = int(i) - 4096
            got = model_doone_words(t, q, pos, icap)
            want = O.doone(t, q, pos)
            assert [g[:3] for g in got] == [tuple(x) for x in want.tolist()], (pos, icap)


# ---------------------------------------------------------------------------
# Word screen on 4-check blocks and byte-lane exact bits (the kernel's current
# form).  The arithmetic below is the kernel's, on 32-bit words.
# ---------------------------------------------------------------------------
def nib_popc(x):
    """Per-nibble popcount of a 32-bit word."""
    x = (x - ((x >> 1) & 0x55555555)) & M32
    return ((x & 0x33333333) + ((x >> 2) & 0x33333333)) & M32


def screen_word(e2, e1, e0):
    """True when some 4-check block of the word (checks 4b..4b+3, b < 8) has
    >= 19 equal bases in its 49-position span: the block count c(b) = c(0) +
    sum_{k<b} (entering nibble k - leaving nibble k), formed for the eight
    blocks at once in byte lanes (even blocks 2j, odd blocks 2j+1)."""
    U = (e1 << 32) | e2
    pl = nib_popc((U >> 19) & M32)   # nibble k: span bits leaving between blocks k and k+1
    pe = nib_popc(e0 >> 4)           # nibble k: bits entering
    de = ((pe & 0x0F0F0F0F) + 0x04040404 - (pl & 0x0F0F0F0F)) & M32          # 4 + d(2j)
    do = (((pe >> 4) & 0x0F0F0F0F) + 0x04040404 - ((pl >> 4) & 0x0F0F0F0F)) & M32   # 4 + d(2j+1)
    sx = (((de + do) & M32) * 0x01010100) & M32                                # sum_{i<j} (8 + d(2i) + d(2i+1))
    c0 = popc(U >> 19) + popc(e0 & 0xF)
    x = (sx + (c0 + 128 - MIN_HITS) * 0x01010101 - 0x18100800) & M32           # 128 - 19 + c(2j)
    x2 = (x + de - 0x04040404) & M32                                           # 128 - 19 + c(2j+1)
    return ((x | x2) & 0x80808080) != 0


def exact_word(e2, e1, e0):
    """Bit u set when check u's window [u-45, u] (in the word's frame) holds
    >= 19 equal bases: four byte lanes (u = 8j + s) step s = 0..7 together."""
    U = (e1 << 32) | e2
    w = 0
    for j in range(4):
        u = 8 * j
        w |= (popc(U >> (u + 19)) + popc(e0 & lowmask(u + 1))) << (8 * j)
    lv = (U >> 19) & M32   # bit 8j+s: the position leaving after check 8j+s
    en = e0 >> 1           # bit 8j+s: the position entering at check 8j+s+1
    g = 0
    for s in range(8):
        if s:
            w = (w + ((en >> (s - 1)) & 0x01010101) - ((lv >> (s - 1)) & 0x01010101)) & M32
        g |= (((w + (128 - MIN_HITS) * 0x01010101) >> 7) & 0x01010101) << s
    return g


def test_word_screen_and_exact_bits_bruteforce():
    rng = np.random.default_rng(81)
    for it in range(4000):
        dens = rng.choice([0.25, 0.4, 0.55, 0.9])
        e = [int(sum(int(b) << k for k, b in enumerate(rng.random(32) < dens))) for _ in range(3)]
        e2, e1, e0 = e
        V = e2 | (e1 << 32) | (e0 << 64)
        win = [popc((V >> (u + 19)) & ((1 << 46) - 1)) for u in range(32)]
        want_g = sum(1 << u for u in range(32) if win[u] >= MIN_HITS)
        assert exact_word(e2, e1, e0) == want_g
        spans = [popc((V >> (4 * b + 19)) & ((1 << 49) - 1)) for b in range(8)]
        assert screen_word(e2, e1, e0) == any(s >= MIN_HITS for s in spans)
        # necessary condition: a word with a passing check is marked
        assert not want_g or screen_word(e2, e1, e0)


def model_doone_words4(t, q, pos, icap=4096):
    """Pass 1 marks words (screen_word); phase A gives each marked word its
    exact bits (exact_word); phases B and C as in model_doone_words, a run
    open at a word's last check closing when the next word is unmarked."""
    T, Q = len(t), len(q)
    TW = max(T, Q) // 32 + 2
    tb0, tb1 = planes(t, TW + 2)
    qb0, qb1 = planes(q, TW + 8, pad=2)
    i0 = max(0, -pos)
    iend = min(T - 1, Q - pos)
    cfirst, clast = i0 + 46, iend - 1
    if clast < cfirst:
        return []

    def fs(lo, hi, sh):
        return ((hi << 32 | lo) >> sh) & M32

    def eword(w):
        if w < 0:
            return 0
        qo = 32 * w + pos + 64
        qw, sh = qo >> 5, qo & 31
        return ~((tb0[w] ^ fs(qb0[qw], qb0[qw + 1], sh)) | (tb1[w] ^ fs(qb1[qw], qb1[qw + 1], sh))) & M32

    def vmask(w):
        lo, hi = max(cfirst - 32 * w, 0), min(clast - 32 * w, 31)
        return (M32 >> (31 - hi)) & (M32 << lo) & M32

    wfirst, wlast = cfirst >> 5, clast >> 5
    words = [w for w in range(wfirst, wlast + 1) if screen_word(eword(w - 2), eword(w - 1), eword(w))]
    marked = set(words)
    G = [exact_word(eword(w - 2), eword(w - 1), eword(w)) & vmask(w) for w in words]
    # the kernel's bit of the check before each word, from the word's own
    # equality words (window bits 18..63 of e2:e1), equals bit 31 of the
    # previous word's exact bits when that word is marked, else 0
    for k, w in enumerate(words):
        U = (eword(w - 1) << 32) | eword(w - 2)
        pb = int(32 * w - 1 >= cfirst and popc(U >> 18) >= MIN_HITS)
        prev = (G[k - 1] >> 31) if k > 0 and words[k - 1] == w - 1 else 0
        assert pb == prev, (pos, w)

    segs = []
    carry = None
    for g0 in range(0, len(words), icap):
        g1 = min(len(words), g0 + icap)

        def pbit_of(i):
            if i > g0:
                return (G[i - 1] >> 31) if words[i - 1] == words[i] - 1 else 0
            if carry is not None and carry[0] == words[i] - 1:
                return carry[1] >> 31
            return 0

        def rise_of(i):
            return G[i] & ~(((G[i] << 1) | pbit_of(i)) & M32) & M32

        def run_start(i, u):
            rb = rise_of(i) & lowmask(u)
            while not rb:
                i -= 1
                if i < g0:
                    return carry[2]
                rb = rise_of(i)
            return 32 * words[i] + rb.bit_length() - 1

        for i in range(g0, g1):
            w, g = words[i], G[i]
            vm = vmask(w)
            hi = min(clast - 32 * w, 31)
            fall = ~g & (((g << 1) | pbit_of(i)) & M32) & vm & M32
            for u in range(32):
                if (fall >> u) & 1:
                    segs.append((run_start(i, u) - 45, 32 * w + u))
            if (g >> hi) & 1:
                if 32 * w + hi == clast:
                    segs.append((run_start(i, hi + 1) - 45, iend))
                elif w + 1 not in marked:
                    segs.append((run_start(i, 32) - 45, 32 * w + 32))
        last = g1 - 1
        carry = (words[last], G[last], run_start(last, 32) if (G[last] >> 31) & 1 else -1)
    segs.sort()
    return [(s, s + pos, e - s, equal_bases(t, q, s, pos, e - s)) for s, e in segs]


@pytest.mark.parametrize("icap", [4096, 5, 1])
def test_word4_model_matches_oracle_doone(O, icap):
    rng = np.random.default_rng(82)
    cases = W.uniform_batch(4, seed=17) + [W.plain_pair(7)]
    t = W.random_bases(rng, 4096)
    cases.append((t.tobytes(), t.tobytes()))
    cases.append((t.tobytes(), W.tandem_repeat(rng, 4096, 2, 3).tobytes()))
    cases.append((t[:1000].tobytes(), t[:999].tobytes()))
    for t, q in cases:
        offs = O.findtop(O.xcorr64(t, q, 8192), 1.8)
        extra = rng.integers(-len(t) + 1, len(q), size=10)
        for i in list(offs[:20]) + [int(x) + 4096 for x in extra]:
            pos = int(i) - 4096
            got = model_doone_words4(t, q, pos, icap)
            want = O.doone(t, q, pos)
            assert [g[:3] for g in got] == [tuple(x) for x in want.tolist()], (pos, icap)


# ---------------------------------------------------------------------------
# Bitplanes from 16-byte pieces and reverse-complement planes (build_planes
# and the strand-1 construction in scan_kernel), 32-bit arithmetic as there.
# ---------------------------------------------------------------------------
def build_planes_model(buf, ln, nw):
    """buf: the chunk bytes padded to 16 (bytes past ln are garbage)."""
    p0 = [0] * nw
    p1 = [0] * nw
    half = {}
    for c in range(2 * nw):
        m0 = m1 = 0
        if 16 * c < ln:
            for k in range(4):
                x = int.from_bytes(buf[16 * c + 4 * k:16 * c + 4 * k + 4], "little")
                cd = ((x >> 1) ^ (x >> 2)) & 0x03030303
                m0 |= ((((cd & 0x01010101) * 0x10204080) & M32) >> 28) << (4 * k)
                m1 |= (((((cd >> 1) & 0x01010101) * 0x10204080) & M32) >> 28) << (4 * k)
            valid = ln - 16 * c
            if valid < 16:
                m0 &= (1 << valid) - 1
                m1 &= (1 << valid) - 1
        half[c] = (m0, m1)
    for j in range(nw):
        (a0, a1), (b0, b1) = half[2 * j], half[2 * j + 1]
        p0[j] = a0 | (b0 << 16)
        p1[j] = a1 | (b1 << 16)
    return p0, p1


def brev32(x):
    return int("{:032b}".format(x)[::-1], 2)


def rc_planes_model(f0, f1, Q, nw):
    r0, r1 = [0] * nw, [0] * nw
    for w in range(nw):
        lim = Q - 32 * w
        if lim <= 0:
            continue
        s0 = lim - 32
        if s0 >= 0:
            fw, sh = s0 >> 5, s0 & 31
            g0 = ((f0[fw + 1] << 32 | f0[fw]) >> sh) & M32
            g1 = ((f1[fw + 1] << 32 | f1[fw]) >> sh) & M32
        else:
            g0 = (f0[0] << -s0) & M32
            g1 = (f1[0] << -s0) & M32
        m = lowmask(lim)
        r0[w] = ~brev32(g0) & m & M32
        r1[w] = ~brev32(g1) & m & M32
    return r0, r1


@pytest.mark.parametrize("n", [0, 1, 15, 16, 17, 31, 32, 33, 1000, 4095, 4096])
def test_plane_build_and_reverse_complement(O, n):
    rng = np.random.default_rng(90 + n)
    seq = W.random_bases(rng, n).tobytes()
    pad = (n + 15) // 16 * 16 + 16
    buf = seq + bytes(rng.integers(0, 256, pad - n, dtype=np.uint8))   # garbage past the chunk
    nw = 4096 // 32 + 2
    want0, want1 = planes(seq, nw)
    got0, got1 = build_planes_model(buf, n, nw)
    assert got0 == want0[:nw] and got1 == want1[:nw]
    rw0, rw1 = planes(O.rc(seq), nw)
    r0, r1 = rc_planes_model(got0, got1, n, nw)
    assert r0 == rw0[:nw] and r1 == rw1[:nw]
