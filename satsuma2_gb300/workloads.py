"""Seeded synthetic chunk-pair workloads (numpy; default seed 42).

No public dataset exists for this path, so every workload is generated from a
seed and printed with it.  Shapes follow the five benchmark configurations of
the cross-correlation path:

* ``plain_pair``    -- one 4096x4096 pair, query = 85% identity copy of
                       target[500:3500] with a 1-5 bp indel per 500 bp, flanked
                       by random bases (FFT length 8192, cutoff 1.8).
* ``uniform_batch`` -- 4096 pairs of 4096x4096; homolog length U[200,3500],
                       identity U[70,95]%; 25% without homology, 25% with the
                       homolog reverse-complemented.
* ``uneven_batch``  -- 20000 pairs with tLen, qLen ~ U[300,4096]; GC U[35,60]%;
                       10% carry tandem repeats (period 2-6, 50-400 bp) on
                       both sides; FFT length nextpow2(2*max(tLen,qLen)).
* ``serving_genomes`` -- a target genome (GC 41%) and an 80% identity query
                       derived from it with inversions, segmental duplications
                       and 10% novel insertions, chunked as the slave does;
                       ``grid_search_blocks`` orders its 24x24 chunk blocks as
                       a grid search would submit them.
* ``large_batch``   -- 16384x16384 pairs (FFT length 32768), 30% of the
                       sequence low-complexity microsatellites, GC U[25,70]%.
"""
import numpy as np

ACGT = np.frombuffer(b"ACGT", np.uint8)
_COMP = np.zeros(256, np.uint8)
for _a, _b in zip(b"ACGT", b"TGCA"):
    _COMP[_a] = _b


def random_bases(rng, n, gc=0.5):
    """n i.i.d. bases with the given G+C fraction."""
    p = np.array([(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2])
    return ACGT[rng.choice(4, size=n, p=p)]


def revcomp(s):
    return _COMP[s[::-1]]


def mutate(rng, s, identity, indel_every=500, indel_max=5):
    """Uniform substitutions at rate 1-identity plus one indel of 1..indel_max bp
    per indel_every bp (insertions and deletions equally likely)."""
    s = s.copy()
    n = len(s)
    sub = rng.random(n) > identity
    if sub.any():
        shift = rng.integers(1, 4, size=int(sub.sum()))
        idx = np.searchsorted(ACGT, s[sub])
        idx = np.clip(idx, 0, 3)
        s[sub] = ACGT[(idx + shift) % 4]
    if indel_every and n > indel_every:
        out = []
        prev = 0
        for k in range(n // indel_every):
            p = int(rng.integers(k * indel_every, (k + 1) * indel_every))
            ln = int(rng.integers(1, indel_max + 1))
            out.append(s[prev:p])
            if rng.random() < 0.5:
                out.append(random_bases(rng, ln))
                prev = p
            else:
                prev = min(n, p + ln)
        out.append(s[prev:])
        s = np.concatenate(out)
    return s


def tandem_repeat(rng, length, period_lo, period_hi):
    unit = random_bases(rng, int(rng.integers(period_lo, period_hi + 1)))
    reps = length // len(unit) + 1
    return np.tile(unit, reps)[:length]


def _embed(rng, flank_len_total, core, gc=0.5):
    """core placed at a random position inside random flanks to the total length."""
    if len(core) >= flank_len_total:
        return core[:flank_len_total]
    left = int(rng.integers(0, flank_len_total - len(core) + 1))
    right = flank_len_total - len(core) - left
    return np.concatenate([random_bases(rng, left, gc), core, random_bases(rng, right, gc)])


def plain_pair(seed=42, length=4096):
    """One 4096x4096 pair: the query holds an 85%-identity copy of target[500:3500]."""
    rng = np.random.default_rng(seed)
    t = random_bases(rng, length)
    core = mutate(rng, t[500:3500], 0.85)
    q = _embed(rng, length, core)
    return t.tobytes(), q.tobytes()


def uniform_batch(n=4096, seed=42, length=4096):
    """n pairs of length x length (defaults: 4096 pairs of 4096 bp)."""
    rng = np.random.default_rng(seed)
    pairs = []
    for i in range(n):
        t = random_bases(rng, length)
        kind = rng.random()
        if kind < 0.25:
            q = random_bases(rng, length)
        else:
            hl = int(rng.integers(200, 3501))
            hl = min(hl, length)
            st = int(rng.integers(0, length - hl + 1))
            core = mutate(rng, t[st:st + hl], float(rng.uniform(0.70, 0.95)))
            if kind >= 0.75:
                core = revcomp(core)
            q = _embed(rng, length, core)
        pairs.append((t.tobytes(), q.tobytes()))
    return pairs


def next_pow2(x):
    b = 1
    while b < x:
        b *= 2
    return b


def uneven_fft_len(tlen, qlen):
    """Bucket rule nextpow2(2*max(tLen,qLen)) (CCSignal::SetSize, CrossCorr.cc:155-177)."""
    return max(1024, next_pow2(2 * max(tlen, qlen)))


def uneven_batch(n=20000, seed=42):
    """n pairs with independent lengths U[300,4096], GC U[35,60]%, 10% tandem repeats."""
    rng = np.random.default_rng(seed)
    pairs = []
    for i in range(n):
        tl = int(rng.integers(300, 4097))
        ql = int(rng.integers(300, 4097))
        gc = float(rng.uniform(0.35, 0.60))
        t = random_bases(rng, tl, gc)
        if rng.random() < 0.5:
            hl = int(rng.integers(min(100, tl, ql), min(tl, ql) + 1))
            st = int(rng.integers(0, tl - hl + 1))
            core = mutate(rng, t[st:st + hl], float(rng.uniform(0.70, 0.95)))
            if rng.random() < 0.3:
                core = revcomp(core)
            q = _embed(rng, ql, core[:ql], gc)
        else:
            q = random_bases(rng, ql, gc)
        if rng.random() < 0.10:
            rl = int(rng.integers(50, 401))
            rep = tandem_repeat(rng, rl, 2, 6)
            for which in (0, 1):
                s = t if which == 0 else q
                rl2 = min(rl, len(s))
                p = int(rng.integers(0, len(s) - rl2 + 1))
                s = s.copy()
                s[p:p + rl2] = mutate(rng, rep[:rl2], 0.95, indel_every=0)
                if which == 0:
                    t = s
                else:
                    q = s
        pairs.append((t.tobytes(), q.tobytes()))
    return pairs


def large_batch(n=2000, seed=42, length=16384):
    """n pairs of 16384x16384 with 30% microsatellite sequence and GC U[25,70]%."""
    rng = np.random.default_rng(seed)
    pairs = []

    def lowcomplex(s):
        s = s.copy()
        target = int(0.30 * len(s))
        done = 0
        while done < target:
            rl = int(rng.integers(20, 400))
            rl = min(rl, target - done, len(s))
            p = int(rng.integers(0, len(s) - rl + 1))
            s[p:p + rl] = tandem_repeat(rng, rl, 1, 4)
            done += rl
        return s

    for i in range(n):
        gc = float(rng.uniform(0.25, 0.70))
        t = lowcomplex(random_bases(rng, length, gc))
        if rng.random() < 0.6:
            hl = int(rng.integers(500, length))
            st = int(rng.integers(0, length - hl + 1))
            core = mutate(rng, t[st:st + hl], float(rng.uniform(0.70, 0.95)))
            if rng.random() < 0.3:
                core = revcomp(core)
            q = _embed(rng, length, core, gc)
        else:
            q = random_bases(rng, length, gc)
        q = lowcomplex(q)
        pairs.append((t.tobytes(), q.tobytes()))
    return pairs


def serving_genomes(seed=42, size=20_000_000, n_inv=30, inv_range=(10_000, 200_000),
                    n_dup=20, dup_range=(5_000, 50_000), novel_frac=0.10, identity=0.80, with_map=False):
    """Target genome (GC 41%) and a derived query: 80% identity, inversions,
    segmental duplications and novel insertions (about novel_frac of the length).

    with_map: also returns (src, rev), for every query base the target
    position it derives from (-1 for novel bases) and whether it is
    reverse-complemented."""
    rng = np.random.default_rng(seed)
    target = random_bases(rng, size, 0.41)
    q = target.copy()
    src = np.arange(size, dtype=np.int32) if with_map else None
    rev = np.zeros(size, bool) if with_map else None
    for _ in range(n_inv):
        ln = int(rng.integers(*inv_range))
        ln = min(ln, size // 4)
        p = int(rng.integers(0, size - ln))
        q[p:p + ln] = revcomp(q[p:p + ln])
        if with_map:
            src[p:p + ln] = src[p:p + ln][::-1].copy()
            rev[p:p + ln] = ~rev[p:p + ln][::-1]
    pieces, spieces, rpieces = [q], [src], [rev]
    for _ in range(n_dup):
        ln = int(rng.integers(*dup_range))
        ln = min(ln, size // 8)
        p = int(rng.integers(0, size - ln))
        pieces.append(q[p:p + ln].copy())
        if with_map:
            spieces.append(src[p:p + ln].copy())
            rpieces.append(rev[p:p + ln].copy())
    q = np.concatenate(pieces)
    if with_map:
        src = np.concatenate(spieces)
        rev = np.concatenate(rpieces)
    sub = rng.random(len(q)) > identity
    shift = rng.integers(1, 4, size=int(sub.sum()))
    idx = np.clip(np.searchsorted(ACGT, q[sub]), 0, 3)
    q[sub] = ACGT[(idx + shift) % 4]
    n_ins = 200
    total_ins = int(novel_frac * size)
    cuts = np.sort(rng.integers(0, len(q), size=n_ins))
    lens = rng.multinomial(total_ins, np.ones(n_ins) / n_ins)
    out, so, ro, prev = [], [], [], 0
    for c, ln in zip(cuts, lens):
        out.append(q[prev:c])
        out.append(random_bases(rng, int(ln), 0.41))
        if with_map:
            so += [src[prev:c], np.full(int(ln), -1, np.int32)]
            ro += [rev[prev:c], np.zeros(int(ln), bool)]
        prev = c
    out.append(q[prev:])
    query = np.concatenate(out)
    if with_map:
        so.append(src[prev:])
        ro.append(rev[prev:])
        return target.tobytes(), query.tobytes(), (np.concatenate(so), np.concatenate(ro))
    return target.tobytes(), query.tobytes()


def grid_search_blocks(src, n_tchunks, n_qchunks, t_step=3072, q_step=4096, block=24, seed_every=8,
                       per_round=64, probes=4):
    """Blocks of block x block chunk pairs in the order a grid search over the
    chunk matrix would submit them (GridSearch::CollectTargets,
    analysis/GridSearch.cc:354-411): blocks holding homology (found from the
    query-to-target map src, probes positions per query chunk) are the hits;
    every seed_every-th hit in query order seeds the search; each round then
    takes up to per_round unknown blocks next to processed hits, ordered by
    the number of processed hits around them (descending), then by target and
    query block, as CollectTargets sorts GridTarget.  Returns [(tf, tt, qf,
    qt)] inclusive chunk ranges, query blocks of one target block row-major
    in submission order."""
    ntb = (n_tchunks + block - 1) // block
    nqb = (n_qchunks + block - 1) // block
    hits = set()
    for j in range(n_qchunks):
        for k in range(probes):
            pos = j * q_step + (k * q_step) // probes + q_step // (2 * probes)
            if pos >= len(src) or src[pos] < 0:
                continue
            i = min(int(src[pos]) // t_step, n_tchunks - 1)
            hits.add((i // block, j // block))
    known = {}
    order = []
    seeds = sorted(hits, key=lambda b: (b[1], b[0]))[::seed_every]
    count = {}

    def take(b):
        known[b] = True
        order.append(b)
        if b in hits:
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    nb = (b[0] + dx, b[1] + dy)
                    if (dx or dy) and 0 <= nb[0] < ntb and 0 <= nb[1] < nqb and nb not in known:
                        count[nb] = count.get(nb, 0) + 1

    for b in seeds:
        take(b)
    while True:
        cand = sorted((b for b in count if b not in known), key=lambda b: (-count[b], b[0], b[1]))[:per_round]
        if not cand:
            break
        for b in cand:
            take(b)
    return [(x * block, min((x + 1) * block, n_tchunks) - 1, y * block, min((y + 1) * block, n_qchunks) - 1)
            for x, y in order]


def chunk_starts(length, size, overlap):
    """ChunkManager::ChunkItSelect (SeqChunk.cc:72-165) for one sequence:
    (start, end) of every chunk; sequences under 6 bp give none."""
    if length < 6:
        return []
    step = size - overlap
    n = 1 + length // step
    out = []
    for j in range(n):
        st = max(0, j * step)
        en = min((j + 1) * step + overlap, length)
        out.append((st, en))
    return out
