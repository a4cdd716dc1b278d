"""CPU model of the correlation kernel's transform layout (xc_device.cuh,
xc_corr.cu): the in-place mixed-radix passes, the digit-reversed bin position
(posof) and the shared-memory swizzle, restated in numpy.

* the passes applied in the kernel's order compute the DFT (forward, natural
  order in, posof order out) and its unnormalised inverse;
* under the swizzle, the transform passes touch 16 distinct 8-byte slots per
  half-warp (no bank conflicts) for N >= 1024, and the spectrum phases at most
  two-way (one borrow in a partner-bin sequence); the plain digit-reversed
  layout had 16-way conflicts there.
"""
import numpy as np
import pytest

PLANS = {9: (3, 3, 3), 10: (4, 4, 2), 11: (4, 4, 3), 12: (4, 4, 4), 13: (4, 4, 4, 1), 14: (4, 4, 4, 2)}


def swz(p):
    p = np.asarray(p)
    return p ^ (((p >> 4) ^ (p >> 8) ^ (p >> 12)) & 15)


def posof(k, log2n, plans=PLANS):
    p, off, used = 0, 0, 0
    for lr in plans[log2n]:
        used += lr
        p |= ((k >> off) & ((1 << lr) - 1)) << (log2n - used)
        off += lr
    return p


def passes(log2n, plans=PLANS):
    n = 1 << log2n
    out, span = [], n
    for lr in plans[log2n]:
        out.append((1 << lr, span))
        span >>= lr
    return out


def run_pass(buf, n, R, S, inverse):
    d = S // R
    b = np.arange(n // R)
    j = b & (d - 1)
    base = (b - j) * R + j
    idx = base[:, None] + d * np.arange(R)[None, :]
    x = buf[idx]
    rr = np.arange(R)
    W = np.exp((1 if inverse else -1) * 2j * np.pi * np.outer(rr, rr) / R)
    tw = np.exp(-2j * np.pi * (j[:, None] * rr[None, :]) * (n // S) / n)
    if not inverse:
        x = x @ W.T
        x = x * tw
    else:
        x = x * np.conj(tw)
        x = x @ W.T
    buf[idx] = x


@pytest.mark.parametrize("log2n", sorted(PLANS))
def test_passes_compute_dft(log2n):
    n = 1 << log2n
    rng = np.random.default_rng(log2n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    buf = x.copy()
    for R, S in passes(log2n):
        run_pass(buf, n, R, S, False)
    k = np.arange(n)
    pos = np.array([posof(int(v), log2n) for v in k])
    assert sorted(pos.tolist()) == list(range(n))
    assert np.allclose(buf[pos], np.fft.fft(x), atol=1e-9 * n)
    for R, S in reversed(passes(log2n)):
        run_pass(buf, n, R, S, True)
    assert np.allclose(buf / n, x, atol=1e-9)


def worst_multiplicity(addr_rows):
    """addr_rows: [half-warp][16] element indices -> worst slot multiplicity."""
    worst = 1
    for row in addr_rows:
        slots = swz(np.asarray(row)) & 15
        worst = max(worst, int(np.bincount(slots, minlength=16).max()))
    return worst


def halfwarps(items):
    items = list(items)
    return [items[i:i + 16] for i in range(0, len(items) - len(items) % 16, 16)]


@pytest.mark.parametrize("log2n", sorted(PLANS))
def test_fft_passes_conflict_free(log2n):
    n = 1 << log2n
    for R, S in passes(log2n):
        d = S // R
        b = np.arange(n // R)
        j = b & (d - 1)
        base = (b - j) * R + j
        for r in range(R):
            assert worst_multiplicity(halfwarps(base + r * d)) <= (1 if log2n >= 10 else 2), (R, S, r)


@pytest.mark.parametrize("log2n", sorted(PLANS))
def test_spectrum_phases_conflict_free(log2n):
    n = 1 << log2n
    m_even = np.arange(n // 2 + 1)
    m_odd = np.arange(n // 2)
    pos = np.vectorize(lambda k: posof(int(k), log2n))
    lim = 2 if log2n >= 10 else 3
    # product phase: A at posof(m), B at posof(partner)
    assert worst_multiplicity(halfwarps(pos(m_even))) <= lim
    assert worst_multiplicity(halfwarps(pos((n - m_even) & (n - 1)))) <= lim
    assert worst_multiplicity(halfwarps(pos(m_odd))) <= lim
    assert worst_multiplicity(halfwarps(pos(n - 1 - m_odd))) <= lim
    # inverse preparation writes Z(k), Z(N-k)
    k = np.arange(1, n // 2)
    assert worst_multiplicity(halfwarps(pos(k))) <= lim
    assert worst_multiplicity(halfwarps(pos(n - k))) <= lim
    # signal construction and FindTop read natural order
    assert worst_multiplicity(halfwarps(np.arange(n))) == 1

