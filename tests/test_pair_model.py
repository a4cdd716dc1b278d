"""CPU model of corr_pair_kernel's premise (csrc/xc_corr.cu): for an
A/C/G/T pair whose query length is a multiple of the entropy window (or below
1024), the reverse-complemented query's signal in channel c is the forward
query's signal in the complement channel, reversed in time, bit for bit; so
its spectrum is W_L^((Q-1)k) conj(Q_comp(c)(k)) and the reverse strand's
product sum is W_L^((Q-1)k) conj(sum_c T_c Q_comp(c)).  Signals come from the
oracle's CCSignal restatement (CrossCorr.cc:35-123)."""
import numpy as np
import pytest

import oracle
from satsuma2_gb300 import workloads as W

COMP = [3, 2, 1, 0]   # A<->T, C<->G in channel order A, C, G, T
L = 8192


@pytest.fixture(scope="module")
def O():
    return oracle.Oracle()


def pairs():
    rng = np.random.default_rng(61)
    out = []
    for qlen in (4096, 2048 + 16 * 37, 800, 1024):
        t = W.random_bases(rng, 4096, gc=0.45).tobytes()
        q = W.random_bases(rng, qlen, gc=0.55).tobytes()
        out.append((t, q))
    t, q = W.plain_pair(8)
    out.append((t, q))
    return out


@pytest.mark.parametrize("k", range(5))
def test_reverse_signal_is_reversed_complement_channel(O, k):
    t, q = pairs()[k]
    Q = len(q)
    assert Q < 1024 or Q % (L // 512) == 0
    sq = O.signal(q, L)
    sr = O.signal(O.rc(q), L)
    for c in range(4):
        assert np.array_equal(sr[c, :Q], sq[COMP[c], :Q][::-1]), c
        assert not np.any(sr[c, Q:])


def test_ragged_query_breaks_the_identity(O):
    """A query of >= 1024 bases that is not a multiple of the 16-base window
    puts the reverse windows across forward windows: such pairs go to the
    per-strand kernel."""
    rng = np.random.default_rng(62)
    q = W.random_bases(rng, 4096 - 7).tobytes()
    sq = O.signal(q, L)
    sr = O.signal(O.rc(q), L)
    Q = len(q)
    assert any(not np.array_equal(sr[c, :Q], sq[COMP[c], :Q][::-1]) for c in range(4))


@pytest.mark.parametrize("k", range(5))
def test_reverse_product_sum_from_forward_spectra(O, k):
    t, q = pairs()[k]
    Q = len(q)
    st = O.signal(t, L).astype(np.float64)
    sq = O.signal(q, L).astype(np.float64)
    sr = O.signal(O.rc(q), L).astype(np.float64)
    T = np.fft.rfft(st, axis=1)                 # bins 0..L/2
    Qf = np.fft.rfft(sq, axis=1)
    Qr = np.fft.rfft(sr, axis=1)
    direct = np.sum(np.conj(T) * Qr, axis=0)
    kk = np.arange(L // 2 + 1)
    w = np.exp(-2j * np.pi * (((Q - 1) * kk) % L) / L)
    R = np.sum(T * Qf[COMP], axis=0)
    shared = w * np.conj(R)
    scale = np.abs(direct).max()
    assert np.abs(direct - shared).max() <= 1e-9 * scale
