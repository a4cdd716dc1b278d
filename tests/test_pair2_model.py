"""CPU model of corr_pair2_kernel's arithmetic (csrc/xc_corr.cu), in FP64
numpy: the per-bin step that forms the channel sums from the packed spectra
without separating the channels, the factors of two it leaves in, and the
reverse strand's sum through i conj(x + iy) = y + ix.

For each channel pair (A, T) then (C, G): z = t_c0 + i t_c1 and
w = q_c0 + i q_c1 as their N-point even-bin transforms Zt, Zq and odd-bin
transforms (of z W_L^n); per bin, with A = Zt(m), B = Zt(N-m), C = Zq(m),
D = Zq(N-m):
    F' += conj(A) C + B conj(D)          (= 2 sum_c conj(T_c) Q_c)
    R' += A C - conj(B D)                (= 2i (T_c0 Q_c1 + T_c1 Q_c0))
bin 0 by the same formula (B = A, D = C: the product of real values), bins
N-1 and N target-only.  The sums are checked against the channel-separated
form the reference computes (CrossCorr.cc:477-492), and the whole strand --
Hermitian pack without its halves, N-point inverse, scale 1/(4N) -- against
the direct FP64 correlation, for both strands.  Signals come from the
oracle's CCSignal restatement."""
import numpy as np
import pytest

import oracle
from satsuma2_gb300 import workloads as W

COMP = [3, 2, 1, 0]   # A<->T, C<->G in channel order A, C, G, T
L = 8192
N = L // 2


@pytest.fixture(scope="module")
def O():
    return oracle.Oracle()


def pairs():
    rng = np.random.default_rng(81)
    out = [W.plain_pair(9), W.uniform_batch(3, seed=14)[2]]
    t = W.random_bases(rng, 4096).tobytes()
    out.append((t, W.random_bases(rng, 2048 + 16 * 11).tobytes()))
    out.append((W.random_bases(rng, 700).tobytes(), W.random_bases(rng, 900).tobytes()))
    return out


def kernel_sums(st, sq):
    """F' (L-bins 0..N) and R' (L-bins 0..N-2) as the kernel forms them."""
    n = np.arange(N)
    wl = np.exp(-2j * np.pi * n / L)
    FE = np.zeros(N // 2 + 1, complex)
    FO = np.zeros(N // 2, complex)
    RE = np.zeros(N // 2 + 1, complex)
    RO = np.zeros(N // 2, complex)
    for c0, c1 in ((0, 3), (1, 2)):
        z = st[c0, :N] + 1j * st[c1, :N]
        w = sq[c0, :N] + 1j * sq[c1, :N]
        ZE, ZO, WE, WO = np.fft.fft(z), np.fft.fft(z * wl), np.fft.fft(w), np.fft.fft(w * wl)
        m = np.arange(N // 2 + 1)
        A, B, C, D = ZE[m], ZE[(N - m) % N], WE[m], WE[(N - m) % N]
        f = np.conj(A) * C + B * np.conj(D)
        f[N // 2] = 2 * (A[N // 2].real + A[N // 2].imag)
        r = A * C - np.conj(B * D)
        r[N // 2] = 0
        FE += f
        RE += r
        m = np.arange(N // 2)
        A, B, C, D = ZO[m], ZO[N - 1 - m], WO[m], WO[N - 1 - m]
        f = np.conj(A) * C + B * np.conj(D)
        a, b = A[-1], B[-1]
        f[-1] = (a + np.conj(b)) - 1j * (a - np.conj(b))
        r = A * C - np.conj(B * D)
        r[-1] = 0
        FO += f
        RO += r
    F = np.zeros(N + 1, complex)
    R = np.zeros(N + 1, complex)
    F[0::2], F[1::2] = FE, FO
    R[0::2], R[1::2] = RE, RO
    return F, R


def pack_inverse(S):
    """hermitian_pack with HALF = 1 and the N-point inverse, then lag i of the
    L-point correlation at r[(i + N) mod L] * 1/(4N)."""
    k = np.arange(N)
    Sk, Sn = S[k], S[N - k]
    E = Sk + np.conj(Sn)
    Dv = Sk - np.conj(Sn)
    Ov = Dv * np.conj(np.exp(-2j * np.pi * k / L))
    Z = E + 1j * Ov
    zt = np.fft.ifft(Z) * N            # unnormalised inverse
    r = np.empty(L)
    r[0::2], r[1::2] = zt.real, zt.imag
    return np.roll(r, -N) / (4 * N)


@pytest.mark.parametrize("k", range(4))
def test_sums_equal_the_channel_separated_form(O, k):
    t, q = pairs()[k]
    st = O.signal(t, L).astype(np.float64)
    sq = O.signal(q, L).astype(np.float64)
    F, R = kernel_sums(st, sq)
    T = np.fft.rfft(st, axis=1)        # bins 0..N of the L-point spectra
    Qf = np.fft.rfft(sq, axis=1)
    want_F = np.sum(np.conj(T) * Qf, axis=0)
    want_F[0] = np.sum(T[:, 0].real * Qf[:, 0].real)
    want_F[N - 1:] = np.sum(T[:, N - 1:], axis=0)
    scale = np.abs(want_F).max()
    assert np.abs(F / 2 - want_F).max() <= 1e-9 * scale
    want_R = np.sum(T * Qf[COMP], axis=0)
    assert np.abs(R[:N - 1] / 2j - want_R[:N - 1]).max() <= 1e-9 * scale


@pytest.mark.parametrize("k", range(4))
def test_both_strands_equal_the_direct_correlation(O, k):
    t, q = pairs()[k]
    Q = len(q)
    assert Q < 1024 or Q % (L // 512) == 0
    st = O.signal(t, L).astype(np.float64)
    sq = O.signal(q, L).astype(np.float64)
    F, R = kernel_sums(st, sq)
    fwd = pack_inverse(F)
    kk = np.arange(N + 1)
    wq = np.exp(-2j * np.pi * (((Q - 1) * kk) % L) / L)
    Sr = wq * (R.imag + 1j * R.real)   # W_L^((Q-1)k) i conj(R')
    Sr[N - 1:] = F[N - 1:]
    rev = pack_inverse(Sr)
    for got, qq in ((fwd, q), (rev, O.rc(q))):
        want = O.xcorr64(t, qq, L)
        assert np.abs(got - want).max() <= 1e-9 * max(1.0, np.abs(want).max())
