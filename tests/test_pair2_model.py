"""CPU model of corr_pair2_kernel's arithmetic (csrc/xc_corr.cu), in FP64
numpy: the signals in the basis u = s_A - s_T, v = s_C - s_G, w = s_A + s_T,
the per-bin steps that form the channel sums from the packed spectra, the
factors of four they leave in, and the reverse strand's sum through
i conj(x + iy) = y + ix.

At an A/C/G/T position the four channels sum to zero (one holds
entropy * (1 - mean), the others entropy * (0 - mean), and the means sum to
one), so w = -(s_C + s_G) and, with U, V, W the spectra,
    sum_c conj(T_c) Q_c = conj(Wt) Wq + (conj(Ut) Uq + conj(Vt) Vq) / 2
    sum_c T_c Q_comp(c) = Wt Wq - (Ut Uq + Vt Vq) / 2.
Stage 1: u + i v of each sequence as its N-point even-bin transform Z and
odd-bin transform (of z W_L^n); per bin, with A = Zt(m), B = Zt(N-m),
C = Zq(m), D = Zq(N-m):
    F' = conj(A) C + B conj(D)           (= 2 (conj(Ut) Uq + conj(Vt) Vq))
    R' = -i (A conj(D) + conj(B) C)      (= -2i (Ut Uq + Vt Vq))
Stage 2: y = wt + i wq, with E = Y(m), H = Y(N-m):
    F' += 2 Im(H E) - i (|E|^2 - |H|^2) (= 4 conj(Wt) Wq)
    R' += E^2 - conj(H)^2                (= 4i Wt Wq)
bin 0 by the same formulas (B = A, D = C, H = E), the target-only bins N-1
and N zero (sum_c T_c).  The FP32 channel values the kernel starts from sum
to zero only up to their rounding, so the sums are checked against the
channel-separated form the reference computes (CrossCorr.cc:477-492) to
within that residual, and the whole strand -- Hermitian pack without its
halves, N-point inverse, scale 1/(8N) -- against the direct FP64
correlation, for both strands.  The spectra path (spec_kernel,
corr_spec_kernel) stores u + i v and w's real spectrum per chunk and forms
4 conj(Wt) Wq and 4i Wt Wq at each bin alone; its sums are checked against
the same two forms.  Signals come from the oracle's CCSignal restatement."""
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
    half = ((np.arange(N // 2 + 1), lambda m: (N - m) % N, 0), (np.arange(N // 2), lambda m: N - 1 - m, 1))
    # stage 1: u + i v per sequence
    z = (st[0] - st[3] + 1j * (st[1] - st[2]))[:N]
    w = (sq[0] - sq[3] + 1j * (sq[1] - sq[2]))[:N]
    for (m, partner, odd), acc_f, acc_r in zip(half, (FE, FO), (RE, RO)):
        Zt, Zq = (np.fft.fft(z * wl), np.fft.fft(w * wl)) if odd else (np.fft.fft(z), np.fft.fft(w))
        A, B, C, D = Zt[m], Zt[partner(m)], Zq[m], Zq[partner(m)]
        acc_f += np.conj(A) * C + B * np.conj(D)
        acc_r += -1j * (A * np.conj(D) + np.conj(B) * C)
    # stage 2: wt + i wq
    y = (st[0] + st[3] + 1j * (sq[0] + sq[3]))[:N]
    for (m, partner, odd), acc_f, acc_r in zip(half, (FE, FO), (RE, RO)):
        Y = np.fft.fft(y * wl) if odd else np.fft.fft(y)
        E, H = Y[m], Y[partner(m)]
        acc_f += 2 * np.imag(H * E) - 1j * (np.abs(E) ** 2 - np.abs(H) ** 2)
        acc_r += E * E - np.conj(H) ** 2
    FE[N // 2] = RE[N // 2] = FO[-1] = RO[-1] = 0   # target-only bins: sum_c T_c = 0
    F = np.zeros(N + 1, complex)
    R = np.zeros(N + 1, complex)
    F[0::2], F[1::2] = FE, FO
    R[0::2], R[1::2] = RE, RO
    return F, R


def pack_inverse(S):
    """hermitian_pack with HALF = 1 and the N-point inverse, then lag i of the
    L-point correlation at r[(i + N) mod L] * 1/(8N)."""
    k = np.arange(N)
    Sk, Sn = S[k], S[N - k]
    E = Sk + np.conj(Sn)
    Dv = Sk - np.conj(Sn)
    Ov = Dv * np.conj(np.exp(-2j * np.pi * k / L))
    Z = E + 1j * Ov
    zt = np.fft.ifft(Z) * N            # unnormalised inverse
    r = np.empty(L)
    r[0::2], r[1::2] = zt.real, zt.imag
    return np.roll(r, -N) / (8 * N)


def residual(st):
    """Largest |sum_c s_c(i)| of the FP32 channel values, and that over the
    largest |s_c(i)|: zero but for their rounding."""
    d = np.abs(st.sum(axis=0)).max()
    return d, d / np.abs(st).max()


@pytest.mark.parametrize("k", range(4))
def test_sums_equal_the_channel_separated_form(O, k):
    t, q = pairs()[k]
    st = O.signal(t, L).astype(np.float64)
    sq = O.signal(q, L).astype(np.float64)
    for s in (st, sq):
        assert residual(s)[1] <= 2.0 ** -22
    F, R = kernel_sums(st, sq)
    T = np.fft.rfft(st, axis=1)        # bins 0..N of the L-point spectra
    Qf = np.fft.rfft(sq, axis=1)
    want_F = np.sum(np.conj(T) * Qf, axis=0)
    want_F[0] = np.sum(T[:, 0].real * Qf[:, 0].real)
    want_F[N - 1:] = np.sum(T[:, N - 1:], axis=0)
    scale = np.abs(want_F).max()
    # the residual's spectrum is at most sqrt(L) residual; times |Q| <= scale
    tol = 1e-9 * scale + 4 * np.sqrt(L) * max(residual(st)[0], residual(sq)[0]) * np.abs(np.concatenate([T, Qf])).max()
    assert np.abs(F / 4 - want_F).max() <= tol
    assert np.abs(want_F[N - 1:]).max() <= 1e-9 * scale   # the reference's target-only bins: zero to rounding
    want_R = np.sum(T * Qf[COMP], axis=0)
    assert np.abs(R[:N - 1] / 4j - want_R[:N - 1]).max() <= tol


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
        # FP32 kernels differ from FP64 by ~5e-7 of max |xc|; the basis's
        # rounding residual contributes ~2e-9
        assert np.abs(got - want).max() <= 2e-8 * max(1.0, np.abs(want).max())


def spectra_sums(st, sq):
    """F' and R' as corr_spec_kernel forms them from chunk-wise stored
    spectra (spec_kernel): u + i v of each chunk (even-bin and odd-bin
    halves) and W, the spectrum of the real signal w = A + T, at each bin
    alone (no partner): 4 conj(Wt) Wq and 4i Wt Wq in place of the joint
    transform's E, H formulas."""
    n = np.arange(N)
    wl = np.exp(-2j * np.pi * n / L)
    F = np.zeros(N + 1, complex)
    R = np.zeros(N + 1, complex)
    z = (st[0] - st[3] + 1j * (st[1] - st[2]))[:N]
    w = (sq[0] - sq[3] + 1j * (sq[1] - sq[2]))[:N]
    Wt = np.fft.fft(st[0] + st[3])   # L-point spectra of the real signals
    Wq = np.fft.fft(sq[0] + sq[3])
    for odd in (0, 1):
        Zt, Zq = (np.fft.fft(z * wl), np.fft.fft(w * wl)) if odd else (np.fft.fft(z), np.fft.fft(w))
        m = np.arange(N // 2) if odd else np.arange(N // 2 + 1)
        mb = (N - 1 - m) if odd else (N - m) % N
        A, B, C, D = Zt[m], Zt[mb], Zq[m], Zq[mb]
        k = 2 * m + odd
        f = np.conj(A) * C + B * np.conj(D) + 4 * np.conj(Wt[k]) * Wq[k]
        r = -1j * (A * np.conj(D) + np.conj(B) * C) + 4j * Wt[k] * Wq[k]
        F[k], R[k] = f, r
    F[N - 1:] = 0   # target-only bins: sum_c T_c = 0
    R[N - 1:] = 0
    return F, R


@pytest.mark.parametrize("k", range(4))
def test_spectra_path_sums(O, k):
    """The spectra path's sums equal the channel-separated form to within the
    FP32 channel values' rounding residual, and the pair kernel's joint form
    to FP64 rounding."""
    t, q = pairs()[k]
    st = O.signal(t, L).astype(np.float64)
    sq = O.signal(q, L).astype(np.float64)
    F, R = spectra_sums(st, sq)
    F2, R2 = kernel_sums(st, sq)
    scale = np.abs(F2).max()
    assert np.abs(F[:N - 1] - F2[:N - 1]).max() <= 1e-9 * scale
    assert np.abs(R[:N - 1] - R2[:N - 1]).max() <= 1e-9 * scale
    T = np.fft.rfft(st, axis=1)
    Qf = np.fft.rfft(sq, axis=1)
    want_F = np.sum(np.conj(T) * Qf, axis=0)
    tol = 1e-9 * scale + 4 * np.sqrt(L) * max(residual(st)[0], residual(sq)[0]) * np.abs(np.concatenate([T, Qf])).max()
    assert np.abs(F[1:N - 1] / 4 - want_F[1:N - 1]).max() <= tol
