// GB300 (sm_103a) kernels of the satsuma2 cross-correlation path.
//
//   corr_kernel<log2 L>  one CTA per (chunk pair, strand).  Builds the
//                        4-channel entropy-weighted signals of target and query
//                        (reverse-complemented in-kernel for strand 1), runs the
//                        4-channel conjugate product-sum of their spectra with
//                        the reference's bin quirks, the inverse transform, and
//                        FindTop's envelope threshold with ordered compaction of
//                        the surviving offsets.  Everything stays in shared
//                        memory; HBM sees the chunk bytes in and the offset
//                        list out.
//   scan_kernel<log2 L>  one CTA per (chunk pair, strand).  DoOne's ungapped
//                        46-wide window scan of every surviving offset on 2-bit
//                        bitplanes (32 positions per word op, 8-position window
//                        screening), an FP32 screen of the match probability,
//                        and the exact FP64 GetMatchProbability / PrintMatch /
//                        FilterMatches tail for the survivors.
//   finalize kernels     order each strand's results as the reference appends
//                        them and pack them densely.
//
// Reference semantics cited per function; paths are relative to the satsuma2
// source tree.
#include "xc_internal.h"

#include <math.h>

namespace xc {

__constant__ unsigned char c_rc[256];   // DNACodec reverse complement (DNAVector.cc:13-58)
__constant__ uchar4 c_w4q[128];         // A,C,G,T weights in quarter units (thirds letters: 0)
__constant__ double c_wd[4][128];       // DNA_A..DNA_T weights (DNAVector.cc:351-369)

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 mul_i(float2 a) { return make_float2(-a.y, a.x); }

__device__ __forceinline__ bool is_acgt(unsigned b) { return b == 'A' || b == 'C' || b == 'G' || b == 'T'; }
__device__ __forceinline__ bool is_third(unsigned b) { return b == 'B' || b == 'V' || b == 'H' || b == 'D'; }
// A=0, C=1, G=2, T=3 for the four ASCII capitals.
__device__ __forceinline__ uint32_t code_of(unsigned b) { return ((b >> 1) ^ (b >> 2)) & 3u; }
__device__ __forceinline__ uint32_t lowmask(int n) { return n >= 32 ? 0xffffffffu : ((1u << n) - 1u); }

// Bank-conflict-free placement of complex element p in a transform buffer:
// XOR the 8-byte slot (low 4 bits) with bits 4..7.  A bijection on any
// power-of-two length >= 16.
__device__ __forceinline__ int swz(int p) { return p ^ ((p >> 4) & 15); }

// ---------------------------------------------------------------------------
// Small DFTs in registers, natural order in and out.  DIR = -1 forward
// (exp(-i...)), +1 inverse.
// ---------------------------------------------------------------------------
template <int DIR>
__device__ __forceinline__ void bf4(float2& x0, float2& x1, float2& x2, float2& x3) {
  const float2 a0 = cadd(x0, x2), a1 = csub(x0, x2), a2 = cadd(x1, x3), a3 = mul_i(csub(x1, x3));
  x0 = cadd(a0, a2);
  x2 = csub(a0, a2);
  if (DIR < 0) { x1 = csub(a1, a3); x3 = cadd(a1, a3); }
  else { x1 = cadd(a1, a3); x3 = csub(a1, a3); }
}

template <int R, int DIR> struct DFT;

template <int DIR> struct DFT<2, DIR> {
  static __device__ __forceinline__ void run(float2* x) {
    const float2 t = x[0];
    x[0] = cadd(t, x[1]);
    x[1] = csub(t, x[1]);
  }
};

template <int DIR> struct DFT<4, DIR> {
  static __device__ __forceinline__ void run(float2* x) { bf4<DIR>(x[0], x[1], x[2], x[3]); }
};

// 8 = 4 x 2: n = 2 n1 + n2, k = k1 + 4 k2.
template <int DIR> struct DFT<8, DIR> {
  static __device__ __forceinline__ void run(float2* x) {
    const float r = 0.70710678118654752f;
    bf4<DIR>(x[0], x[2], x[4], x[6]);
    bf4<DIR>(x[1], x[3], x[5], x[7]);
    x[3] = cmul(x[3], make_float2(r, DIR * r));
    x[5] = DIR < 0 ? make_float2(x[5].y, -x[5].x) : make_float2(-x[5].y, x[5].x);
    x[7] = cmul(x[7], make_float2(-r, DIR * r));
    float2 y[8];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
      y[k1] = cadd(x[2 * k1], x[2 * k1 + 1]);
      y[k1 + 4] = csub(x[2 * k1], x[2 * k1 + 1]);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = y[k];
  }
};

// 16 = 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2.
template <int DIR> struct DFT<16, DIR> {
  static __device__ __forceinline__ void run(float2* x) {
    const float c1 = 0.92387953251128674f, s1 = 0.38268343236508978f, r = 0.70710678118654752f;
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) bf4<DIR>(x[n2], x[n2 + 4], x[n2 + 8], x[n2 + 12]);
    // x[n2 + 4 k1] *= W16^(n2 k1)
    x[5] = cmul(x[5], make_float2(c1, DIR * s1));
    x[9] = cmul(x[9], make_float2(r, DIR * r));
    x[13] = cmul(x[13], make_float2(s1, DIR * c1));
    x[6] = cmul(x[6], make_float2(r, DIR * r));
    x[10] = DIR < 0 ? make_float2(x[10].y, -x[10].x) : make_float2(-x[10].y, x[10].x);
    x[14] = cmul(x[14], make_float2(-r, DIR * r));
    x[7] = cmul(x[7], make_float2(s1, DIR * c1));
    x[11] = cmul(x[11], make_float2(-r, DIR * r));
    x[15] = cmul(x[15], make_float2(-c1, -DIR * s1));
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) bf4<DIR>(x[4 * k1], x[4 * k1 + 1], x[4 * k1 + 2], x[4 * k1 + 3]);
    float2 y[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
      for (int k2 = 0; k2 < 4; k2++) y[k1 + 4 * k2] = x[4 * k1 + k2];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = y[k];
  }
};

// One in-place pass of span S and radix R over an N-point buffer.
// Forward (decimation in frequency): butterfly, then twiddle W_S^(j r').
// Inverse (decimation in time, the exact reverse): conjugate twiddle, then
// butterfly.  Forward passes in order S = N, N/R0, ... leave bin k at a
// mixed-radix digit-reversed position (pos_of table); the inverse passes in
// reverse order take that layout back to natural order.
template <int R, bool INV>
__device__ __forceinline__ void fft_pass(float2* __restrict__ buf, int N, int S,
                                         const float2* __restrict__ tw, int t, int nt) {
  const int d = S / R;
  const int B = N / R;
  const int tws = N / S;
  for (int b = t; b < B; b += nt) {
    const int j = b & (d - 1);
    const int base = (b - j) * R + j;
    float2 x[R];
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = buf[swz(base + r * d)];
    if (!INV) {
      DFT<R, -1>::run(x);
      if (d > 1) {
#pragma unroll
        for (int r = 1; r < R; r++) x[r] = cmul(x[r], __ldg(&tw[j * r * tws]));
      }
    } else {
      if (d > 1) {
#pragma unroll
        for (int r = 1; r < R; r++) x[r] = cmulc(x[r], __ldg(&tw[j * r * tws]));
      }
      DFT<R, 1>::run(x);
    }
#pragma unroll
    for (int r = 0; r < R; r++) buf[swz(base + r * d)] = x[r];
  }
}

// Radix plans (must match radix_plan() in the runtime):
//   N=512: 8,8,8   1024: 16,16,4   2048: 16,16,8   4096: 16,16,16   8192: 16,16,16,2
// Every thread of the CTA must call these (they contain __syncthreads).
template <int LOG2N>
__device__ __forceinline__ void fft_forward(float2* buf, const float2* tw, int t, int nt) {
  constexpr int N = 1 << LOG2N;
  if constexpr (LOG2N == 9) {
    fft_pass<8, false>(buf, N, 512, tw, t, nt); __syncthreads();
    fft_pass<8, false>(buf, N, 64, tw, t, nt); __syncthreads();
    fft_pass<8, false>(buf, N, 8, tw, t, nt); __syncthreads();
  } else if constexpr (LOG2N == 10) {
    fft_pass<16, false>(buf, N, 1024, tw, t, nt); __syncthreads();
    fft_pass<16, false>(buf, N, 64, tw, t, nt); __syncthreads();
    fft_pass<4, false>(buf, N, 4, tw, t, nt); __syncthreads();
  } else if constexpr (LOG2N == 11) {
    fft_pass<16, false>(buf, N, 2048, tw, t, nt); __syncthreads();
    fft_pass<16, false>(buf, N, 128, tw, t, nt); __syncthreads();
    fft_pass<8, false>(buf, N, 8, tw, t, nt); __syncthreads();
  } else if constexpr (LOG2N == 12) {
    fft_pass<16, false>(buf, N, 4096, tw, t, nt); __syncthreads();
    fft_pass<16, false>(buf, N, 256, tw, t, nt); __syncthreads();
    fft_pass<16, false>(buf, N, 16, tw, t, nt); __syncthreads();
  } else {
    static_assert(LOG2N == 13, "unsupported transform length");
    fft_pass<16, false>(buf, N, 8192, tw, t, nt); __syncthreads();
    fft_pass<16, false>(buf, N, 512, tw, t, nt); __syncthreads();
    fft_pass<16, false>(buf, N, 32, tw, t, nt); __syncthreads();
    fft_pass<2, false>(buf, N, 2, tw, t, nt); __syncthreads();
  }
}

template <int LOG2N>
__device__ __forceinline__ void fft_inverse(float2* buf, const float2* tw, int t, int nt) {
  constexpr int N = 1 << LOG2N;
  if constexpr (LOG2N == 9) {
    fft_pass<8, true>(buf, N, 8, tw, t, nt); __syncthreads();
    fft_pass<8, true>(buf, N, 64, tw, t, nt); __syncthreads();
    fft_pass<8, true>(buf, N, 512, tw, t, nt); __syncthreads();
  } else if constexpr (LOG2N == 10) {
    fft_pass<4, true>(buf, N, 4, tw, t, nt); __syncthreads();
    fft_pass<16, true>(buf, N, 64, tw, t, nt); __syncthreads();
    fft_pass<16, true>(buf, N, 1024, tw, t, nt); __syncthreads();
  } else if constexpr (LOG2N == 11) {
    fft_pass<8, true>(buf, N, 8, tw, t, nt); __syncthreads();
    fft_pass<16, true>(buf, N, 128, tw, t, nt); __syncthreads();
    fft_pass<16, true>(buf, N, 2048, tw, t, nt); __syncthreads();
  } else if constexpr (LOG2N == 12) {
    fft_pass<16, true>(buf, N, 16, tw, t, nt); __syncthreads();
    fft_pass<16, true>(buf, N, 256, tw, t, nt); __syncthreads();
    fft_pass<16, true>(buf, N, 4096, tw, t, nt); __syncthreads();
  } else {
    static_assert(LOG2N == 13, "unsupported transform length");
    fft_pass<2, true>(buf, N, 2, tw, t, nt); __syncthreads();
    fft_pass<16, true>(buf, N, 32, tw, t, nt); __syncthreads();
    fft_pass<16, true>(buf, N, 512, tw, t, nt); __syncthreads();
    fft_pass<16, true>(buf, N, 8192, tw, t, nt); __syncthreads();
  }
}

// Ent (CrossCorr.cc:28-33) for windows holding a one-third IUPAC letter.
__device__ __forceinline__ double ent_dev(double p) {
  if (p < 0.001) return 0.0;
  return __ddiv_rn(__dmul_rn(p, log(p)), 0.69314718056);
}

// ---------------------------------------------------------------------------
// Correlation + FindTop kernel
// ---------------------------------------------------------------------------
size_t corr_smem_bytes(int log2L) {
  const size_t N = (size_t)1 << (log2L - 1);
  return 3 * N * sizeof(float2)        // even / odd transform buffers, spectrum accumulator
         + 2 * N                       // target and query bytes
         + 2 * 256 * sizeof(float)     // entropy weight per window, target and query
         + 2 * 256 * sizeof(float2);   // per-window signal values of the current channel
}

template <int LOG2L>
__global__ void __launch_bounds__(NT_CORR, (LOG2L <= 13) ? 2 : 1) corr_kernel(const CorrParams P) {
  constexpr int L = 1 << LOG2L;
  constexpr int N = L >> 1;
  constexpr int LOG2N = LOG2L - 1;
  constexpr int WIN = L / 512;   // CCSignal::ComputeEntropy window (CrossCorr.cc:46)
  constexpr int NWIN = 256;      // N / WIN

  extern __shared__ __align__(16) unsigned char smem[];
  float2* bufE = reinterpret_cast<float2*>(smem);
  float2* bufO = bufE + N;
  float2* acc = bufO + N;
  uint8_t* st = reinterpret_cast<uint8_t*>(acc + N);
  uint8_t* sq = st + N;
  float* Et = reinterpret_cast<float*>(sq + N);
  float* Eq = Et + NWIN;
  float2* vt = reinterpret_cast<float2*>(Eq + NWIN);
  float2* vq = vt + NWIN;
  __shared__ int s_cnt4[8];
  __shared__ double s_off[8];
  __shared__ float s_nyq;
  __shared__ int s_warp[NT_CORR / 32];

  const int tid = threadIdx.x;
  const int pidx = P.first + blockIdx.x;
  const int strand = blockIdx.y;
  const PairDesc D = P.pairs[pidx];
  const int T = D.tlen, Q = D.qlen;
  const uint8_t* __restrict__ gt = P.pool + D.t_off;
  const uint8_t* __restrict__ gq = P.pool + D.q_off;

  // ---- chunk bytes to shared memory; strand 1 reverse-complements the query
  //      (DNAVector::ReverseComplement, DNAVector.cc:482-500) ----
  int high = 0, nonacgt = 0, th_t = 0, th_q = 0;
  for (int i = tid; i < N; i += NT_CORR) {
    unsigned b = 0;
    if (i < T) {
      b = gt[i];
      high |= b >> 7;
      nonacgt |= !is_acgt(b);
      th_t |= is_third(b);
    }
    st[i] = (uint8_t)b;
    unsigned c = 0;
    if (i < Q) {
      const unsigned raw = strand ? gq[Q - 1 - i] : gq[i];
      high |= raw >> 7;
      c = strand ? c_rc[raw] : raw;
      nonacgt |= !is_acgt(c);
      th_q |= is_third(c);
    }
    sq[i] = (uint8_t)c;
  }
  if (tid < 8) s_cnt4[tid] = 0;
  if (tid == 0) s_nyq = 0.f;
  const int any_high = __syncthreads_or(high);
  const int generic = __syncthreads_or(nonacgt);
  th_t = __syncthreads_or(th_t);
  th_q = __syncthreads_or(th_q);
  if (any_high) {
    if (tid == 0) {
      P.off_cnt[pidx * 2 + strand] = 0;
      if (strand == 0) P.pair_flags[pidx] = PF_INVALID;
    }
    return;
  }
  if (tid == 0 && strand == 0) P.pair_flags[pidx] = (D.flags & PF_FAST) | (generic ? PF_GENERIC : 0u);
  for (int i = tid; i < N; i += NT_CORR) acc[i] = make_float2(0.f, 0.f);

  // ---- entropy weight per window (CCSignal::ComputeEntropy, CrossCorr.cc:35-93).
  //      Threads 0..255: target windows, 256..511: query windows.  Windows
  //      without one-third letters have exact quarter-unit base sums, so Ent
  //      comes from a table the host computed with the same double
  //      expression; others repeat the reference's double arithmetic here. ----
  {
    const int which = tid >> 8, w = tid & 255;
    const uint8_t* s = which ? sq : st;
    const int len = which ? Q : T;
    const int third = which ? th_q : th_t;
    float E = 0.f;
    if (len < 1024) {
      E = 1.f;
    } else if (w * WIN < len) {
      const int i0 = w * WIN;
      const int k = min(WIN, len - i0);
      bool has3 = false;
      if (third)
        for (int j = 0; j < k; j++) has3 |= is_third(s[i0 + j]);
      double sv;
      if (!has3) {
        int a4 = 0, c4 = 0, g4 = 0, t4 = 0;
        for (int j = 0; j < k; j++) {
          const uchar4 q = c_w4q[s[i0 + j]];
          a4 += q.x; c4 += q.y; g4 += q.z; t4 += q.w;
        }
        const double* et = P.tab.ent + k * (4 * WIN + 1);
        sv = __dadd_rn(__dadd_rn(__dadd_rn(__ldg(et + a4), __ldg(et + c4)), __ldg(et + g4)), __ldg(et + t4));
      } else {
        double a = 0, c = 0, g = 0, t = 0;
        for (int j = 0; j < k; j++) {
          const int b = s[i0 + j];
          a = __dadd_rn(a, c_wd[0][b]);
          c = __dadd_rn(c, c_wd[1][b]);
          g = __dadd_rn(g, c_wd[2][b]);
          t = __dadd_rn(t, c_wd[3][b]);
        }
        a = __ddiv_rn(a, (double)k);
        c = __ddiv_rn(c, (double)k);
        g = __ddiv_rn(g, (double)k);
        t = __ddiv_rn(t, (double)k);
        sv = __dadd_rn(__dadd_rn(__dadd_rn(ent_dev(a), ent_dev(c)), ent_dev(g)), ent_dev(t));
      }
      E = __double2float_rn(-sv);
      if (E < 0.f) E = 0.f;
    }
    (which ? Eq : Et)[w] = E;
  }

  // ---- channel means (SeqToPCM, CrossCorr.cc:108-116): exact quarter-unit
  //      sums, or the sequential double sum when one-third letters occur ----
  {
    int cn[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = tid; i < N; i += NT_CORR) {
      if (i < T) { const uchar4 q = c_w4q[st[i]]; cn[0] += q.x; cn[1] += q.y; cn[2] += q.z; cn[3] += q.w; }
      if (i < Q) { const uchar4 q = c_w4q[sq[i]]; cn[4] += q.x; cn[5] += q.y; cn[6] += q.z; cn[7] += q.w; }
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int v = __reduce_add_sync(0xffffffffu, cn[k]);
      if ((tid & 31) == 0 && v) atomicAdd(&s_cnt4[k], v);
    }
  }
  __syncthreads();
  if (tid < 8) {
    const int which = tid >> 2, c = tid & 3;
    const int len = which ? Q : T;
    const int third = which ? th_q : th_t;
    double off = 0.0;
    if (len > 0) {
      if (!third) {
        off = __ddiv_rn((double)s_cnt4[tid] * 0.25, (double)len);
      } else {
        const uint8_t* s = which ? sq : st;
        double sum = 0.0;
        for (int i = 0; i < len; i++) sum = __dadd_rn(sum, c_wd[c][s[i]]);
        off = __ddiv_rn(sum, (double)len);
      }
    }
    s_off[tid] = off;
  }
  __syncthreads();

  const int grp = tid >> 8;   // 0: even-bin transform, 1: odd-bin transform
  const int gtid = tid & 255;

  for (int c = 0; c < 4; c++) {
    // Per-window channel values: out = float(entropy * (weight - mean))
    // (CrossCorr.cc:123), weight 0 or 1 for A/C/G/T.
    if (!generic) {
      const double off = s_off[grp * 4 + c];
      const double E = (double)(grp ? Eq : Et)[gtid];
      float2 v;
      v.x = __double2float_rn(__dmul_rn(E, __dsub_rn(0.0, off)));
      v.y = __double2float_rn(__dmul_rn(E, __dsub_rn(1.0, off)));
      (grp ? vq : vt)[gtid] = v;
    }
    __syncthreads();

    // z[n] = target_c[n] + i*query_c[n]; the odd-bin group pre-twiddles by
    // W_L^n.  Both signals are zero past N, so the even bins of the L-point
    // transform are the N-point transform of z and the odd bins that of
    // z*W_L^n.
    {
      float2* buf = grp ? bufO : bufE;
      const double offt = s_off[c], offq = s_off[4 + c];
      for (int n = gtid; n < N; n += 256) {
        float x = 0.f, y = 0.f;
        const int w = n / WIN;
        if (!generic) {
          if (n < T) { const float2 v = vt[w]; x = code_of(st[n]) == (uint32_t)c ? v.y : v.x; }
          if (n < Q) { const float2 v = vq[w]; y = code_of(sq[n]) == (uint32_t)c ? v.y : v.x; }
        } else {
          if (n < T) x = __double2float_rn(__dmul_rn((double)Et[w], __dsub_rn(c_wd[c][st[n]], offt)));
          if (n < Q) y = __double2float_rn(__dmul_rn((double)Eq[w], __dsub_rn(c_wd[c][sq[n]], offq)));
        }
        if (P.dbg_sig && grp == 0) {
          float* ds = P.dbg_sig + (size_t)(pidx * 2 + strand) * 8 * L;
          ds[(size_t)c * L + n] = x;
          ds[(size_t)(4 + c) * L + n] = y;
        }
        float2 z = make_float2(x, y);
        if (grp) z = cmul(z, __ldg(&P.tab.twL[n]));
        buf[swz(n)] = z;
      }
    }
    __syncthreads();

    fft_forward<LOG2N>(grp ? bufO : bufE, P.tab.twN, gtid, 256);

    // Per-bin product (CrossCorrelation::DoOne, CrossCorr.cc:477-492):
    // X = target spectrum, Y = query spectrum from Z(k), Z(L-k).
    // conj(X)Y on bins 1..N-2, X(0)Y(0) on bin 0, and the target's own value
    // on bins N-1 and N, which the reference's loop leaves unmultiplied.
    if (grp == 0) {
      for (int m = gtid; m <= N / 2; m += 256) {
        const int k = 2 * m;
        const float2 A = bufE[swz(P.tab.pos_of[m])];
        const float2 B = bufE[swz(P.tab.pos_of[(N - m) & (N - 1)])];
        const float2 X = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
        const float2 Y = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
        if (k == N) s_nyq += X.x;
        else acc[k] = cadd(acc[k], cmulc(Y, X));
      }
    } else {
      for (int m = gtid; m < N / 2; m += 256) {
        const int k = 2 * m + 1;
        const float2 A = bufO[swz(P.tab.pos_of[m])];
        const float2 B = bufO[swz(P.tab.pos_of[N - 1 - m])];
        const float2 X = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
        const float2 Y = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
        acc[k] = cadd(acc[k], k == N - 1 ? X : cmulc(Y, X));
      }
    }
    __syncthreads();
  }

  // ---- inverse: half-length complex transform of the Hermitian spectrum.
  //      Z(k) = E(k) + i O(k), E = (S(k) + conj S(N-k))/2,
  //      O = (S(k) - conj S(N-k)) conj(W_L^k)/2; z[m] = r[2m] + i r[2m+1]. ----
  for (int k = tid; k <= N / 2; k += NT_CORR) {
    const float2 Sk = acc[k];
    const float2 Sn = k == 0 ? make_float2(s_nyq, 0.f) : acc[N - k];
    {
      const float2 Ev = make_float2(0.5f * (Sk.x + Sn.x), 0.5f * (Sk.y - Sn.y));
      const float2 Dv = make_float2(0.5f * (Sk.x - Sn.x), 0.5f * (Sk.y + Sn.y));
      const float2 Ov = cmulc(Dv, __ldg(&P.tab.twL[k]));
      bufE[swz(P.tab.pos_of[k])] = make_float2(Ev.x - Ov.y, Ev.y + Ov.x);
    }
    if (k != 0 && k != N / 2) {
      const float2 Ev = make_float2(0.5f * (Sn.x + Sk.x), 0.5f * (Sn.y - Sk.y));
      const float2 Dv = make_float2(0.5f * (Sn.x - Sk.x), 0.5f * (Sn.y + Sk.y));
      const float2 Ov = cmulc(Dv, __ldg(&P.tab.twL[N - k]));
      bufE[swz(P.tab.pos_of[N - k])] = make_float2(Ev.x - Ov.y, Ev.y + Ov.x);
    }
  }
  __syncthreads();
  fft_inverse<LOG2N>(bufE, P.tab.twN, tid < 256 ? tid : (1 << 30), 256);

  // ---- FindTop (SeqAnalyzer::FindTop, CrossCorr.cc:878-944): xc[i] =
  //      r[(i + N) mod L] / N; envelope over 256-sample blocks when L/256 > 8;
  //      keep i with xc[i] > env*cutoff + 1 in increasing i. ----
  constexpr int EPT = L / NT_CORR;
  const int ib = tid * EPT;
  const float scale = 1.0f / (float)N;
  auto xval = [&](int i) -> float {
    const int n = (i + N) & (L - 1);
    const float2 z = bufE[swz(n >> 1)];
    return ((n & 1) ? z.y : z.x) * scale;
  };
  float thr = 1.0f;
  if constexpr (L / 256 > 8) {
    // Squares are float products as in the reference; the block sum is
    // compensated in FP32 per thread and combined in FP64.
    float s = 0.f, comp = 0.f;
#pragma unroll 4
    for (int e = 0; e < EPT; e++) {
      const float x = xval(ib + e);
      const float v = __fmul_rn(x, x);
      const float y = __fsub_rn(v, comp);
      const float t2 = __fadd_rn(s, y);
      comp = __fsub_rn(__fsub_rn(t2, s), y);
      s = t2;
    }
    double ds = __dsub_rn((double)s, (double)comp);
    constexpr int G = 256 / EPT;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) ds = __dadd_rn(ds, __shfl_xor_sync(0xffffffffu, ds, o));
    const double env = __dsqrt_rn(__ddiv_rn(ds, 256.0));
    const double cut = (D.flags & PF_FAST) ? P.cutoff_fast : P.cutoff;
    // x > t (double) <=> x > round_down_to_float(t) for a float x.
    thr = __double2float_rd(__dadd_rn(__dmul_rn(env, cut), 1.0));
  }
  int cnt = 0;
  for (int e = 0; e < EPT; e++) cnt += xval(ib + e) > thr;
  // block exclusive scan of cnt
  const int lane = tid & 31, warp = tid >> 5;
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int v = lane < NT_CORR / 32 ? s_warp[lane] : 0;
    int w = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    if (lane < NT_CORR / 32) s_warp[lane] = w - v;
  }
  __syncthreads();
  int k = s_warp[warp] + incl - cnt;
  int* out = P.off_list + D.off_base + (size_t)strand * L;
  for (int e = 0; e < EPT; e++) {
    const float x = xval(ib + e);
    if (x > thr) out[k++] = ib + e;
    if (P.dbg_xc) P.dbg_xc[(size_t)(pidx * 2 + strand) * L + ib + e] = x;
  }
  if (tid == NT_CORR - 1) P.off_cnt[pidx * 2 + strand] = k;
}

// ---------------------------------------------------------------------------
// Scan kernel: DoOne + FilterMatches
// ---------------------------------------------------------------------------
template <int LOG2L> struct ScanGeom {
  static constexpr int L = 1 << LOG2L;
  static constexpr int N = L >> 1;
  static constexpr int TW = N / 32;        // 32-position words per chunk
  static constexpr int TWP = TW + 2;       // target plane words (zero padded)
  static constexpr int QPAD = 2;           // leading zero words of the query planes
  static constexpr int QWP = TW + 6;       // query plane words
  static constexpr size_t bytes =
      (size_t)(2 * TWP + (TW + 1) + 2 * QWP + (TW + 1) + OFF_CHUNK) * 4 + OFF_CHUNK * 2 + 2 * N;
};

size_t scan_smem_bytes(int log2L) {
  switch (log2L) {
    case 10: return ScanGeom<10>::bytes;
    case 11: return ScanGeom<11>::bytes;
    case 12: return ScanGeom<12>::bytes;
    case 13: return ScanGeom<13>::bytes;
    case 14: return ScanGeom<14>::bytes;
  }
  return 0;
}

// Diagonal work length of offset pos: positions i0..iend-1 of DoOne's loop.
__device__ __forceinline__ int diag_len(int pos, int T, int Q) {
  const int i0 = max(0, -pos);
  const int iend = min(T - 1, Q - pos);
  return max(0, iend - i0);
}

// Count of G/C bases in [a, e) from a per-word prefix and the bitplanes.
__device__ __forceinline__ int gc_count(const uint32_t* b0, const uint32_t* b1, const int* pref, int a, int e) {
  const int wa = a >> 5, we = e >> 5;
  const int ga = pref[wa] + __popc((b0[wa] ^ b1[wa]) & lowmask(a & 31));
  const int ge = pref[we] + __popc((b0[we] ^ b1[we]) & lowmask(e & 31));
  return ge - ga;
}

// Warp-cooperative inclusive prefix of per-word G/C counts -> pref[0..nw].
__device__ __forceinline__ void gc_prefix(const uint32_t* b0, const uint32_t* b1, int* pref, int nw, int lane) {
  int run = 0;
  for (int w0 = 0; w0 < nw; w0 += 32) {
    const int w = w0 + lane;
    const int c = w < nw ? __popc(b0[w] ^ b1[w]) : 0;
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (w < nw) pref[w] = run + incl - c;
    run += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) pref[nw] = run;
}

template <int LOG2L>
__global__ void __launch_bounds__(NT_SCAN) scan_kernel(const ScanParams P) {
  using Gm = ScanGeom<LOG2L>;
  constexpr int L = Gm::L, N = Gm::N, TW = Gm::TW, TWP = Gm::TWP, QPAD = Gm::QPAD, QWP = Gm::QWP;
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* tb0 = reinterpret_cast<uint32_t*>(smem);
  uint32_t* tb1 = tb0 + TWP;
  int* tgp = reinterpret_cast<int*>(tb1 + TWP);
  uint32_t* qb0 = reinterpret_cast<uint32_t*>(tgp + (TW + 1));
  uint32_t* qb1 = qb0 + QWP;
  int* qgp = reinterpret_cast<int*>(qb1 + QWP);
  int* offs = qgp + (TW + 1);
  uint16_t* order = reinterpret_cast<uint16_t*>(offs + OFF_CHUNK);
  uint8_t* st = reinterpret_cast<uint8_t*>(order + OFF_CHUNK);
  uint8_t* sq = st + N;
  __shared__ int s_hist[64];
  __shared__ int s_next;
  __shared__ int s_res;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int pidx = P.first + blockIdx.x;
  const int strand = blockIdx.y;
  const int slot = pidx * 2 + strand;
  const PairDesc D = P.pairs[pidx];
  const uint32_t flags = P.pair_flags[pidx];
  const int cnt = P.off_cnt[slot];
  if ((flags & PF_INVALID) || cnt <= 0) {
    if (tid == 0) P.res_cnt[slot] = 0;
    return;
  }
  const int T = D.tlen, Q = D.qlen;
  const bool generic = (flags & PF_GENERIC) != 0;
  const uint8_t* __restrict__ gt = P.pool + D.t_off;
  const uint8_t* __restrict__ gq = P.pool + D.q_off;

  for (int i = tid; i < N; i += NT_SCAN) {
    st[i] = i < T ? gt[i] : 0;
    unsigned c = 0;
    if (i < Q) {
      const unsigned raw = strand ? gq[Q - 1 - i] : gq[i];
      c = strand ? c_rc[raw] : raw;
    }
    sq[i] = (uint8_t)c;
  }
  if (tid == 0) s_res = 0;
  __syncthreads();
  if (!generic) {
    // 2-bit codes as two bitplanes, bit u of word w = position 32w+u.
    for (int w = tid; w < TWP; w += NT_SCAN) {
      uint32_t b0 = 0, b1 = 0;
      if (w < TW) {
        for (int u = 0; u < 32; u++) {
          const int i = 32 * w + u;
          if (i < T) { const uint32_t cd = code_of(st[i]); b0 |= (cd & 1u) << u; b1 |= (cd >> 1) << u; }
        }
      }
      tb0[w] = b0;
      tb1[w] = b1;
    }
    for (int w = tid; w < QWP; w += NT_SCAN) {
      uint32_t b0 = 0, b1 = 0;
      const int ww = w - QPAD;
      if (ww >= 0 && ww < TW) {
        for (int u = 0; u < 32; u++) {
          const int i = 32 * ww + u;
          if (i < Q) { const uint32_t cd = code_of(sq[i]); b0 |= (cd & 1u) << u; b1 |= (cd >> 1) << u; }
        }
      }
      qb0[w] = b0;
      qb1[w] = b1;
    }
    __syncthreads();
    if (warp == 0) gc_prefix(tb0, tb1, tgp, TW, lane);
    if (warp == 1) gc_prefix(qb0 + QPAD, qb1 + QPAD, qgp, TW, lane);
  }
  __syncthreads();

  const int* __restrict__ olist = P.off_list + D.off_base + (size_t)strand * L;

  // Emits one DoOne segment [s0, s1) on offset pos (CrossCorr.cc:693,713) and
  // applies FilterMatches (HomologyByXCorrSlave.cc:171-212) to it.  hits:
  // exact equal-base count for A/C/G/T pairs (ignored on the generic path).
  auto emit = [&](int key, int pos, int s0, int s1, int hits) {
    const int len = s1 - s0;
    if (P.dbg) {
      const int d = atomicAdd(P.dbg_cnt, 1);
      if (d < P.dbg_cap) {
        DbgSeg g;
        g.slot = slot; g.key = key; g.tstart = s0; g.qstart = s0 + pos; g.len = len;
        g.pad[0] = g.pad[1] = g.pad[2] = 0;
        P.dbg[d] = g;
      } else {
        atomicOr(P.err, 2);
      }
    }
    if (len < P.min_len) return;
    double matches, gcT, gcQ;
    if (!generic) {
      const int gT = gc_count(tb0, tb1, tgp, s0, s1);
      const int gQ = gc_count(qb0 + QPAD, qb1 + QPAD, qgp, s0 + pos, s1 + pos);
      if (!P.ptable) {
        // FP32 screen: reject only when the expectation clears the bound by
        // 1%, far beyond FP32 error; anything else goes to the exact test.
        const float Nf = (float)len, gq = (float)gQ, gtf = (float)gT / Nf;
        const float pm = (gq * gtf + (Nf - gq) * (1.f - gtf)) / Nf * 0.5f;
        const float sg = sqrtf(pm * (1.f - pm) * Nf);
        const float arg = (pm * Nf - (float)hits) / sg * 0.70710678118654752f;
        const float ex = 0.5f * erfcf(-arg) * P.target_total_f;
        if (ex > P.screen_expect) return;
      }
      matches = (double)hits;
      gcT = (double)gT;
      gcQ = (double)gQ;
    } else {
      // GetMatchProbabilityEx's sums, in its order (AlignProbability.cc:79-95).
      matches = 0.0; gcT = 0.0; gcQ = 0.0;
      for (int i = 0; i < len; i++) {
        const int a = st[s0 + i], b = sq[s0 + pos + i];
        matches = __dadd_rn(matches, __ldg(&P.eq[a * 128 + b]));
        gcT = __dadd_rn(gcT, __ldg(&P.gcw[a]));
        gcQ = __dadd_rn(gcQ, __ldg(&P.gcw[b]));
      }
    }
    // GetMatchProbabilityEx (AlignProbability.cc:107-125) in FP64, no FMA.
    const double Nd = (double)len;
    const double ident = __ddiv_rn(matches, Nd);
    const double gct = __ddiv_rn(gcT, Nd);
    double r = __dmul_rn(gcQ, gct);
    r = __dadd_rn(r, __dmul_rn(__dsub_rn(Nd, gcQ), __dsub_rn(1.0, gct)));
    const double pm = __ddiv_rn(__ddiv_rn(r, Nd), 2.0);
    double prob;
    if (!P.ptable) {
      const double sg = __dsqrt_rn(__dmul_rn(__dmul_rn(pm, __dsub_rn(1.0, pm)), Nd));
      const double m = __dmul_rn(pm, Nd);
      const double x = __dmul_rn(Nd, ident);
      const double cdf = __dmul_rn(0.5, __dadd_rn(1.0, erf(__ddiv_rn(__ddiv_rn(__dsub_rn(m, x), sg), 1.414213562))));
      prob = exp(-__dmul_rn(cdf, P.target_total));
    } else {
      // ProbTable::GetMatchProbability / IsGood (ProbTable.cc:58-74,105-140).
      // Row 0 of the reference table is empty (undefined there); not good here.
      const int idx = (int)__dmul_rn(pm, 511.0);
      prob = 0.0;
      if (idx > 0 && idx < 512) {
        const int l = len >= 2048 ? 2047 : len;
        if (ident >= __ldg(&P.ptable[(size_t)idx * 2048 + l])) prob = P.ptable_cutoff;
      }
    }
    if (prob < P.min_prob) return;
    DevResult rec;
    rec.key = key; rec.tstart = s0; rec.qstart = s0 + pos; rec.len = len; rec.prob = prob; rec.ident = ident;
    const int k = atomicAdd(&s_res, 1);
    if (k < P.slots) {
      P.res[(size_t)slot * P.slots + k] = rec;
    } else {
      const int o = atomicAdd(P.ovf_cnt, 1);
      if (o < P.ovf_cap) {
        DevResultX x;
        x.slot = slot; x.pad[0] = x.pad[1] = x.pad[2] = 0; x.r = rec;
        P.ovf[o] = x;
      } else {
        atomicOr(P.err, 1);
      }
    }
  };

  for (int c0 = 0; c0 < cnt; c0 += OFF_CHUNK) {
    const int nc = min(OFF_CHUNK, cnt - c0);
    if (tid < 64) s_hist[tid] = 0;
    __syncthreads();
    // Longest diagonals first so the warps of the CTA stay balanced.
    for (int k = tid; k < nc; k += NT_SCAN) {
      const int o = olist[c0 + k];
      offs[k] = o;
      const int b = 63 - (int)(((long long)diag_len(o - N, T, Q) * 64) / N);
      atomicAdd(&s_hist[b], 1);
    }
    __syncthreads();
    if (warp == 0) {
      const int v0 = s_hist[lane], v1 = s_hist[lane + 32];
      int a = v0 + v1;   // lanes own bins lane and lane+32: scan two halves
      int i0 = v0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, i0, o);
        if (lane >= o) i0 += u;
      }
      const int tot0 = __shfl_sync(0xffffffffu, i0, 31);
      int i1 = v1;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, i1, o);
        if (lane >= o) i1 += u;
      }
      (void)a;
      s_hist[lane] = i0 - v0;
      s_hist[lane + 32] = tot0 + i1 - v1;
    }
    __syncthreads();
    for (int k = tid; k < nc; k += NT_SCAN) {
      const int b = 63 - (int)(((long long)diag_len(offs[k] - N, T, Q) * 64) / N);
      const int p = atomicAdd(&s_hist[b], 1);
      order[p] = (uint16_t)k;
    }
    if (tid == 0) s_next = 0;
    __syncthreads();

    for (;;) {
      const int k = atomicAdd(&s_next, 1);
      if (k >= nc) break;
      const int li = order[k];
      const int pos = offs[li] - N;
      const int key = c0 + li;
      const int i0 = max(0, -pos);
      const int iend = min(T - 1, Q - pos);
      if (generic) {
        // SeqAnalyzer::DoOne, OPTIM_DOONE (CrossCorr.cc:667-724), byte table.
        int match = 0, last = -1, n = 0;
        for (int i = i0; i < T; i++) {
          const int j = i + pos;
          if (j >= Q || i + 1 >= T) {
            if (last != -1) emit(key, pos, last, i, 0);
            break;
          }
          match += __ldg(&P.score[st[i] * 128 + sq[j]]);
          if (n > 45) {
            match -= __ldg(&P.score[st[i - 46] * 128 + sq[j - 46]]);
            if (match > 1889) {
              if (last == -1) last = i - 45;
            } else {
              if (last != -1) emit(key, pos, last, i, 0);
              last = -1;
            }
          }
          n++;
        }
        continue;
      }
      // A/C/G/T: window sums are 100 x equal-base counts, so a window passes
      // when it holds >= 19 equal bases.  Check positions c run from i0+46 to
      // iend-1; window(c) = [c-45, c]; a segment is a maximal run of passing
      // checks [a..b], emitted as [a-45, b+1) (or [a-45, iend) at the end).
      const int cfirst = i0 + 46, clast = iend - 1;
      if (clast < cfirst) continue;
      const int wfirst = cfirst >> 5, wlast = clast >> 5;
      auto eword = [&](int w) -> uint32_t {
        if (w < 0) return 0u;
        const int qo = 32 * w + pos + 32 * QPAD;
        const int qw = qo >> 5, sh = qo & 31;
        const uint32_t q0 = __funnelshift_r(qb0[qw], qb0[qw + 1], sh);
        const uint32_t q1 = __funnelshift_r(qb1[qw], qb1[qw + 1], sh);
        return ~((tb0[w] ^ q0) | (tb1[w] ^ q1));
      };
      uint32_t e2 = eword(wfirst - 2), e1 = eword(wfirst - 1);
      int pref = __popc(e2) + __popc(e1);
      bool open = false;
      int start = 0, base = 0;
      for (int w = wfirst; w <= wlast; w++) {
        const uint32_t e0 = eword(w);
        const uint64_t U = ((uint64_t)e1 << 32) | e2;
        const int lo = max(cfirst - 32 * w, 0), hi = min(clast - 32 * w, 31);
        const uint32_t vm = (0xffffffffu >> (31 - hi)) & (0xffffffffu << lo);
        uint32_t g = 0;
#pragma unroll
        for (int sb = 0; sb < 4; sb++) {
          if (!((vm >> (8 * sb)) & 0xffu)) continue;
          const int a = 8 * sb + 19;
          const int c53 = __popcll(U >> a) + __popc(e0 & lowmask(a - 11));
          if (c53 < MIN_HITS) continue;
#pragma unroll
          for (int u = 8 * sb; u < 8 * sb + 8; u++) {
            const int wc = __popcll(U >> (u + 19)) + __popc(e0 & lowmask(u + 1));
            if (wc >= MIN_HITS) g |= 1u << u;
          }
        }
        g &= vm;
        const uint32_t prev = (g << 1) | (open ? 1u : 0u);
        const uint32_t rise = g & ~prev;
        const uint32_t fall = ~g & prev & vm;
        uint32_t ev = rise | fall;
        while (ev) {
          const int u = __ffs(ev) - 1;
          ev &= ev - 1;
          if ((rise >> u) & 1u) {
            start = 32 * w + u - 45;
            base = pref - __popcll(U >> (u + 19));
          } else {
            emit(key, pos, start, 32 * w + u, pref + __popc(e0 & lowmask(u)) - base);
          }
        }
        open = (g >> hi) & 1u;
        if (w == wlast && open) emit(key, pos, start, iend, pref + __popc(e0 & lowmask(iend - 32 * w)) - base);
        pref += __popc(e0);
        e2 = e1;
        e1 = e0;
      }
    }
    __syncthreads();
  }
  if (tid == 0) P.res_cnt[slot] = s_res;
}

// ---------------------------------------------------------------------------
// Finalize: dense, ordered results
// ---------------------------------------------------------------------------
// dense_base[i] = sum_{j<i} min(cnt[j], slots); dense_base[n] = total.  One CTA.
__global__ void __launch_bounds__(1024) count_scan_kernel(const int* __restrict__ cnt, int n, int slots,
                                                          int* __restrict__ base) {
  __shared__ int s_w[32];
  __shared__ int s_carry;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_carry = 0;
  __syncthreads();
  for (int c0 = 0; c0 < n; c0 += 1024) {
    const int i = c0 + tid;
    const int v = i < n ? min(cnt[i], slots) : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const int x = s_w[lane];
      int y = x;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) y += u;
      }
      s_w[lane] = y - x;
    }
    __syncthreads();
    const int carry = s_carry;
    if (i < n) base[i] = carry + s_w[warp] + incl - v;
    __syncthreads();
    if (tid == 1023) s_carry = carry + s_w[warp] + incl;
    __syncthreads();
  }
  if (tid == 0) base[n] = s_carry;
}

// One warp per pair strand: order its slot records by (offset index, tstart)
// and write them at dense_base.
__global__ void __launch_bounds__(256) gather_sort_kernel(const int* __restrict__ cnt, const DevResult* __restrict__ res,
                                                          int slots, int n, const int* __restrict__ base,
                                                          DevResult* __restrict__ dense) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (gw >= n) return;
  const int c = min(cnt[gw], slots);
  const DevResult* src = res + (size_t)gw * slots;
  DevResult* dst = dense + base[gw];
  for (int r = lane; r < c; r += 32) {
    const DevResult a = src[r];
    int rank = 0;
    for (int q = 0; q < c; q++) {
      const DevResult b = src[q];
      rank += (b.key < a.key) || (b.key == a.key && b.tstart < a.tstart);
    }
    dst[rank] = a;
  }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template <int LOG2L>
static cudaError_t set_attrs() {
  cudaError_t e = cudaFuncSetAttribute(corr_kernel<LOG2L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)corr_smem_bytes(LOG2L));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(scan_kernel<LOG2L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)scan_smem_bytes(LOG2L));
}

cudaError_t prepare_kernels() {
  cudaError_t e;
  if ((e = set_attrs<10>()) != cudaSuccess) return e;
  if ((e = set_attrs<11>()) != cudaSuccess) return e;
  if ((e = set_attrs<12>()) != cudaSuccess) return e;
  if ((e = set_attrs<13>()) != cudaSuccess) return e;
  return set_attrs<14>();
}

cudaError_t launch_corr(int log2L, const CorrParams& p, int npairs, cudaStream_t s) {
  if (npairs <= 0) return cudaSuccess;
  const dim3 grid(npairs, 2);
  const size_t sm = corr_smem_bytes(log2L);
  switch (log2L) {
    case 10: corr_kernel<10><<<grid, NT_CORR, sm, s>>>(p); break;
    case 11: corr_kernel<11><<<grid, NT_CORR, sm, s>>>(p); break;
    case 12: corr_kernel<12><<<grid, NT_CORR, sm, s>>>(p); break;
    case 13: corr_kernel<13><<<grid, NT_CORR, sm, s>>>(p); break;
    case 14: corr_kernel<14><<<grid, NT_CORR, sm, s>>>(p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_scan(int log2L, const ScanParams& p, int npairs, cudaStream_t s) {
  if (npairs <= 0) return cudaSuccess;
  const dim3 grid(npairs, 2);
  const size_t sm = scan_smem_bytes(log2L);
  switch (log2L) {
    case 10: scan_kernel<10><<<grid, NT_SCAN, sm, s>>>(p); break;
    case 11: scan_kernel<11><<<grid, NT_SCAN, sm, s>>>(p); break;
    case 12: scan_kernel<12><<<grid, NT_SCAN, sm, s>>>(p); break;
    case 13: scan_kernel<13><<<grid, NT_SCAN, sm, s>>>(p); break;
    case 14: scan_kernel<14><<<grid, NT_SCAN, sm, s>>>(p); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_finalize(const int* res_cnt, const DevResult* res, int slots, int nslots, int* dense_base,
                            DevResult* dense, int* /*scan_tmp*/, cudaStream_t s) {
  if (nslots <= 0) return cudaSuccess;
  count_scan_kernel<<<1, 1024, 0, s>>>(res_cnt, nslots, slots, dense_base);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int blocks = (nslots * 32 + 255) / 256;
  gather_sort_kernel<<<blocks, 256, 0, s>>>(res_cnt, res, slots, nslots, dense_base, dense);
  return cudaGetLastError();
}

cudaError_t upload_constants(const unsigned char* rc256, const uchar4* w4q128, const double* w4d) {
  cudaError_t e = cudaMemcpyToSymbol(c_rc, rc256, 256);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyToSymbol(c_w4q, w4q128, 128 * sizeof(uchar4));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_wd, w4d, 4 * 128 * sizeof(double));
}

}  // namespace xc
