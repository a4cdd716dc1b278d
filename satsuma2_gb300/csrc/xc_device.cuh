// Device-side building blocks shared by the kernels of the satsuma2
// cross-correlation path: complex helpers, the shared-memory layout of
// transform buffers, register DFTs, the in-place mixed-radix passes and the
// codec constants.  Included by xc_corr.cu and xc_scan.cu (each translation
// unit gets its own copy of the constant tables; upload_constants fills both).
#pragma once
#include "xc_internal.h"

#include <math.h>

namespace xc {

static __constant__ unsigned char c_rc[256];   // DNACodec reverse complement (DNAVector.cc:13-58)
static __constant__ uchar4 c_w4q[128];         // A,C,G,T weights in quarter units (thirds letters: 0)
static __constant__ double c_wd[4][128];       // DNA_A..DNA_T weights (DNAVector.cc:351-369)

static cudaError_t upload_constants_here(const unsigned char* rc256, const uchar4* w4q128, const double* w4d) {
  cudaError_t e = cudaMemcpyToSymbol(c_rc, rc256, 256);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyToSymbol(c_w4q, w4q128, 128 * sizeof(uchar4));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_wd, w4d, 4 * 128 * sizeof(double));
}

// -----------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
// Complex add and subtract as packed FP32x2 instructions (one issue slot for
// both components); multiplies stay scalar FMUL/FFMA, which need no operand
// shuffles.
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
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

// Placement of complex element p in a transform buffer: the 8-byte slot (low
// 4 bits, one of 16 per 128-byte row) is XORed with every higher nibble, so
// the 16 addresses a half-warp touches -- strided by any power of two, or
// consecutive bins in digit-reversed order -- land in distinct banks.  A
// bijection on any power-of-two length >= 16 (only the low nibble changes).
__host__ __device__ constexpr int swz(int p) { return p ^ (((p >> 4) ^ (p >> 8) ^ (p >> 12)) & 15); }
// swz is linear over XOR, so swz(a | b) = swz(a) ^ swz(b) when a and b share no
// set bit; the transform passes use that to turn every access into one XOR
// with a compile-time constant.

// cos(pi m / 16) and sin(pi m / 16) for any integer m, for compile-time twiddles.
__host__ __device__ constexpr float cos_pi16(int m) {
  constexpr float c[9] = {1.0f, 0.98078528040323043f, 0.92387953251128674f, 0.83146961230254524f,
                          0.70710678118654752f, 0.55557023301960218f, 0.38268343236508978f,
                          0.19509032201612826f, 0.0f};
  m &= 31;                       // period 2*pi
  if (m > 16) m = 32 - m;        // cos is even
  return m <= 8 ? c[m] : -c[16 - m];
}
__host__ __device__ constexpr float sin_pi16(int m) { return cos_pi16(8 - m); }

// Twiddle W_N^m from two small shared tables: hi[a] = W_N^(64a), lo[b] = W_N^b.
__device__ __forceinline__ float2 tw2(const float2* hi, const float2* lo, int m) {
  return cmul(hi[m >> 6], lo[m & 63]);
}

// Radix plans (log2 of each pass's radix), shared by the transforms and the
// digit-reversed position of a bin (tests/test_smem_layout.py models them).
template <int LOG2N> struct Plan;
template <int A, int B, int C, int D>
struct PlanR {
  static constexpr int n = D ? 4 : 3;
  __host__ __device__ static constexpr int lr(int s) { return s == 0 ? A : s == 1 ? B : s == 2 ? C : D; }
};
template <> struct Plan<9> : PlanR<3, 3, 3, 0> {};
template <> struct Plan<10> : PlanR<4, 4, 2, 0> {};
template <> struct Plan<11> : PlanR<4, 4, 3, 0> {};
template <> struct Plan<12> : PlanR<4, 4, 4, 0> {};
template <> struct Plan<13> : PlanR<4, 4, 4, 1> {};
template <> struct Plan<14> : PlanR<4, 4, 4, 2> {};

// Position of bin k after the forward (decimation-in-frequency) passes: the
// digit of radix R_s (least significant first in k) moves to place value
// N / (R_0 ... R_s).
template <int LOG2N, class PL = Plan<LOG2N>>
__host__ __device__ constexpr int posof(int k) {
  int p = 0, off = 0, used = 0;
#pragma unroll
  for (int s = 0; s < PL::n; s++) {
    used += PL::lr(s);
    p |= ((k >> off) & ((1 << PL::lr(s)) - 1)) << (LOG2N - used);
    off += PL::lr(s);
  }
  return p;
}

// Shared-memory index of bin k: swz(posof(k)).  Both maps are XOR-linear, so
// lp(a | b) = lp(a) ^ lp(b) for bit-disjoint a and b.
template <int LOG2N, class PL = Plan<LOG2N>>
__host__ __device__ constexpr int lp(int k) { return swz(posof<LOG2N, PL>(k)); }

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

// Twiddles W^(j r), r = 1..15, of a radix-16 pass: W^m and W^(4m) from the
// two-level tables (m = j * N/S), the others by products; about 4 ulp each.
struct Tw16 {
  float2 w1, w2, w3, w4, w8, w12;
};
__device__ __forceinline__ Tw16 tw16(const float2* twh, const float2* twl, int m1) {
  Tw16 t;
  t.w1 = tw2(twh, twl, m1);
  t.w4 = tw2(twh, twl, 4 * m1);
  t.w2 = cmul(t.w1, t.w1);
  t.w3 = cmul(t.w2, t.w1);
  t.w8 = cmul(t.w4, t.w4);
  t.w12 = cmul(t.w8, t.w4);
  return t;
}
// W^(j r) for a compile-time r = 4a + b.
__device__ __forceinline__ float2 tw16_r(const Tw16& t, int r) {
  const int a = r >> 2, bb = r & 3;
  const float2 wa = a == 1 ? t.w4 : a == 2 ? t.w8 : t.w12;
  const float2 wb = bb == 1 ? t.w1 : bb == 2 ? t.w2 : t.w3;
  return a == 0 ? wb : bb == 0 ? wa : cmul(wa, wb);
}

// One forward radix-16 pass of span S over two N-point buffers at once
// (butterfly b of each): the twiddles are generated once for both.  Same
// arithmetic per buffer as fft_pass<16, N, S, false>.
template <int N, int S>
__device__ __forceinline__ void fft_pass16_x2(float2* __restrict__ bufA, float2* __restrict__ bufB,
                                              const float2* __restrict__ twh, const float2* __restrict__ twl,
                                              int b) {
  constexpr int d = S / 16;
  const int j = b & (d - 1);
  const int sb = swz((b - j) * 16 + j);
  float2 xa[16], xb[16];
#pragma unroll
  for (int r = 0; r < 16; r++) {
    xa[r] = bufA[sb ^ swz(r * d)];
    xb[r] = bufB[sb ^ swz(r * d)];
  }
  DFT<16, -1>::run(xa);
  DFT<16, -1>::run(xb);
  if constexpr (d > 1) {
    const Tw16 t = tw16(twh, twl, j * (N / S));
#pragma unroll
    for (int r = 1; r < 16; r++) {
      const float2 w = tw16_r(t, r);
      xa[r] = cmul(xa[r], w);
      xb[r] = cmul(xb[r], w);
    }
  }
#pragma unroll
  for (int r = 0; r < 16; r++) {
    bufA[sb ^ swz(r * d)] = xa[r];
    bufB[sb ^ swz(r * d)] = xb[r];
  }
}

// Twiddles of the radix-16 passes whose butterflies have j < 16 (span S =
// 16 * 16: the forward pass after the first, the inverse pass before the
// last): row j of 17 entries holds W_N^(j r N/S) for r < 16, formed by the
// same products as tw16 / fft_pass, one row per j; the odd row length
// spreads a half-warp's rows over the banks.
constexpr int TW16_ROW = 17;
__device__ __forceinline__ void build_tw16_table(float2* tab, const float2* twh, const float2* twl, int m_step, int t) {
  if (t >= 256) return;
  const int j = t >> 4, r = t & 15;
  const Tw16 tw = tw16(twh, twl, j * m_step);
  const int a = r >> 2, bb = r & 3;
  const float2 wa = a == 1 ? tw.w4 : a == 2 ? tw.w8 : tw.w12;
  const float2 wb = bb == 1 ? tw.w1 : bb == 2 ? tw.w2 : tw.w3;
  tab[j * TW16_ROW + r] = r == 0 ? make_float2(1.f, 0.f) : a == 0 ? wb : bb == 0 ? wa : cmul(wa, wb);
}

// fft_pass16_x2 for span S = 256 (j < 16) with the twiddles from the table.
template <int N, int S>
__device__ __forceinline__ void fft_pass16_x2_tab(float2* __restrict__ bufA, float2* __restrict__ bufB,
                                                  const float2* __restrict__ tab, int b) {
  constexpr int d = S / 16;
  static_assert(d == 16, "table rows are j < 16");
  const int j = b & (d - 1);
  const int sb = swz((b - j) * 16 + j);
  float2 xa[16], xb[16];
#pragma unroll
  for (int r = 0; r < 16; r++) {
    xa[r] = bufA[sb ^ swz(r * d)];
    xb[r] = bufB[sb ^ swz(r * d)];
  }
  DFT<16, -1>::run(xa);
  DFT<16, -1>::run(xb);
  const float2* tr = tab + j * TW16_ROW;
#pragma unroll
  for (int r = 1; r < 16; r++) {
    const float2 w = tr[r];
    xa[r] = cmul(xa[r], w);
    xb[r] = cmul(xb[r], w);
  }
#pragma unroll
  for (int r = 0; r < 16; r++) {
    bufA[sb ^ swz(r * d)] = xa[r];
    bufB[sb ^ swz(r * d)] = xb[r];
  }
}

// fft_pass<16, N, S, false> for span S = 256 (j < 16), butterfly b, with the
// twiddles from the table.
template <int N, int S>
__device__ __forceinline__ void fft_pass16_tab(float2* __restrict__ buf, const float2* __restrict__ tab, int b) {
  constexpr int d = S / 16;
  static_assert(d == 16, "table rows are j < 16");
  const int j = b & (d - 1);
  const int sb = swz((b - j) * 16 + j);
  float2 x[16];
#pragma unroll
  for (int r = 0; r < 16; r++) x[r] = buf[sb ^ swz(r * d)];
  DFT<16, -1>::run(x);
  const float2* tr = tab + j * TW16_ROW;
#pragma unroll
  for (int r = 1; r < 16; r++) x[r] = cmul(x[r], tr[r]);
#pragma unroll
  for (int r = 0; r < 16; r++) buf[sb ^ swz(r * d)] = x[r];
}

// The inverse radix-16 pass of span S = 256 (fft_pass<16, N, 256, true>) for
// butterfly b, its twiddles from the table.
template <int N, int S>
__device__ __forceinline__ void fft_pass16_inv_tab(float2* __restrict__ buf, const float2* __restrict__ tab, int b) {
  constexpr int d = S / 16;
  static_assert(d == 16, "table rows are j < 16");
  const int j = b & (d - 1);
  const int sb = swz((b - j) * 16 + j);
  float2 x[16];
#pragma unroll
  for (int r = 0; r < 16; r++) x[r] = buf[sb ^ swz(r * d)];
  const float2* tr = tab + j * TW16_ROW;
#pragma unroll
  for (int r = 1; r < 16; r++) x[r] = cmulc(x[r], tr[r]);
  DFT<16, 1>::run(x);
#pragma unroll
  for (int r = 0; r < 16; r++) buf[sb ^ swz(r * d)] = x[r];
}

// One in-place pass of span S and radix R over an N-point buffer.
// Forward (decimation in frequency): butterfly, then twiddle W_S^(j r').
// Inverse (decimation in time, the exact reverse): conjugate twiddle, then
// butterfly.  Forward passes in order S = N, N/R0, ... leave bin k at a
// mixed-radix digit-reversed position (pos_of table); the inverse passes in
// reverse order take that layout back to natural order.
template <int R, int N, int S, bool INV>
__device__ __forceinline__ void fft_pass(float2* __restrict__ buf, const float2* __restrict__ twh,
                                         const float2* __restrict__ twl, int t, int nt) {
  constexpr int d = S / R;
  constexpr int B = N / R;
  constexpr int tws = N / S;
  for (int b = t; b < B; b += nt) {
    const int j = b & (d - 1);
    const int base = (b - j) * R + j;   // bits of base and of r*d never overlap
    const int sb = swz(base);
    float2 x[R];
#pragma unroll
    for (int r = 0; r < R; r++) x[r] = buf[sb ^ swz(r * d)];
    if (!INV) DFT<R, -1>::run(x);
    if (d > 1) {
      if constexpr (R == 16) {
        // W^r for r = 4a + b from W^m and W^(4m) (two table lookups): keeps
        // six twiddles live instead of fifteen; about 4 ulp per twiddle.
        const int m1 = j * tws;
        const float2 w1 = tw2(twh, twl, m1), w4 = tw2(twh, twl, 4 * m1);
        const float2 w2 = cmul(w1, w1), w3 = cmul(w2, w1);
        const float2 w8 = cmul(w4, w4), w12 = cmul(w8, w4);
#pragma unroll
        for (int r = 1; r < 16; r++) {
          const int a = r >> 2, bb = r & 3;
          const float2 wa = a == 1 ? w4 : a == 2 ? w8 : w12;
          const float2 wb = bb == 1 ? w1 : bb == 2 ? w2 : w3;
          const float2 w = a == 0 ? wb : bb == 0 ? wa : cmul(wa, wb);
          x[r] = INV ? cmulc(x[r], w) : cmul(x[r], w);
        }
      } else {
#pragma unroll
        for (int r = 1; r < R; r++) x[r] = INV ? cmulc(x[r], tw2(twh, twl, j * r * tws)) : cmul(x[r], tw2(twh, twl, j * r * tws));
      }
    }
    if (INV) DFT<R, 1>::run(x);
#pragma unroll
    for (int r = 0; r < R; r++) buf[sb ^ swz(r * d)] = x[r];
  }
}

template <int LR, int N, int S, bool INV>
__device__ __forceinline__ void pass_lr(float2* buf, const float2* h, const float2* l, int t, int nt) {
  if constexpr (LR == 1) fft_pass<2, N, S, INV>(buf, h, l, t, nt);
  else if constexpr (LR == 2) fft_pass<4, N, S, INV>(buf, h, l, t, nt);
  else if constexpr (LR == 3) fft_pass<8, N, S, INV>(buf, h, l, t, nt);
  else fft_pass<16, N, S, INV>(buf, h, l, t, nt);
}

template <int LOG2N, int s, class PL = Plan<LOG2N>>
__host__ __device__ constexpr int plan_used() {   // sum of the log-radices of passes 0..s-1
  int u = 0;
  for (int i = 0; i < s; i++) u += PL::lr(i);
  return u;
}

// Barriers ending a transform pass: the whole CTA, or a named barrier over
// a warp-aligned group of n threads that transforms its own buffer.
struct CtaBarrier {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct GroupBarrier {
  int id, n;   // id 1..15 (0 is __syncthreads), n a multiple of 32
  __device__ __forceinline__ void operator()() const { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
};

// Forward transform, natural order in, digit-reversed out (posof).  Every
// thread of the barrier's group must call it: each pass ends in the barrier.
template <int LOG2N, int s = 0, class SY = CtaBarrier>
__device__ __forceinline__ void fft_forward(float2* buf, const float2* h, const float2* l, int t, int nt,
                                            SY sync = SY()) {
  if constexpr (s < Plan<LOG2N>::n) {
    pass_lr<Plan<LOG2N>::lr(s), (1 << LOG2N), ((1 << LOG2N) >> plan_used<LOG2N, s>()), false>(buf, h, l, t, nt);
    sync();
    fft_forward<LOG2N, s + 1, SY>(buf, h, l, t, nt, sync);
  }
}

// Inverse (unnormalised), digit-reversed in, natural order out: the forward
// passes undone in reverse order.
template <int LOG2N, class PL = Plan<LOG2N>, int s = PL::n - 1, class SY = CtaBarrier>
__device__ __forceinline__ void fft_inverse(float2* buf, const float2* h, const float2* l, int t, int nt,
                                            SY sync = SY()) {
  if constexpr (s >= 0) {
    pass_lr<PL::lr(s), (1 << LOG2N), ((1 << LOG2N) >> plan_used<LOG2N, s, PL>()), true>(buf, h, l, t, nt);
    sync();
    fft_inverse<LOG2N, PL, s - 1, SY>(buf, h, l, t, nt, sync);
  }
}

// W = h + l + r exactly, three floats (h = float(W), l = float(W - h), r the
// rest, at most a few bits), for mul_round_f32.
struct Split3 {
  float h, l, r;
};
__device__ __forceinline__ Split3 split3(double W) {
  Split3 s;
  s.h = __double2float_rn(W);
  const double d = __dsub_rn(W, (double)s.h);   // exact
  s.l = __double2float_rn(d);
  s.r = __double2float_rn(__dsub_rn(d, (double)s.l));   // exact, representable
  return s;
}

// A channel's mean terms 0 - mean and 1 - mean, mean = count / len as the
// reference forms it in double (CrossCorr.cc:109-123), with cnt4 = 4 count,
// in double and split into three floats.  When len is a power of two and
// count a whole number (a full 4096-base A/C/G/T chunk), count / len and
// (len - count) / len are exact in FP32, so FP32 arithmetic gives the same
// bits as the FP64 division and subtraction, and the split is (value, 0, 0).
__device__ __forceinline__ void mean_terms(int cnt4, int len, double& w0, double& w1, Split3& f0, Split3& f1) {
  if (len > 0 && (len & (len - 1)) == 0 && (cnt4 & 3) == 0 && len <= (1 << 24)) {
    const float inv = __int_as_float((127 - (__ffs(len) - 1)) << 23);   // 2^-k, len = 2^k
    const float m = (float)(cnt4 >> 2) * inv;
    const float a = 0.f - m, b = (float)(len - (cnt4 >> 2)) * inv;
    w0 = (double)a;
    w1 = (double)b;
    f0 = Split3{a, 0.f, 0.f};
    f1 = Split3{b, 0.f, 0.f};
    return;
  }
  const double off = len > 0 ? __ddiv_rn((double)cnt4 * 0.25, (double)len) : 0.0;
  w0 = __dsub_rn(0.0, off);
  w1 = __dsub_rn(1.0, off);
  f0 = split3(w0);
  f1 = split3(w1);
}

// __double2float_rn(__dmul_rn((double)E, W)) without FP64 in the common
// case, for finite E and W with |E*W| >= 2^-100 or zero.  E*W = E*h + E*l +
// E*r is formed as p1 + t to within 2^-45 |E*W| from FMA-exact products; the
// FP32 rounding f of p1 + t then equals the rounding of the double product,
// except within 2^-16 ulp of a rounding boundary (where the double rounding
// may part) or when f is a power of two (a boundary a half-ulp nearer below),
// which take the FP64 product.  Zero keeps the sign the double product has.
__device__ __forceinline__ float mul_round_f32(float E, const Split3& w, double W) {
  const float p1 = __fmul_rn(E, w.h);
  if (p1 == 0.f) return p1;
  const float e1 = __fmaf_rn(E, w.h, -p1);
  const float p2 = __fmul_rn(E, w.l);
  const float e2 = __fmaf_rn(E, w.l, -p2);
  const float p3 = __fmul_rn(E, w.r);
  const float t = __fadd_rn(__fadd_rn(e1, p2), __fadd_rn(e2, p3));
  const float f = __fadd_rn(p1, t);
  const float r = __fadd_rn(__fsub_rn(p1, f), t);   // p1 - f exact
  const uint32_t fb = __float_as_uint(f);
  const float ulp = __uint_as_float((fb & 0x7f800000u) - (23u << 23));
  if ((fb & 0x007fffffu) == 0u || fabsf(r) >= __fmul_rn(ulp, 0.49998f))
    return __double2float_rn(__dmul_rn((double)E, W));
  return f;
}

// Ent (CrossCorr.cc:28-33) for windows holding a one-third IUPAC letter.
__device__ __forceinline__ double ent_dev(double p) {
  if (p < 0.001) return 0.0;
  return __ddiv_rn(__dmul_rn(p, log(p)), 0.69314718056);
}

}  // namespace xc
