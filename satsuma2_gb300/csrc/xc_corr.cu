// Correlation + FindTop kernels of the satsuma2 cross-correlation path (sm_103a).
//
// At FFT 8192, both strands from one set of spectra (A/C/G/T pairs whose
// query windows map onto each other under reverse complement; described at
// corr_pair_kernel):
//   corr_pair2_kernel<13>  persistent, one CTA of 512 threads per SM walking
//                          the pairs (the default);
//   corr_pair_kernel<13>   one CTA of 1024 threads per pair (a tuner form);
//   spec_kernel<13> + corr_spec_kernel<13>  batches whose pairs share chunks:
//                          each distinct chunk transformed once, each pair
//                          correlated from the stored spectra.
// Pairs whose query is >= 1024 bases and not a multiple of the entropy window
// (outside the premise) are placed last in the bucket by the host, or go on
// a second hand-back list, to
//   corr_rcq_kernel<13>    persistent, both strands per CTA, the reverse
//                          complement's spectra computed;
// the other pairs outside it go on a hand-back list to
// corr_kernel<log2 L, NT>: one CTA per (chunk pair, strand), which also runs
// every other FFT length.  Its steps:
//   1. chunk bytes to shared memory; strand 1 reverse-complements the query
//   2. CCSignal: per-window entropy weights and per-channel means
//   3. per channel: z = target_c + i*query_c; the even-bin group (threads
//      0..255) transforms z, the odd-bin group (256..511) z*W_L^n, each an
//      N = L/2 point in-place mixed-radix transform; then the conjugate
//      product of the two spectra is added to the channel sum
//   4. inverse: half-length complex transform of the Hermitian channel sum
//   5. FindTop: envelope per 256 samples, threshold, ordered compaction
// Everything stays in shared memory; HBM sees the chunk bytes in and the
// offset list out.  At L = 32768 the two transforms and the channel sums no
// longer fit one SM: the even and odd transforms then run in turn on all 512
// threads in one buffer, and the channel sums go to a per-strand scratch in
// global memory (128 KB, L2-resident while the CTA runs).  Reference
// semantics cited per step; paths are relative to the satsuma2 source tree.
#include "xc_device.cuh"

#include <algorithm>
#include <type_traits>

namespace xc {

size_t corr_smem_bytes(int log2L) {
  const size_t N = (size_t)1 << (log2L - 1);
  const size_t NH = N / 64;
  const size_t bufs = log2L > MAX_SMEM_LOG2L ? N : 2 * N + (N / 2 + 8) + N / 2;   // transforms (+ sums)
  return (bufs + 2 * (NH + 64)) * sizeof(float2)                         // and twiddles
         + 2 * N                                                         // target and query bytes
         + 2 * 256 * sizeof(float)                                       // entropy weight per window
         + 2 * 256 * sizeof(float2);                                     // per-window channel values
}

// ---------------------------------------------------------------------------
// Steps shared by both correlation kernels
// ---------------------------------------------------------------------------

// Step 4: the half-length complex array of the Hermitian sum S (bins
// k = 0..N of the L-point spectrum, N = L/2; S2(k, a, b) gives a = S(k) and
// b = S(N-k)), ready for the N-point inverse: Z(k) = E(k) + i O(k),
// E = (S(k) + conj S(N-k))/2, O = (S(k) - conj S(N-k)) conj(W_L^k)/2; the
// inverse then holds z[m] = r[2m] + i r[2m+1].  W_L^(N-k) = -conj(W_L^k)
// (W_L^N = -1), so one twiddle serves both bins.  Threads t < NTF.
// HALF = 0.5f as written; the both-strands pair kernel passes 1.0f (its
// inverse then carries a power of two, which FindTop's scale removes
// exactly).
template <int LOG2L, int NTF = NT_CORR, class SF>
__device__ __forceinline__ void hermitian_pack(float2* __restrict__ buf, const SF& S2, const float2* twLh,
                                               const float2* twLl, int t, float HALF = 0.5f) {
  constexpr int N = 1 << (LOG2L - 1);
  constexpr int LOG2N = LOG2L - 1;
  const int la = lp<LOG2N>(t);
  const int lb = lp<LOG2N>((NTF - t) & (NTF - 1));
#pragma unroll
  for (int it = 0; it <= N / (2 * NTF); it++) {
    const int k = t + NTF * it;
    if (k > N / 2) break;
    float2 Sk, Sn;
    S2(k, Sk, Sn);
    const float2 w = tw2(twLh, twLl, k);   // W_L^k
    {
      const float2 Ev = make_float2(HALF * (Sk.x + Sn.x), HALF * (Sk.y - Sn.y));
      const float2 Dv = make_float2(HALF * (Sk.x - Sn.x), HALF * (Sk.y + Sn.y));
      const float2 Ov = cmulc(Dv, w);
      buf[la ^ lp<LOG2N>(NTF * it)] = make_float2(Ev.x - Ov.y, Ev.y + Ov.x);
    }
    if (k != 0 && k != N / 2) {
      // N-k = (N - NTF(it+1)) | (NTF - t) for t >= 1
      const int pb = t ? (lb ^ lp<LOG2N>(N - NTF * (it + 1))) : lp<LOG2N>(N - NTF * it);
      const float2 Ev = make_float2(HALF * (Sn.x + Sk.x), HALF * (Sn.y - Sk.y));
      const float2 Dv = make_float2(HALF * (Sn.x - Sk.x), HALF * (Sn.y + Sk.y));
      const float2 Ov = cmulc(Dv, make_float2(-w.x, w.y));   // W_L^(N-k)
      buf[pb] = make_float2(Ev.x - Ov.y, Ev.y + Ov.x);
    }
  }
}

// S2 for hermitian_pack from a per-bin S(k).
template <int N, class SF>
struct BothBins {
  const SF& S;
  __device__ __forceinline__ void operator()(int k, float2& a, float2& b) const {
    a = S(k);
    b = S(N - k);
  }
};
template <int N, class SF>
__device__ __forceinline__ BothBins<N, SF> both_bins(const SF& S) {
  return BothBins<N, SF>{S};
}

// Step 5: FindTop (SeqAnalyzer::FindTop, CrossCorr.cc:878-944) over the
// inverse in buf, for one strand: xc[i] = r[(i + N) mod L] / N; envelope
// over 256-sample blocks when L/256 > 8; keep i with xc[i] > env*cutoff + 1
// in increasing i.  Threads t < NTF; warp w of them owns the contiguous
// range [w*L/(NTF/32), (w+1)*L/(NTF/32)) in steps of 64 lags, lane l taking
// lags 2l and 2l+1 of a step (one complex value of the inverse).  Every
// thread of the barrier's group calls it (two barriers).  s_warp holds
// 2 * NTF/32 ints.  scale is 1/N for an inverse of the spectrum itself (a
// power of two smaller when the inverse carries a power-of-two factor).
//
// Near-threshold lags: with P.strad_cnt set, every lag whose FP32 value lies
// within straddle_rel(L) * max(1, max|xc|) of its FP32 threshold is counted
// in strad_cnt[pair*2+strand] and the first STRAD_CAP of them are listed.
// There the reference's FP32 FFT and this one may decide differently; every
// other lag's decision is the same for both.  A warp walks its lags for
// them only when one of its lanes saw a lag that close.
template <int LOG2L, int NTF = NT_CORR, class SY = CtaBarrier, int KMAX = (NTF <= 256 ? 32 : 16)>
__device__ __forceinline__ void find_top(const CorrParams& P, uint32_t flags, uint32_t off_base, int pidx,
                                         int strand, const float2* __restrict__ buf, int t, int* s_warp,
                                         SY sync = SY(), float scale = 1.0f / (float)(1 << (LOG2L - 1))) {
  constexpr int L = 1 << LOG2L;
  constexpr int N = L >> 1;
  constexpr int NW = NTF / 32;   // warps of the group
  const int lane = t & 31, warp = t >> 5;
  constexpr int PER_WARP = L / NW;
  constexpr int ITER = PER_WARP / 64;   // steps of 64 lags
  static_assert(PER_WARP % 64 == 0, "a warp's range is whole steps");
  constexpr bool ENV = L / 256 > 8;
  static_assert(!ENV || PER_WARP % 256 == 0, "envelope blocks lie within one warp's range");
  const int wbase = warp * PER_WARP;
  // lags wbase + 64 e + 2 lane and the one after (even n: one complex value)
  auto xpair = [&](int e) -> float2 {
    const int n = (wbase + 64 * e + 2 * lane + N) & (L - 1);
    const float2 z = buf[swz(n >> 1)];
    return make_float2(z.x * scale, z.y * scale);
  };
  // Up to KMAX values a lane's values stay in registers across the passes
  // (envelope, count, compaction); more are re-read from the buffer.
  constexpr bool KEEP = 2 * ITER <= KMAX;
  float2 xs[KEEP ? ITER : 1];
  if constexpr (KEEP) {
#pragma unroll
    for (int e = 0; e < ITER; e++) xs[e] = xpair(e);
  }
  auto xat = [&](int e) -> float2 {
    if constexpr (KEEP) return xs[e];
    else return xpair(e);
  };
  float thrb[ENV ? PER_WARP / 256 : 1];
  if constexpr (ENV) {
    const float cut = (float)((flags & PF_FAST) ? P.cutoff_fast : P.cutoff);
#pragma unroll
    for (int bb = 0; bb < PER_WARP / 256; bb++) {
      // squares are float products as in the reference; compensated FP32
      // sum per lane (its eight lags of the block), pairwise across the warp
      float s = 0.f, comp = 0.f;
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const float2 x2 = xat(bb * 4 + e);
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const float x = h ? x2.y : x2.x;
          const float v = __fmul_rn(x, x);
          const float y = __fsub_rn(v, comp);
          const float t2 = __fadd_rn(s, y);
          comp = __fsub_rn(__fsub_rn(t2, s), y);
          s = t2;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        s = __fadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
        comp = __fadd_rn(comp, __shfl_xor_sync(0xffffffffu, comp, o));
      }
      // env = sqrt(sum / 256) and the threshold env * cutoff + 1 in FP32.
      // The reference forms them in double from its own FP32 xc; ours
      // differ from them by a few FP32 ulps, the order of the difference
      // between the two FP32 correlations themselves, so decisions can
      // only part within that band around the threshold.  (FP64 would cost
      // tens of cycles per warp instruction here.)
      const float env = __fsqrt_rn(__fmul_rn(__fsub_rn(s, comp), 0.00390625f));
      thrb[bb] = __fadd_rn(__fmul_rn(env, cut), 1.0f);
    }
  } else {
    thrb[0] = 1.0f;
  }
  auto thr_of = [&](int e) -> float { return thrb[ENV ? (e >> 2) : 0]; };
  int wcount = 0;
  float amax = 0.f;      // max |xc| of the lane's lags (for the near-threshold band)
  float dmin = 3.0e38f;  // min |xc - threshold| of the lane's lags
  constexpr bool KEEPM = KEEP && ITER <= 16;   // ballots kept too (registers allowing)
  unsigned msk[KEEPM ? 2 * ITER : 1];
#pragma unroll(KEEP ? ITER : 4)
  for (int e = 0; e < ITER; e++) {
    const float2 x = xat(e);
    const float thr = thr_of(e);
    const unsigned me = __ballot_sync(0xffffffffu, x.x > thr), mo = __ballot_sync(0xffffffffu, x.y > thr);
    if constexpr (KEEPM) {
      msk[2 * e] = me;
      msk[2 * e + 1] = mo;
    }
    wcount += __popc(me) + __popc(mo);
    amax = fmaxf(amax, fmaxf(fabsf(x.x), fabsf(x.y)));
    dmin = fminf(dmin, fminf(fabsf(x.x - thr), fabsf(x.y - thr)));
    if (P.dbg_xc)
      *reinterpret_cast<float2*>(P.dbg_xc + (size_t)(pidx * 2 + strand) * L + wbase + 64 * e + 2 * lane) = x;
  }
  int* s_max = s_warp + NW;   // max |xc| bits per warp (non-negative floats order as ints)
  if (P.strad_cnt) {
    const unsigned mb = __reduce_max_sync(0xffffffffu, __float_as_uint(amax));
    if (lane == 0) s_max[warp] = (int)mb;
  }
  if (lane == 0) s_warp[warp] = wcount;
  sync();
  if (warp == 0) {
    const int v = lane < NW ? s_warp[lane] : 0;
    int w = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    if (lane < NW) s_warp[lane] = w - v;
    if (lane == NW - 1) P.off_cnt[pidx * 2 + strand] = w;
  }
  sync();
  int run = s_warp[warp];
  float band = -1.f;   // no near-threshold lags without a list
  if (P.strad_cnt) {
    unsigned mb = 0u;
#pragma unroll
    for (int k = 0; k < NW; k++) mb = max(mb, (unsigned)s_max[k]);
    band = straddle_rel(LOG2L) * fmaxf(1.0f, __uint_as_float(mb));
  }
  int* out = P.off_list + off_base + (size_t)strand * L;
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll(KEEP ? ITER : 4)
  for (int e = 0; e < ITER; e++) {
    const int i = wbase + 64 * e + 2 * lane;
    unsigned me, mo;
    if constexpr (KEEPM) {
      me = msk[2 * e];
      mo = msk[2 * e + 1];
    } else {
      const float2 x = xat(e);
      const float thr = thr_of(e);
      me = __ballot_sync(0xffffffffu, x.x > thr);
      mo = __ballot_sync(0xffffffffu, x.y > thr);
    }
    const unsigned be = (me >> lane) & 1u;
    const int k = run + __popc(me & lt) + __popc(mo & lt);
    if (be) out[k] = i;
    if ((mo >> lane) & 1u) out[k + (int)be] = i + 1;
    run += __popc(me) + __popc(mo);
  }
  if (__any_sync(0xffffffffu, dmin <= band)) {
#pragma unroll(KEEP ? ITER : 4)
    for (int e = 0; e < ITER; e++) {
      const float2 x = xat(e);
      const float thr = thr_of(e);
      const unsigned ne = __ballot_sync(0xffffffffu, fabsf(x.x - thr) <= band);
      const unsigned no = __ballot_sync(0xffffffffu, fabsf(x.y - thr) <= band);
      if (ne | no) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&P.strad_cnt[pidx * 2 + strand], __popc(ne) + __popc(no));
        base = __shfl_sync(0xffffffffu, base, 0);
        const unsigned be = (ne >> lane) & 1u;
        const int k = base + __popc(ne & lt) + __popc(no & lt);
        const int i = wbase + 64 * e + 2 * lane;
        int* lst = P.strad_list + (size_t)(pidx * 2 + strand) * STRAD_CAP;
        if (be && k < STRAD_CAP) lst[k] = i;
        if (((no >> lane) & 1u) && k + (int)be < STRAD_CAP) lst[k + (int)be] = i + 1;
      }
    }
  }
}

// One (pair, strand) on the CTA's NT threads (512, or 256 / 128 at short FFT
// lengths, where more CTAs then share an SM; the autotuner picks per length);
// each of the two transform groups has NT/2 threads.  slot indexes the global
// channel-sum scratch at L = 32768.
template <int LOG2L, int NT>
__device__ __forceinline__ void corr_strand(const CorrParams& P, int pidx, int slot, int strand,
                                            unsigned char* smem) {
  constexpr int L = 1 << LOG2L;
  constexpr int N = L >> 1;
  constexpr int LOG2N = LOG2L - 1;
  constexpr int WIN = L / 512;   // CCSignal::ComputeEntropy window (CrossCorr.cc:46)
  constexpr int NWIN = 256;      // N / WIN
  constexpr int NH = N / 64;
  constexpr bool SEQ = LOG2L > MAX_SMEM_LOG2L;   // one transform buffer, channel sums in global memory

  float2* bufE = reinterpret_cast<float2*>(smem);
  float2* bufO = bufE + N;              // (not SEQ)
  float2* accE = bufO + N;              // channel sum at bins 2m, m = 0..N/2 (N/2: Nyquist, real)
  float2* accO = accE + (N / 2 + 8);    // bins 2m+1, m < N/2; 8 slots off accE's banks
  float2* twNh = SEQ ? bufE + N : accO + N / 2;   // W_N^(64a)
  float2* twNl = twNh + NH;             // W_N^b, b < 64
  float2* twLh = twNl + 64;             // W_L^(64a)
  float2* twLl = twLh + NH;             // W_L^b
  uint8_t* st = reinterpret_cast<uint8_t*>(twLl + 64);
  uint8_t* sq = st + N;
  float* Et = reinterpret_cast<float*>(sq + N);
  float* Eq = Et + NWIN;
  float2* vt = reinterpret_cast<float2*>(Eq + NWIN);
  float2* vq = vt + NWIN;
  __shared__ int s_cnt4[8];
  __shared__ double s_off[8];
  __shared__ double s_wmo[2][8];   // 0 - mean and 1 - mean per (sequence, channel)
  __shared__ Split3 s_wf[2][8];    // the same as three floats each
  __shared__ int s_warp[2 * NT / 32];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const PairDesc D = P.pairs[pidx];
  const int T = D.tlen, Q = D.qlen;
  const uint8_t* __restrict__ gt = P.pool + D.t_off;
  const uint8_t* __restrict__ gq = P.pool + D.q_off;

  // ---- 1. chunk bytes (DNAVector::ReverseComplement, DNAVector.cc:482-500) ----
  int high = 0, nonacgt = 0, th_t = 0, th_q = 0;
  for (int i = tid; i < N; i += NT) {
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
  for (int i = tid; i < NH; i += NT) {
    twNh[i] = P.tab.twN_hi[i];
    twLh[i] = P.tab.twL_hi[i];
  }
  if (tid < 64) {
    twNl[tid] = P.tab.twN_lo[tid];
    twLl[tid] = P.tab.twL_lo[tid];
  }
  if (tid < 8) s_cnt4[tid] = 0;
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
  if constexpr (!SEQ)
    for (int i = tid; i < N + 8; i += NT) accE[i] = make_float2(0.f, 0.f);   // accE and accO
  float2* gaccE = nullptr;   // SEQ: this strand's channel sums in global memory
  float2* gaccO = nullptr;
  if constexpr (SEQ) {
    gaccE = P.acc + (size_t)(slot * 2 + strand) * acc_stride(LOG2L);
    gaccO = gaccE + (N / 2 + 8);
  }

  // ---- 2a. entropy weight per window (CCSignal::ComputeEntropy, CrossCorr.cc:35-93).
  //      Threads 0..255: target windows, 256..511: query windows.  Windows
  //      without one-third letters have exact quarter-unit base sums, so Ent
  //      comes from a table the host computed with the same double
  //      expression; others repeat the reference's double arithmetic here. ----
  for (int x = tid; x < 2 * NWIN; x += NT) {
    const int which = x >> 8, w = x & 255;
    const uint8_t* s = which ? sq : st;
    const int len = which ? Q : T;
    const int third = which ? th_q : th_t;
    float E = 0.f;
    if (len < 1024) {
      E = 1.f;
    } else if (!generic && w * WIN + WIN <= len) {
      // A/C/G/T pair, full window: base counts from the 2-bit codes (one
      // 8-bit field per base), weight from the host table
      const int i0 = w * WIN;
      uint32_t cnt = 0;
      for (int j = 0; j < WIN; j++) cnt += 1u << (8 * code_of(s[i0 + j]));
      const int a = cnt & 255u, c = (cnt >> 8) & 255u, g = (cnt >> 16) & 255u;
      E = __ldg(&P.tab.ent_acgt[(a * (WIN + 1) + c) * (WIN + 1) + g]);
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

  // ---- 2b. channel means (SeqToPCM, CrossCorr.cc:108-116): exact quarter-unit
  //      sums, or the sequential double sum when one-third letters occur ----
  {
    int cn[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (!generic) {
      // A/C/G/T: one 8-bit count field per base (at most N / 512 <= 32 per thread)
      uint32_t ct = 0, cq = 0;
      for (int i = tid; i < N; i += NT) {
        if (i < T) ct += 1u << (8 * code_of(st[i]));
        if (i < Q) cq += 1u << (8 * code_of(sq[i]));
      }
#pragma unroll
      for (int k = 0; k < 4; k++) {
        cn[k] = 4 * (int)((ct >> (8 * k)) & 255u);
        cn[4 + k] = 4 * (int)((cq >> (8 * k)) & 255u);
      }
    } else {
      for (int i = tid; i < N; i += NT) {
        if (i < T) { const uchar4 q = c_w4q[st[i]]; cn[0] += q.x; cn[1] += q.y; cn[2] += q.z; cn[3] += q.w; }
        if (i < Q) { const uchar4 q = c_w4q[sq[i]]; cn[4] += q.x; cn[5] += q.y; cn[6] += q.z; cn[7] += q.w; }
      }
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int v = __reduce_add_sync(0xffffffffu, cn[k]);
      if (lane == 0 && v) atomicAdd(&s_cnt4[k], v);
    }
  }
  __syncthreads();
  if (tid < 8) {
    const int which = tid >> 2, c = tid & 3;
    const int len = which ? Q : T;
    const int third = which ? th_q : th_t;
    if (!third) {
      mean_terms(s_cnt4[tid], len, s_wmo[0][tid], s_wmo[1][tid], s_wf[0][tid], s_wf[1][tid]);
      s_off[tid] = __dsub_rn(0.0, s_wmo[0][tid]);   // the mean itself, exact
    } else {
      double off = 0.0;
      if (len > 0) {
        const uint8_t* s = which ? sq : st;
        double sum = 0.0;
        for (int i = 0; i < len; i++) sum = __dadd_rn(sum, c_wd[c][s[i]]);
        off = __ddiv_rn(sum, (double)len);
      }
      s_off[tid] = off;
      s_wmo[0][tid] = __dsub_rn(0.0, off);
      s_wmo[1][tid] = __dsub_rn(1.0, off);
      s_wf[0][tid] = split3(s_wmo[0][tid]);
      s_wf[1][tid] = split3(s_wmo[1][tid]);
    }
  }
  __syncthreads();

  constexpr int HG = NT / 2;   // threads of a transform group
  const int grp = tid / HG;    // 0: even-bin transform, 1: odd-bin transform
  const int gtid = tid % HG;

  for (int c = 0; c < 4; c++) {
    // Per-window channel values: out = float(entropy * (weight - mean))
    // (CrossCorr.cc:123), weight 0 or 1 for A/C/G/T.
    if (!generic) {
      for (int w = gtid; w < NWIN; w += HG) {
        const float E = (grp ? Eq : Et)[w];
        const int k = grp * 4 + c;
        float2 v;
        v.x = mul_round_f32(E, s_wf[0][k], s_wmo[0][k]);
        v.y = mul_round_f32(E, s_wf[1][k], s_wmo[1][k]);
        (grp ? vq : vt)[w] = v;
      }
    }
    __syncthreads();

    if constexpr (SEQ) {
      // ---- 3 (L = 32768): the even-bin transform of z, then the odd-bin
      //      transform of z*W_L^n, each on all threads in one buffer; the
      //      per-bin products go to the global channel sums (set on channel
      //      0, added after). ----
      const double offt = s_off[c], offq = s_off[4 + c];
      const int stid = swz(tid);
      for (int g = 0; g < 2; g++) {
#pragma unroll 4
        for (int it = 0; it < N / NT; it++) {
          const int n = tid + NT * it;
          float x = 0.f, y = 0.f;
          const int w = n / WIN;
          if (!generic) {
            if (n < T) { const float2 v = vt[w]; x = code_of(st[n]) == (uint32_t)c ? v.y : v.x; }
            if (n < Q) { const float2 v = vq[w]; y = code_of(sq[n]) == (uint32_t)c ? v.y : v.x; }
          } else {
            if (n < T) x = __double2float_rn(__dmul_rn((double)Et[w], __dsub_rn(c_wd[c][st[n]], offt)));
            if (n < Q) y = __double2float_rn(__dmul_rn((double)Eq[w], __dsub_rn(c_wd[c][sq[n]], offq)));
          }
          if (P.dbg_sig && g == 0) {
            float* ds = P.dbg_sig + (size_t)(pidx * 2 + strand) * 8 * L;
            ds[(size_t)c * L + n] = x;
            ds[(size_t)(4 + c) * L + n] = y;
          }
          const float2 z = make_float2(x, y);
          bufE[stid ^ swz(NT * it)] = g ? cmul(z, tw2(twLh, twLl, n)) : z;
        }
        __syncthreads();
        fft_forward<LOG2N>(bufE, twNh, twNl, tid, NT);
        if (g == 0) {
          for (int m = tid; m <= N / 2; m += NT) {
            const float2 A = bufE[lp<LOG2N>(m)];
            const float2 B = bufE[lp<LOG2N>((N - m) & (N - 1))];
            const float2 X = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
            const float2 Y = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
            const float2 v = m == N / 2 ? make_float2(X.x, 0.f) : cmulc(Y, X);
            gaccE[m] = c ? cadd(gaccE[m], v) : v;
          }
        } else {
          for (int m = tid; m < N / 2; m += NT) {
            const float2 A = bufE[lp<LOG2N>(m)];
            const float2 B = bufE[lp<LOG2N>(N - 1 - m)];
            const float2 X = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
            const float2 Y = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
            const float2 v = m == N / 2 - 1 ? X : cmulc(Y, X);
            gaccO[m] = c ? cadd(gaccO[m], v) : v;
          }
        }
        __syncthreads();
      }
      continue;
    }

    // ---- 3. z[n] = target_c[n] + i*query_c[n] to the even buffer and
    //      z[n]*W_L^n to the odd buffer.  Both signals are zero past N, so the
    //      even bins of the L-point transform are the N-point transform of z
    //      and the odd bins that of z*W_L^n.  W_L^n = W_L^tid * W_L^(512 it):
    //      one per-thread twiddle times a compile-time constant. ----
    {
      const double offt = s_off[c], offq = s_off[4 + c];
      const int stid = swz(tid);
      const float2 wt = tw2(twLh, twLl, tid);
#pragma unroll
      for (int it = 0; it < N / NT; it++) {
        const int n = tid + NT * it;
        float x = 0.f, y = 0.f;
        const int w = n / WIN;
        if (!generic) {
          if (n < T) { const float2 v = vt[w]; x = code_of(st[n]) == (uint32_t)c ? v.y : v.x; }
          if (n < Q) { const float2 v = vq[w]; y = code_of(sq[n]) == (uint32_t)c ? v.y : v.x; }
        } else {
          if (n < T) x = __double2float_rn(__dmul_rn((double)Et[w], __dsub_rn(c_wd[c][st[n]], offt)));
          if (n < Q) y = __double2float_rn(__dmul_rn((double)Eq[w], __dsub_rn(c_wd[c][sq[n]], offq)));
        }
        if (P.dbg_sig) {
          float* ds = P.dbg_sig + (size_t)(pidx * 2 + strand) * 8 * L;
          ds[(size_t)c * L + n] = x;
          ds[(size_t)(4 + c) * L + n] = y;
        }
        const int sn = stid ^ swz(NT * it);   // tid and NT*it share no bit
        // W_L^(NT it) = exp(-i pi (32 NT it / L) / 16)
        const float2 wc = make_float2(cos_pi16((32 * NT / L) * it), -sin_pi16((32 * NT / L) * it));
        bufE[sn] = make_float2(x, y);
        bufO[sn] = cmul(make_float2(x, y), cmul(wt, wc));
      }
    }
    __syncthreads();

    fft_forward<LOG2N>(grp ? bufO : bufE, twNh, twNl, gtid, HG);

    // Per-bin product (CrossCorrelation::DoOne, CrossCorr.cc:477-492):
    // X = target spectrum, Y = query spectrum from Z(k), Z(L-k).
    // conj(X)Y on bins 1..N-2, X(0)Y(0) on bin 0, and the target's own value
    // on bins N-1 and N, which the reference's loop leaves unmultiplied.
    // Addresses: swz(posof(.)) is XOR-linear, so for m = gtid + HG*it it is
    // lp(gtid) ^ lp(HG*it) with the second term a compile-time constant.
    if (grp == 0) {
      const int la = lp<LOG2N>(gtid);
      const int lb = lp<LOG2N>((HG - gtid) & (HG - 1));
#pragma unroll
      for (int it = 0; it <= N / (2 * HG); it++) {
        const int m = gtid + HG * it;
        if (m > N / 2) break;
        // partner N-m = (N - HG(it+1)) | (HG - gtid) for gtid >= 1
        const int pb = gtid ? (lb ^ lp<LOG2N>(N - HG * (it + 1))) : lp<LOG2N>((N - HG * it) & (N - 1));
        const float2 A = bufE[la ^ lp<LOG2N>(HG * it)];
        const float2 B = bufE[pb];
        const float2 X = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
        const float2 Y = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
        if (m == N / 2) accE[m].x += X.x;
        else accE[m] = cadd(accE[m], cmulc(Y, X));
      }
    } else {
      const int la = lp<LOG2N>(gtid);
#pragma unroll
      for (int it = 0; it < N / (2 * HG); it++) {
        const int m = gtid + HG * it;
        const int pa = la ^ lp<LOG2N>(HG * it);
        const float2 A = bufO[pa];
        const float2 B = bufO[pa ^ lp<LOG2N>(N - 1)];   // N-1-m = m ^ (N-1)
        const float2 X = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
        const float2 Y = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
        accO[m] = cadd(accO[m], m == N / 2 - 1 ? X : cmulc(Y, X));
      }
    }
    __syncthreads();
  }

  // ---- 4. inverse: half-length complex transform of the Hermitian sum S.
  //      Z(k) = E(k) + i O(k), E = (S(k) + conj S(N-k))/2,
  //      O = (S(k) - conj S(N-k)) conj(W_L^k)/2; z[m] = r[2m] + i r[2m+1]. ----
  auto S = [&](int k) -> float2 {
    if constexpr (SEQ) return (k & 1) ? gaccO[k >> 1] : gaccE[k >> 1];
    return (k & 1) ? accO[k >> 1] : accE[k >> 1];
  };
  hermitian_pack<LOG2L, NT>(bufE, both_bins<N>(S), twLh, twLl, tid);
  __syncthreads();
  fft_inverse<LOG2N>(bufE, twNh, twNl, tid, NT);

  // ---- 5. FindTop ----
  find_top<LOG2L, NT, CtaBarrier, 16>(P, D.flags, D.off_base, pidx, strand, bufE, tid, s_warp);
}

// Resident CTAs per SM the register budget is set for (64 registers per thread).
__host__ __device__ constexpr int corr_min_blocks(int log2L, int nt) { return log2L <= 13 ? 1024 / nt : 1; }

template <int LOG2L, int NT = NT_CORR>
__global__ void __launch_bounds__(NT, corr_min_blocks(LOG2L, NT)) corr_kernel(const CorrParams P) {
  static_assert(NT == 512 || (NT >= 128 && 32 * NT % (1 << LOG2L) == 0 && LOG2L <= 13),
                "fewer threads per strand only where W_L^(NT it) is a multiple of pi/16");
  extern __shared__ __align__(16) unsigned char smem[];
  // One pair per CTA column, or (fb_list) the pairs corr_pair_kernel handed
  // back, CTA columns striding over the list.
  const int cnt = P.fb_list ? *P.fb_cnt : (int)blockIdx.x + 1;
  for (int j = blockIdx.x; j < cnt; j += gridDim.x) {
    const int pidx = P.fb_list ? P.fb_list[j] : P.first + j;
    if (P.fb_list && P.strad_cnt && threadIdx.x == 0) {
      // a pair corr_rcq_kernel passed on after a void pass may hold its count
      P.strad_cnt[pidx * 2 + blockIdx.y] = 0;
    }
    __syncthreads();
    corr_strand<LOG2L, NT>(P, pidx, j, blockIdx.y, smem);
    __syncthreads();
  }
}

size_t corr_pair_smem_bytes(int log2L) {
  const size_t N = (size_t)1 << (log2L - 1);
  const size_t NH = N / 64;
  return (4 * N + 2 * (N + 8) + 2 * (NH + 64)) * sizeof(float2)   // transforms, two sums, twiddles
         + 2 * N                                                    // target and query bytes
         + 2 * 256 * sizeof(float)                                  // entropy weight per window
         + 4 * 256 * sizeof(float2);                                // per-window channel values
}

// corr_pair_kernel<log2 L>: one CTA of 1024 threads per chunk pair, both
// strands from one set of spectra.  For A/C/G/T chunks the reverse strand's
// query signal in channel c is the forward query's signal in the complement
// channel comp(c), reversed in time: the per-channel means are equal (the
// same base counts), and when the query length is a multiple of the entropy
// window (or below 1024, weight 1) every reverse window holds the complement
// bases of one forward window, whose weight the host table gives identically
// (the host checks the table's complement symmetry before enabling this
// kernel).  With q_r[n] = q_comp[Q-1-n], Q_r(k) = W_L^((Q-1)k) conj(Q_comp(k)),
// so the reverse strand's product sum is
//   sum_c conj(T_c) Q_r,c = W_L^((Q-1)k) conj(R(k)),  R = sum_c T_c Q_comp(c).
// Channels go in two stages, (A, T) then (C, G): z = t_c0 + i t_c1 and
// w = q_c0 + i q_c1, each as its even-bin and odd-bin N-point transform, the
// four on 256 threads each; the per-bin step separates T_c0, T_c1, Q_c0,
// Q_c1 and adds conj(T_c)Q_c to the forward sum and T_c0 Q_c1 + T_c1 Q_c0
// to R.  Eight N-point transforms and two inverses per pair, where two
// corr_kernel CTAs take sixteen and two.  Pairs outside that case (a byte
// other than A/C/G/T, a ragged query window, debug signal output) go on
// P.fb_list for corr_kernel; pairs with a byte >= 128 are rejected here.
template <int LOG2L>
__global__ void __launch_bounds__(NT_PAIR, 1) corr_pair_kernel(const CorrParams P) {
  constexpr int L = 1 << LOG2L;
  constexpr int N = L >> 1;
  constexpr int LOG2N = LOG2L - 1;
  constexpr int WIN = L / 512;
  constexpr int NWIN = 256;
  constexpr int NH = N / 64;
  static_assert(N % 1024 == 0, "two 512-thread halves over N/2 bins");

  extern __shared__ __align__(16) unsigned char smem[];
  float2* ZE = reinterpret_cast<float2*>(smem);   // z = t_c0 + i t_c1, even-bin transform
  float2* ZO = ZE + N;                            // z * W_L^n, odd-bin transform
  float2* WE = ZO + N;                            // w = q_c0 + i q_c1
  float2* WO = WE + N;
  float2* aFE = WO + N;                           // forward-strand sum, bins 2m, m <= N/2
  float2* aFO = aFE + (N / 2 + 8);                // bins 2m+1
  float2* aRE = aFO + N / 2;                      // R, bins 2m (m < N/2)
  float2* aRO = aRE + (N / 2 + 8);                // R, bins 2m+1
  float2* twNh = aRO + N / 2;
  float2* twNl = twNh + NH;
  float2* twLh = twNl + 64;
  float2* twLl = twLh + NH;
  uint8_t* st = reinterpret_cast<uint8_t*>(twLl + 64);
  uint8_t* sq = st + N;
  float* Et = reinterpret_cast<float*>(sq + N);
  float* Eq = Et + NWIN;
  float2* vv = reinterpret_cast<float2*>(Eq + NWIN);   // [t c0, t c1, q c0, q c1][window]
  __shared__ int s_cnt4[8];
  __shared__ double s_wmo[2][8];   // 0 - mean and 1 - mean per (sequence, channel)
  __shared__ Split3 s_wf[2][8];    // the same as three floats each
  __shared__ int s_warp[2][2 * NT_CORR / 32];

  const int tid = threadIdx.x;
  const int half = tid >> 9;       // steps 3b-5: 0 target / forward strand, 1 query / reverse strand
  const int ht = tid & 511;
  const int pidx = P.first + blockIdx.x;
  const int T = P.pairs[pidx].tlen, Q = P.pairs[pidx].qlen;
  const uint8_t* __restrict__ gt = P.pool + P.pairs[pidx].t_off;
  const uint8_t* __restrict__ gq = P.pool + P.pairs[pidx].q_off;

  // ---- 1. chunk bytes, forward strand only: threads 0..N/16-1 take one
  //      16-byte piece of the target each, the next N/16 one of the query
  //      (pool chunks are 16-byte aligned and padded to 16); bytes past the
  //      chunk end are zeroed.  Per byte, exactly: (y & 0x7f) + 0x7f | y has
  //      bit 7 clear iff y == 0. ----
  static_assert(2 * (N / 16) <= NT_PAIR, "one 16-byte piece per thread");
  int high = 0, nonacgt = 0;
  if (tid < 2 * (N / 16)) {
    const int which = tid / (N / 16), c = tid % (N / 16);
    const int len = which ? Q : T;
    const int valid = len - 16 * c;   // bytes of this piece inside the chunk
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (valid > 0) v = *reinterpret_cast<const uint4*>((which ? gq : gt) + 16 * c);
    uint32_t x[4] = {v.x, v.y, v.z, v.w};
    auto nz = [](uint32_t y) { return (((y & 0x7f7f7f7fu) + 0x7f7f7f7fu) | y) & 0x80808080u; };
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int vk = min(max(valid - 4 * k, 0), 4);
      const uint32_t m = vk >= 4 ? 0xffffffffu : (1u << (8 * vk)) - 1u;
      x[k] &= m;
      high |= (x[k] & 0x80808080u) != 0u;
      const uint32_t bad = nz(x[k] ^ 0x41414141u) & nz(x[k] ^ 0x43434343u) & nz(x[k] ^ 0x47474747u) &
                           nz(x[k] ^ 0x54545454u);   // bit 7: byte is not A, C, G or T
      nonacgt |= (bad & m & 0x80808080u) != 0u;
    }
    *reinterpret_cast<uint4*>((which ? sq : st) + 16 * c) = make_uint4(x[0], x[1], x[2], x[3]);
  }
  for (int i = tid; i < NH; i += NT_PAIR) {
    twNh[i] = P.tab.twN_hi[i];
    twLh[i] = P.tab.twL_hi[i];
  }
  if (tid < 64) {
    twNl[tid] = P.tab.twN_lo[tid];
    twLl[tid] = P.tab.twL_lo[tid];
  }
  if (tid < 8) s_cnt4[tid] = 0;
  const int any_high = __syncthreads_or(high);
  const int generic = __syncthreads_or(nonacgt);
  if (any_high) {
    if (tid == 0) {
      P.off_cnt[pidx * 2] = 0;
      P.off_cnt[pidx * 2 + 1] = 0;
      P.pair_flags[pidx] = PF_INVALID;
    }
    return;
  }
  if (generic || (Q >= 1024 && Q % WIN != 0) || P.dbg_sig) {
    if (tid == 0) P.fb_list[atomicAdd(P.fb_cnt, 1)] = pidx;
    return;
  }
  if (tid == 0) P.pair_flags[pidx] = P.pairs[pidx].flags & PF_FAST;
  for (int i = tid; i < 2 * N + 16; i += NT_PAIR) aFE[i] = make_float2(0.f, 0.f);   // both sums

  // ---- 2a. entropy weight per window (CCSignal::ComputeEntropy,
  //      CrossCorr.cc:35-93), A/C/G/T only: threads 0..255 target windows,
  //      256..511 query windows ----
  if (tid < 512) {
    const int which = tid >> 8, w = tid & 255;
    const uint8_t* s = which ? sq : st;
    const int len = which ? Q : T;
    float E = 0.f;
    if (len < 1024) {
      E = 1.f;
    } else if (w * WIN + WIN <= len) {
      const int i0 = w * WIN;
      uint32_t cnt = 0;
      for (int j = 0; j < WIN; j++) cnt += 1u << (8 * code_of(s[i0 + j]));
      const int a = cnt & 255u, c = (cnt >> 8) & 255u, g = (cnt >> 16) & 255u;
      E = __ldg(&P.tab.ent_acgt[(a * (WIN + 1) + c) * (WIN + 1) + g]);
    } else if (w * WIN < len) {
      const int i0 = w * WIN;
      const int k = len - i0;
      int a4 = 0, c4 = 0, g4 = 0, t4 = 0;
      for (int j = 0; j < k; j++) {
        const uchar4 q = c_w4q[s[i0 + j]];
        a4 += q.x; c4 += q.y; g4 += q.z; t4 += q.w;
      }
      const double* et = P.tab.ent + k * (4 * WIN + 1);
      const double sv =
          __dadd_rn(__dadd_rn(__dadd_rn(__ldg(et + a4), __ldg(et + c4)), __ldg(et + g4)), __ldg(et + t4));
      E = __double2float_rn(-sv);
      if (E < 0.f) E = 0.f;
    }
    (which ? Eq : Et)[w] = E;
  }

  // ---- 2b. channel means (SeqToPCM, CrossCorr.cc:108-116): exact quarter-unit sums ----
  {
    uint32_t ct = 0, cq = 0;   // one 8-bit count field per base, at most N / 1024 each
    for (int i = tid; i < N; i += NT_PAIR) {
      if (i < T) ct += 1u << (8 * code_of(st[i]));
      if (i < Q) cq += 1u << (8 * code_of(sq[i]));
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int vt = __reduce_add_sync(0xffffffffu, 4 * (int)((ct >> (8 * k)) & 255u));
      const int vq = __reduce_add_sync(0xffffffffu, 4 * (int)((cq >> (8 * k)) & 255u));
      if ((tid & 31) == 0) {
        if (vt) atomicAdd(&s_cnt4[k], vt);
        if (vq) atomicAdd(&s_cnt4[4 + k], vq);
      }
    }
  }
  __syncthreads();
  if (tid < 8) {
    const int len = (tid >> 2) ? Q : T;
    mean_terms(s_cnt4[tid], len, s_wmo[0][tid], s_wmo[1][tid], s_wf[0][tid], s_wf[1][tid]);
  }
  __syncthreads();

  // one stage per channel pair, the channels compile-time constants
  auto stage = [&](auto C0, auto C1) {
    constexpr int c0 = decltype(C0)::value, c1 = decltype(C1)::value;
    // ---- 3a. per-window channel values float(entropy * (weight - mean))
    //      (CrossCorr.cc:123), weight 0 or 1 ----
    {
      const int which = tid >> 8, w = tid & 255;
      const int seq = which >> 1, ch = (which & 1) ? c1 : c0;
      const float E = (seq ? Eq : Et)[w];
      const int k = seq * 4 + ch;
      float2 v;
      v.x = mul_round_f32(E, s_wf[0][k], s_wmo[0][k]);
      v.y = mul_round_f32(E, s_wf[1][k], s_wmo[1][k]);
      vv[which * NWIN + w] = v;
    }
    // each half reads only the window values it wrote (target: 0..511, query:
    // 512..1023), and fills only its own transform buffers
    const GroupBarrier sb{7 + half, 512};
    sb();
    // ---- 3b. z (threads 0..511) or w (512..1023) to its even buffer and
    //      times W_L^n to its odd buffer, as corr_kernel builds its z ----
    {
      const uint8_t* src = half ? sq : st;
      const int len = half ? Q : T;
      const float2* va = vv + 2 * half * NWIN;
      const float2* vb = va + NWIN;
      float2* bE = half ? WE : ZE;
      float2* bO = bE + N;
      const int sl = swz(ht);
#pragma unroll 4   // (full unrolling spills at 64 registers)
      for (int it = 0; it < N / 512; it++) {
        const int n = ht + 512 * it;
        float x = 0.f, y = 0.f;
        if (n < len) {
          const int w = n / WIN;
          const uint32_t code = code_of(src[n]);
          const float2 a = va[w], b = vb[w];
          x = code == (uint32_t)c0 ? a.y : a.x;
          y = code == (uint32_t)c1 ? b.y : b.x;
        }
        const int sn = sl ^ swz(512 * it);   // ht and 512*it share no bit
        bE[sn] = make_float2(x, y);
        bO[sn] = cmul(make_float2(x, y), tw2(twLh, twLl, n));   // W_L^n, n < L/2
      }
    }
    sb();
    // ---- 3c. the four N-point transforms, 256 threads each, each group of
    //      8 warps on its own named barrier (1..4) between passes ----
    fft_forward<LOG2N, 0, GroupBarrier>(ZE + (tid >> 8) * N, twNh, twNl, tid & 255, 256,
                                        GroupBarrier{1 + (tid >> 8), 256});
    __syncthreads();   // the per-bin step reads across the groups
    // ---- 3d. per-bin step (CrossCorrelation::DoOne, CrossCorr.cc:477-492):
    //      bin 0 is the product of real values; bins N-1 and N keep the
    //      targets' own values, which the reference's loop leaves
    //      unmultiplied, for both strands.  Threads 0..511: even bins,
    //      512..1023: odd bins. ----
    auto split = [](float2 A, float2 B, float2& X, float2& Y) {
      X = make_float2(0.5f * (A.x + B.x), 0.5f * (A.y - B.y));
      Y = make_float2(0.5f * (A.y + B.y), -0.5f * (A.x - B.x));
    };
    if (half == 0) {
      const int la = lp<LOG2N>(ht);
      const int lb = lp<LOG2N>((512 - ht) & 511);
#pragma unroll
      for (int it = 0; it <= N / 1024; it++) {
        const int m = ht + 512 * it;
        if (m > N / 2) break;
        const int pa = la ^ lp<LOG2N>(512 * it);
        // partner N-m = (N - 512(it+1)) | (512 - ht) for ht >= 1
        const int pb = ht ? (lb ^ lp<LOG2N>(N - 512 * (it + 1))) : lp<LOG2N>((N - 512 * it) & (N - 1));
        float2 t0, t1, q0, q1;
        split(ZE[pa], ZE[pb], t0, t1);
        split(WE[pa], WE[pb], q0, q1);
        if (m == N / 2) {
          aFE[m].x += t0.x + t1.x;
        } else {
          aFE[m] = cadd(aFE[m], cadd(cmulc(q0, t0), cmulc(q1, t1)));
          aRE[m] = cadd(aRE[m], cadd(cmul(t0, q1), cmul(t1, q0)));
        }
      }
    } else {
      const int la = lp<LOG2N>(ht);
#pragma unroll
      for (int it = 0; it < N / 1024; it++) {
        const int m = ht + 512 * it;
        const int pa = la ^ lp<LOG2N>(512 * it);
        const int pb = pa ^ lp<LOG2N>(N - 1);   // N-1-m = m ^ (N-1)
        float2 t0, t1, q0, q1;
        split(ZO[pa], ZO[pb], t0, t1);
        split(WO[pa], WO[pb], q0, q1);
        if (m == N / 2 - 1) {
          aFO[m] = cadd(aFO[m], cadd(t0, t1));
        } else {
          aFO[m] = cadd(aFO[m], cadd(cmulc(q0, t0), cmulc(q1, t1)));
          aRO[m] = cadd(aRO[m], cadd(cmul(t0, q1), cmul(t1, q0)));
        }
      }
    }
    __syncthreads();
  };
  stage(std::integral_constant<int, 0>(), std::integral_constant<int, 3>());   // A, T
  stage(std::integral_constant<int, 1>(), std::integral_constant<int, 2>());   // C, G

  // ---- 4. inverses: forward strand into ZE (threads 0..511), reverse strand
  //      S_r(k) = W_L^((Q-1)k) conj(R(k)) into WE (512..1023); the two
  //      target-only bins are the same for both strands ----
  float2* buf = half ? WE : ZE;
  if (half == 0) {
    auto SF = [&](int k) -> float2 { return (k & 1) ? aFO[k >> 1] : aFE[k >> 1]; };
    hermitian_pack<LOG2L, NT_CORR>(ZE, both_bins<N>(SF), twLh, twLl, ht);
  } else {
    auto SR = [&](int k) -> float2 {
      if (k >= N - 1) return (k & 1) ? aFO[k >> 1] : aFE[k >> 1];
      const float2 r = (k & 1) ? aRO[k >> 1] : aRE[k >> 1];
      const int j = ((Q - 1) * k) & (L - 1);
      float2 w = tw2(twLh, twLl, j & (N - 1));   // W_L^j, j < L/2
      if (j & N) w = make_float2(-w.x, -w.y);   // W_L^(j + L/2) = -W_L^j
      return cmulc(w, r);
    };
    hermitian_pack<LOG2L, NT_CORR>(WE, both_bins<N>(SR), twLh, twLl, ht);
  }
  // each half packs, inverts and scans its own buffer: named barriers 5, 6
  const GroupBarrier hb{5 + half, NT_CORR};
  hb();
  fft_inverse<LOG2N, Plan<LOG2N>, Plan<LOG2N>::n - 1, GroupBarrier>(buf, twNh, twNl, ht, NT_CORR, hb);

  // ---- 5. FindTop, one strand per half ----
  find_top<LOG2L, NT_CORR, GroupBarrier>(P, P.pairs[pidx].flags, P.pairs[pidx].off_base, pidx, half, buf, ht, s_warp[half],
                                hb);
}

// ---------------------------------------------------------------------------
// corr_pair2_kernel<13>: the persistent both-strands form.  One CTA of 512
// threads per SM strides over the FFT-8192 pairs of a launch; the next pair's
// chunk bytes arrive by cp.async while the current one is transformed.  The
// same premise as corr_pair_kernel (reverse strand from the forward spectra),
// with these changes to the work per pair:
//  - the channels are transformed in the basis u = s_A - s_T,
//    v = s_C - s_G, w = s_A + s_T = -(s_C + s_G): at an A/C/G/T position
//    one channel holds entropy * (1 - mean) and the others
//    entropy * (0 - mean), the means sum to one, so the four channels sum to
//    zero and three signals carry them.  u + i v of each sequence takes two
//    half-length transforms (its even-bin and odd-bin halves) and wt + i wq
//    two, six in all where the four channels of two sequences take eight;
//  - in stage 1 (u + i v) each thread carries two butterflies per pass (both
//    halves of its group's transform) and generates their twiddles once; in
//    stage 2 (wt + i wq) group 0 transforms the even-bin half and group 1 the
//    odd-bin half, one butterfly per thread;
//  - the transform input is built in registers inside the first pass: thread
//    g of a group takes positions g + 256 r (r < 16) from one word of 2-bit
//    codes and the windows' channel values (the reference's rounded values,
//    combined by one FP32 add), so no input buffer is written;
//  - the per-bin steps (pair_bin_uv, pair_bin_w) form 4 sum_c conj(T_c) Q_c
//    and 4i sum_c T_c Q_comp(c) from the packed spectra without separating
//    the signals; the reverse strand's sum W_L^((Q-1)k) conj(R) becomes
//    W_L^((Q-1)k) (i conj(4i R)) / 4, i conj(x + iy) = y + ix, and the
//    target-only bins N-1 and N (sum_c T_c, zero) are written as zero;
//  - the factors are left in (exact powers of two) and removed by FindTop's
//    scale 1/(8N).
// Pairs outside the premise go elsewhere, as in corr_pair_kernel.
// ---------------------------------------------------------------------------
// The layout corr_pair2_kernel and corr_rcq_kernel share (the rcq kernel
// adds its own arrays after it).
static size_t pair_base_smem_bytes() {
  constexpr size_t N = 4096, NH = N / 64;
  return (6 * N + 16 + 2 * (NH + 64)) * sizeof(float2)   // 4 transforms, F and R sums, twiddles
         + 2 * N                                           // chunk bytes (target, query)
         + 2 * 256 * sizeof(float)                         // entropy weight per window
         + 2 * 256 * sizeof(float4)                        // window values (pair2: w by base code)
         + 2 * 256 * sizeof(uint32_t);                     // 2-bit codes of positions g + 256 r
}
size_t corr_pair2_smem_bytes() {
  return pair_base_smem_bytes() + 16 * TW16_ROW * sizeof(float2);   // twiddles of the span-256 passes
}

// Bins k and N-k (k <= N/2) of the reverse strand's packed sum in the
// both-strands kernels: S_r(k) = W_L^((Q-1)k) i conj(2i R(k)), with
// i conj(x + iy) = y + ix; bins N-1 and N are the targets' own sums, the same
// for both strands.  W_L^((Q-1)(N-k)) = (-1)^(Q-1) conj(W_L^((Q-1)k)), so one
// twiddle serves both bins.
template <int LOG2L>
__device__ __forceinline__ void reverse_bins(int k, int Q, const float2* aFE, const float2* aFO, const float2* aRE,
                                             const float2* aRO, const float2* twLh, const float2* twLl, float2& a,
                                             float2& b) {
  constexpr int L = 1 << LOG2L, N = L >> 1;
  const int j = ((Q - 1) * k) & (L - 1);
  float2 w = tw2(twLh, twLl, j & (N - 1));   // W_L^j, j < L/2
  if (j & N) w = make_float2(-w.x, -w.y);   // W_L^(j + L/2) = -W_L^j
  const float2 r = (k & 1) ? aRO[k >> 1] : aRE[k >> 1];
  a = cmul(w, make_float2(r.y, r.x));
  const int kn = N - k;
  if (kn >= N - 1) {
    b = (kn & 1) ? aFO[kn >> 1] : aFE[kn >> 1];
  } else {
    const float2 wn = (Q & 1) ? make_float2(w.x, -w.y) : make_float2(-w.x, w.y);   // (-1)^(Q-1) conj(w)
    const float2 rn = (kn & 1) ? aRO[kn >> 1] : aRE[kn >> 1];
    b = cmul(wn, make_float2(rn.y, rn.x));
  }
}

// Per-bin step of the both-strands kernels at a general bin, from the packed
// spectra A = Zt(m), B = Zt(N-m), C = Zq(m), D = Zq(N-m) of one channel pair:
// f = conj(A) C + B conj(D) = 2 sum_c conj(T_c) Q_c and
// r = A C - conj(B D) = 2i (T_c0 Q_c1 + T_c1 Q_c0).
__device__ __forceinline__ void pair_bin(float2 A, float2 B, float2 C, float2 D, float2& f, float2& r) {
  f = cadd(cmulc(C, A), cmulc(B, D));
  const float2 ac = cmul(A, C), bd = cmul(B, D);
  r = make_float2(ac.x - bd.x, ac.y + bd.y);
}
// corr_pair2_kernel's per-bin steps in the basis u = s_A - s_T,
// v = s_C - s_G, w = s_A + s_T.  Stage 1, from the spectra A = Zt(m),
// B = Zt(N-m), C = Zq(m), D = Zq(N-m) of u + i v:
//   f = conj(A) C + B conj(D) = 2 (conj(Ut) Uq + conj(Vt) Vq)
//   r = -i (A conj(D) + conj(B) C) = -2i (Ut Uq + Vt Vq).
// Stage 2, from E = Y(m), H = Y(N-m) of wt + i wq
// (Wt = (E + conj H) / 2, Wq = (E - conj H) / 2i):
//   f = 2 Im(H E) - i (|E|^2 - |H|^2) = 4 conj(Wt) Wq
//   r = E^2 - conj(H)^2 = 4i Wt Wq.
// Summed: 4 sum_c conj(T_c) Q_c and 4i sum_c T_c Q_comp(c).
__device__ __forceinline__ void pair_bin_uv(float2 A, float2 B, float2 C, float2 D, float2& f, float2& r) {
  f = cadd(cmulc(C, A), cmulc(B, D));
  const float2 s = cadd(cmulc(A, D), cmulc(C, B));
  r = make_float2(s.y, -s.x);
}
__device__ __forceinline__ void pair_bin_w(float2 E, float2 H, float2& f, float2& r) {
  const float he = H.x * E.y + H.y * E.x;
  f = make_float2(he + he, (H.x * H.x + H.y * H.y) - (E.x * E.x + E.y * E.y));
  const float exy = E.x * E.y, hxy = H.x * H.y;
  r = make_float2((E.x * E.x - E.y * E.y) - (H.x * H.x - H.y * H.y), 2.f * (exy + hxy));
}
// Target-only bins, which the reference's loop leaves unmultiplied: Nyquist
// (bin N: A = Zt(N/2) of the even-bin transform) 2 (T_c0 + T_c1), real; bin
// N-1 (A = Zt(N/2-1), B = Zt(N/2) of the odd-bin transform)
// 2 (T_c0 + T_c1) = (A + conj B) - i (A - conj B).
__device__ __forceinline__ float2 pair_bin_nyquist(float2 A) { return make_float2(2.f * (A.x + A.y), 0.f); }
__device__ __forceinline__ float2 pair_bin_nm1(float2 A, float2 B) {
  return make_float2((A.x + B.x) + (A.y + B.y), (A.y - B.y) - (A.x - B.x));
}

// First forward pass of a packed signal z at FFT 8192 (N = 4096), its input
// built in registers: thread g takes x_E[r] = z[g + 256 r] and
// x_O[r] = z[g + 256 r] W_L^(g + 256 r), W_L^(256 r) = exp(-i pi r / 16),
// with z[g + 256 r] = zf(r), then the radix-16 butterflies of span N with
// their twiddles W_N^(g r), generated once for both transforms.
template <class ZF>
__device__ __forceinline__ void first_pass_x2(ZF zf, int g, const float2* twLh, const float2* twLl,
                                              const float2* twNh, const float2* twNl, float2* __restrict__ bE,
                                              float2* __restrict__ bO) {
  const float2 wg = tw2(twLh, twLl, g);
  float2 xe[16], xo[16];
#pragma unroll
  for (int r = 0; r < 16; r++) {
    const float2 z = zf(r);
    xe[r] = z;
    xo[r] = cmul(cmul(z, wg), make_float2(cos_pi16(r), -sin_pi16(r)));
  }
  DFT<16, -1>::run(xe);
  DFT<16, -1>::run(xo);
  const Tw16 tw = tw16(twNh, twNl, g);
#pragma unroll
  for (int r = 1; r < 16; r++) {
    const float2 w = tw16_r(tw, r);
    xe[r] = cmul(xe[r], w);
    xo[r] = cmul(xo[r], w);
  }
  const int sb = swz(g);
#pragma unroll
  for (int r = 0; r < 16; r++) {
    bE[sb ^ swz(256 * r)] = xe[r];
    bO[sb ^ swz(256 * r)] = xo[r];
  }
}

// The same pass for one of the two transforms: the even-bin one (odd false)
// or the odd-bin one, with the same arithmetic per transform.
template <class ZF>
__device__ __forceinline__ void first_pass_x1(ZF zf, bool odd, int g, const float2* twLh, const float2* twLl,
                                              const float2* twNh, const float2* twNl, float2* __restrict__ buf) {
  float2 x[16];
  if (odd) {
    const float2 wg = tw2(twLh, twLl, g);
#pragma unroll
    for (int r = 0; r < 16; r++) x[r] = cmul(cmul(zf(r), wg), make_float2(cos_pi16(r), -sin_pi16(r)));
  } else {
#pragma unroll
    for (int r = 0; r < 16; r++) x[r] = zf(r);
  }
  DFT<16, -1>::run(x);
  const Tw16 tw = tw16(twNh, twNl, g);
#pragma unroll
  for (int r = 1; r < 16; r++) x[r] = cmul(x[r], tw16_r(tw, r));
  const int sb = swz(g);
#pragma unroll
  for (int r = 0; r < 16; r++) buf[sb ^ swz(256 * r)] = x[r];
}

// first_pass_x2 of one sequence's channel pair z = s_c0 + i s_c1: position
// g + 256 r from the word of 2-bit codes of those positions and the windows'
// channel values vw[16 r] (window (g >> 4) + 16 r: c0 at weight 0, 1, then
// c1), zero past len.
__device__ __forceinline__ void first_pass_from_codes(uint32_t codes, int len, const float4* __restrict__ vw, int g,
                                                      int c0, int c1, const float2* twLh, const float2* twLl,
                                                      const float2* twNh, const float2* twNl,
                                                      float2* __restrict__ bE, float2* __restrict__ bO) {
  first_pass_x2(
      [&](int r) {
        const float4 v = vw[16 * r];
        const uint32_t code = (codes >> (2 * r)) & 3u;
        float2 z = make_float2(0.f, 0.f);
        if (g + 256 * r < len) z = make_float2(code == (uint32_t)c0 ? v.y : v.x, code == (uint32_t)c1 ? v.w : v.z);
        return z;
      },
      g, twLh, twLl, twNh, twNl, bE, bO);
}

// Per-window channel values float(entropy * (weight - mean)) (CrossCorr.cc:123)
// of channels c0 and c1 at weights 0 and 1, from the sequence's means held
// as (0 - mean, 1 - mean) in double and as three floats each (k = channel).
__device__ __forceinline__ float4 window_values(float E, const Split3 (*wf)[8], const double (*wmo)[8], int k0,
                                                int k1) {
  return make_float4(mul_round_f32(E, wf[0][k0], wmo[0][k0]), mul_round_f32(E, wf[1][k0], wmo[1][k0]),
                     mul_round_f32(E, wf[0][k1], wmo[0][k1]), mul_round_f32(E, wf[1][k1], wmo[1][k1]));
}

// Issues the cp.async copies of pair pidx's chunk bytes into st / sq: thread
// t takes 16-byte piece t & 255 of the target (t < 256) or the query; bytes
// past the chunk end are zero-filled (pool chunks are 16-byte aligned).
__device__ __forceinline__ void pair2_prefetch(const CorrParams& P, int pidx, uint8_t* st, uint8_t* sq, int tid) {
  const PairDesc& D = P.pairs[pidx];
  const int which = tid >> 8, c = tid & 255;
  const int len = which ? D.qlen : D.tlen;
  const uint8_t* src = P.pool + (which ? D.q_off : D.t_off);
  const int valid = min(max(len - 16 * c, 0), 16);
  if (valid > 0) src += 16 * c;   // else: nothing is read; the chunk start stays a valid address
  const uint32_t dst = (uint32_t)__cvta_generic_to_shared((which ? sq : st) + 16 * c);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid) : "memory");
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Work order of the persistent kernels over count items: CTA b takes items
// b + r * grid for rounds r = 0..S (S = count / grid - 2, at least 0), then
// items from the work counter (offset (S + 1) * grid) until none is left.
// The rounds balance equal-cost items with no atomics; the counter absorbs
// items of unequal cost (pairs handed back, chunks flagged) and CTAs that
// start late at the end.
__device__ __forceinline__ int static_rounds(int count) { return max(0, count / (int)gridDim.x - 2); }
__device__ __forceinline__ int take_item(int* work, int r, int S) {
  return r <= S ? (int)blockIdx.x + r * (int)gridDim.x : atomicAdd(work, 1) + (S + 1) * (int)gridDim.x;
}

template <int LOG2L>
__global__ void __launch_bounds__(NT_PAIR2, 1) corr_pair2_kernel(const CorrParams P) {
  constexpr int L = 1 << LOG2L;
  constexpr int N = L >> 1;
  constexpr int LOG2N = LOG2L - 1;
  constexpr int WIN = L / 512;
  constexpr int NWIN = 256;
  constexpr int NH = N / 64;
  static_assert(N == 16 * NWIN && N == 4096, "thread g of a group owns positions g + 256 r, r < 16");

  extern __shared__ __align__(16) unsigned char smem[];
  float2* ZE = reinterpret_cast<float2*>(smem);   // z = t_c0 + i t_c1, even-bin transform
  float2* ZO = ZE + N;                            // z * W_L^n, odd-bin transform
  float2* WE = ZO + N;                            // w = q_c0 + i q_c1
  float2* WO = WE + N;
  float2* aFE = WO + N;                           // 4 x forward-strand sum, bins 2m, m <= N/2
  float2* aFO = aFE + (N / 2 + 8);                // bins 2m+1
  float2* aRE = aFO + N / 2;                      // 4i x R, bins 2m (m < N/2)
  float2* aRO = aRE + (N / 2 + 8);                // bins 2m+1
  float2* twNh = aRO + N / 2;
  float2* twNl = twNh + NH;
  float2* twLh = twNl + 64;
  float2* twLl = twLh + NH;
  float2* tw16t = twLl + 64;   // twiddles of the span-256 passes (build_tw16_table)
  uint8_t* st = reinterpret_cast<uint8_t*>(tw16t + 16 * TW16_ROW);
  uint8_t* sq = st + N;
  float* Et = reinterpret_cast<float*>(sq + N);
  float* Eq = Et + NWIN;
  float4* vv = reinterpret_cast<float4*>(Eq + NWIN);   // [sequence][window]: w by base code
  uint32_t* cw = reinterpret_cast<uint32_t*>(vv + 2 * NWIN);   // [sequence][g]
  __shared__ int s_cnt4[8];
  __shared__ unsigned s_flags;     // bit 0: a byte >= 128; bit 1: a byte other than A, C, G, T
  __shared__ int s_take;           // the CTA's next pair
  __shared__ double s_wmo[2][8];   // 0 - mean and 1 - mean per (sequence, channel)
  __shared__ Split3 s_wf[2][8];    // the same as three floats each
  __shared__ int s_warp[2][2 * 256 / 32];

  const int tid = threadIdx.x;
  const int G = tid >> 8;          // 0: target transforms / forward strand, 1: query / reverse strand
  const int g = tid & 255;
  const GroupBarrier gb{1 + G, 256};

  for (int i = tid; i < NH; i += NT_PAIR2) {
    twNh[i] = P.tab.twN_hi[i];
    twLh[i] = P.tab.twL_hi[i];
  }
  if (tid < 64) {
    twNl[tid] = P.tab.twN_lo[tid];
    twLl[tid] = P.tab.twL_lo[tid];
  }
  if ((int)blockIdx.x < P.count) pair2_prefetch(P, P.first + blockIdx.x, st, sq, tid);
  __syncthreads();
  build_tw16_table(tw16t, twNh, twNl, N / 256, tid);   // read after the first barrier of the loop
  // Pairs in the order take_item gives, each taken one pair ahead (the next
  // pair's bytes are prefetched while this one is worked on; thread 0 uses a
  // counter result one pair after taking it).
  const int S = static_rounds(P.count);
  if (tid == 0) s_take = take_item(P.work, 1, S);

  for (int p = blockIdx.x, r = 0; p < P.count; r++) {
    const int pidx = P.first + p;
    const int T = P.pairs[pidx].tlen, Q = P.pairs[pidx].qlen;
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (tid < 8) s_cnt4[tid] = 0;
    if (tid == 0) s_flags = 0u;
    __syncthreads();   // the chunk bytes are in; the counters are zero; the next pair is known
    const int np = s_take;
    const int next = np < P.count ? P.first + np : -1;
    int take = 0;
    if (tid == 0) take = take_item(P.work, r + 2, S);   // the pair after next

    // ---- 1. thread (G, g) takes bytes 16g..16g+15 of sequence G, which are
    //      also its entropy window (WIN = 16): byte checks (per byte,
    //      exactly, (y & 0x7f) + 0x7f | y has bit 7 clear iff y == 0), the
    //      2-bit codes (A=0 C=1 G=2 T=3), base counts for the channel means
    //      (SeqToPCM, CrossCorr.cc:108-116) and the window's entropy weight
    //      (CCSignal::ComputeEntropy, CrossCorr.cc:35-93).  Bytes past the
    //      chunk end (zero) are masked out. ----
    uint32_t* cwin = reinterpret_cast<uint32_t*>(vv);   // [sequence][window] codes; vv is free until step 3a
    {
      const int len = G ? Q : T;
      const int valid = len - 16 * g;
      const uint8_t* sb = G ? sq : st;
      const uint4 v = *reinterpret_cast<const uint4*>(sb + 16 * g);
      const uint32_t x[4] = {v.x, v.y, v.z, v.w};
      auto nz = [](uint32_t y) { return (((y & 0x7f7f7f7fu) + 0x7f7f7f7fu) | y) & 0x80808080u; };
      uint32_t high = 0u, bad = 0u, p0 = 0u, p1 = 0u, codes = 0u;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int vk = min(max(valid - 4 * k, 0), 4);
        const uint32_t m = vk >= 4 ? 0xffffffffu : (1u << (8 * vk)) - 1u;
        high |= x[k] & m & 0x80808080u;
        bad |= nz(x[k] ^ 0x41414141u) & nz(x[k] ^ 0x43434343u) & nz(x[k] ^ 0x47474747u) & nz(x[k] ^ 0x54545454u) &
               m & 0x80808080u;   // bit 7: byte is not A, C, G or T
        const uint32_t cd = ((x[k] >> 1) ^ (x[k] >> 2)) & 0x03030303u & m;
        p0 |= (((cd & 0x01010101u) * 0x10204080u) >> 28) << (4 * k);          // bit j: code bit 0 of byte j
        p1 |= ((((cd >> 1) & 0x01010101u) * 0x10204080u) >> 28) << (4 * k);   // bit j: code bit 1
        const uint32_t c2 = cd | (cd >> 6);   // codes of bytes 0, 1 in bits 0-3, of bytes 2, 3 in bits 16-19
        codes |= ((c2 & 0xfu) | ((c2 >> 12) & 0xf0u)) << (8 * k);
      }
      cwin[tid] = codes;
      const int nv = min(max(valid, 0), 16);
      const int nt = __popc(p0 & p1), nc = __popc(p0) - nt, ng = __popc(p1) - nt, na = nv - nc - ng - nt;
      float E = 0.f;
      if (len < 1024) {
        E = 1.f;
      } else if (nv == 16) {
        E = __ldg(&P.tab.ent_acgt[(na * (WIN + 1) + nc) * (WIN + 1) + ng]);
      } else if (nv > 0) {
        int a4 = 0, c4 = 0, g4 = 0, t4 = 0;
        for (int j = 0; j < nv; j++) {
          const uchar4 q = c_w4q[sb[16 * g + j] & 127u];   // a byte >= 128 voids the pair
          a4 += q.x; c4 += q.y; g4 += q.z; t4 += q.w;
        }
        const double* et = P.tab.ent + nv * (4 * WIN + 1);
        const double sv =
            __dadd_rn(__dadd_rn(__dadd_rn(__ldg(et + a4), __ldg(et + c4)), __ldg(et + g4)), __ldg(et + t4));
        E = __double2float_rn(-sv);
        if (E < 0.f) E = 0.f;
      }
      (G ? Eq : Et)[g] = E;
      // counts in 16-bit fields (at most 16 x 32 per warp), four quarter
      // units per base
      const uint32_t lo = __reduce_add_sync(0xffffffffu, (uint32_t)na | ((uint32_t)nc << 16));
      const uint32_t hi = __reduce_add_sync(0xffffffffu, (uint32_t)ng | ((uint32_t)nt << 16));
      const uint32_t fl = __reduce_or_sync(0xffffffffu, (high ? 1u : 0u) | (bad ? 2u : 0u));
      if ((tid & 31) == 0) {
        atomicAdd(&s_cnt4[4 * G + 0], 4 * (int)(lo & 0xffffu));
        atomicAdd(&s_cnt4[4 * G + 1], 4 * (int)(lo >> 16));
        atomicAdd(&s_cnt4[4 * G + 2], 4 * (int)(hi & 0xffffu));
        atomicAdd(&s_cnt4[4 * G + 3], 4 * (int)(hi >> 16));
        if (fl) atomicOr(&s_flags, fl);
      }
    }
    __syncthreads();   // the chunk bytes are no longer read: the next pair's may come in
    if (next >= 0) pair2_prefetch(P, next, st, sq, tid);
    const uint32_t flg = s_flags;
    if ((flg & 1u) || (flg & 2u) || (Q >= 1024 && Q % WIN != 0) || P.dbg_sig) {
      if (tid == 0) {
        if (flg & 1u) {
          P.off_cnt[pidx * 2] = 0;
          P.off_cnt[pidx * 2 + 1] = 0;
          P.pair_flags[pidx] = PF_INVALID;
        } else if (P.fb2_list && !(flg & 2u) && !P.dbg_sig) {
          P.fb2_list[atomicAdd(P.fb2_cnt, 1)] = pidx;   // a ragged query window: corr_rcq_kernel takes it
        } else {
          P.fb_list[atomicAdd(P.fb_cnt, 1)] = pidx;   // the per-strand kernel takes it
        }
      }
      if (tid == 0) s_take = take;
      __syncthreads();   // cwin (in vv), the flags and the next pair's index are reused
      p = np;
      continue;
    }
    if (tid == 0) P.pair_flags[pidx] = P.pairs[pidx].flags & PF_FAST;
    // ---- 2. channel means (FP64, as the reference) and the codes of
    //      positions g + 256 r, one word per thread ----
    if (tid < 8) {
      const int len = (tid >> 2) ? Q : T;
      mean_terms(s_cnt4[tid], len, s_wmo[0][tid], s_wmo[1][tid], s_wf[0][tid], s_wf[1][tid]);
    }
    {
      const uint32_t* cs = cwin + G * NWIN + (g >> 4);
      const int sh = 2 * (g & 15);
      uint32_t w = 0;
#pragma unroll
      for (int r = 0; r < 16; r++) w |= ((cs[16 * r] >> sh) & 3u) << (2 * r);
      cw[tid] = w;
    }
    __syncthreads();

    // ---- 3. the channels in the basis u = s_A - s_T, v = s_C - s_G and
    //      w = s_A + s_T = -(s_C + s_G) (an A/C/G/T position holds one base
    //      and the channel means sum to one, so the four channels sum to
    //      zero).  With U, V, W their spectra, per bin
    //        sum_c conj(T_c) Q_c = conj(Wt) Wq + (conj(Ut) Uq + conj(Vt) Vq) / 2
    //        sum_c T_c Q_comp(c) = Wt Wq - (Ut Uq + Vt Vq) / 2,
    //      and the target-only bins N-1 and N (sum_c T_c) are zero.  Stage 1
    //      transforms u + i v of sequence G in group G (both halves), stage 2
    //      wt + i wq (group 0 the even-bin half, group 1 the odd-bin half):
    //      six half-length forward transforms per pair. ----
    // 3a. per-window signal values by base code, from the channel values
    //     float(entropy * (weight - mean)) (CrossCorr.cc:123) at weight 0 or 1
    //     with one FP32 add each: (u, v) into uvt (stage 1; the sums overwrite
    //     it after stage 1's first pass), w into vv (stage 2)
    float2* uvt = reinterpret_cast<float2*>(aFE);   // [sequence][window][code]
    {
      const float E = (G ? Eq : Et)[g];
      const float4 at = window_values(E, s_wf, s_wmo, G * 4 + 0, G * 4 + 3);   // A at 0, 1; T at 0, 1
      const float4 cg = window_values(E, s_wf, s_wmo, G * 4 + 1, G * 4 + 2);   // C at 0, 1; G at 0, 1
      const float u0 = __fsub_rn(at.x, at.z), v0 = __fsub_rn(cg.x, cg.z), w0 = __fadd_rn(at.x, at.z);
      float4* o = reinterpret_cast<float4*>(uvt + (G * NWIN + g) * 4);
      o[0] = make_float4(__fsub_rn(at.y, at.z), v0, u0, __fsub_rn(cg.y, cg.z));   // A, C
      o[1] = make_float4(u0, __fsub_rn(cg.x, cg.w), __fsub_rn(at.x, at.w), v0);   // G, T
      vv[G * NWIN + g] = make_float4(__fadd_rn(at.y, at.z), w0, w0, __fadd_rn(at.x, at.w));
    }
    gb();
    // 3b. stage 1: first pass of u + i v with its input built in registers,
    //     then the other two passes, both halves of the group's transform at once
    {
      const uint32_t codes = cw[tid];
      const int len = G ? Q : T;
      const float2* ub = uvt + (G * NWIN + (g >> 4)) * 4;
      float2* bE = G ? WE : ZE;
      first_pass_x2(
          [&](int r) {
            const float2 z = ub[64 * r + ((codes >> (2 * r)) & 3u)];
            return g + 256 * r < len ? z : make_float2(0.f, 0.f);
          },
          g, twLh, twLl, twNh, twNl, bE, bE + N);
      gb();
      fft_pass16_x2_tab<N, N / 16>(bE, bE + N, tw16t, g);
      gb();
      fft_pass16_x2<N, N / 256>(bE, bE + N, twNh, twNl, g);
    }
    __syncthreads();   // the per-bin step reads both groups' spectra
    // 3c. stage 1 per-bin step (CrossCorrelation::DoOne, CrossCorr.cc:477-492):
    //     group 0 even bins, group 1 odd bins; bin 0 by the general formula
    //     (B = A, D = C: products of real values)
    if (G == 0) {
      const int la = lp<LOG2N>(g);
      const int lb = lp<LOG2N>((256 - g) & 255);
#pragma unroll
      for (int it = 0; it <= N / 512; it++) {
        const int m = g + 256 * it;
        if (m > N / 2) break;
        const int pa = la ^ lp<LOG2N>(256 * it);
        // partner N-m = (N - 256(it+1)) | (256 - g) for g >= 1
        const int pb = g ? (lb ^ lp<LOG2N>(N - 256 * (it + 1))) : lp<LOG2N>((N - 256 * it) & (N - 1));
        if (m == N / 2) {
          aFE[m] = make_float2(0.f, 0.f);
        } else {
          float2 f, r;
          pair_bin_uv(ZE[pa], ZE[pb], WE[pa], WE[pb], f, r);
          aFE[m] = f;
          aRE[m] = r;
        }
      }
    } else {
      const int la = lp<LOG2N>(g);
#pragma unroll
      for (int it = 0; it < N / 512; it++) {
        const int m = g + 256 * it;
        const int pa = la ^ lp<LOG2N>(256 * it);
        const int pb = pa ^ lp<LOG2N>(N - 1);   // N-1-m = m ^ (N-1)
        if (m == N / 2 - 1) {
          aFO[m] = make_float2(0.f, 0.f);
        } else {
          float2 f, r;
          pair_bin_uv(ZO[pa], ZO[pb], WO[pa], WO[pb], f, r);
          aFO[m] = f;
          aRO[m] = r;
        }
      }
    }
    gb();   // stage 2 overwrites the buffer the group's per-bin step read (group 0 ZE, group 1 WO)
    // 3d. stage 2: wt + i wq, the even-bin half in group 0, the odd-bin half in group 1
    float2* bw = G ? WO : ZE;
    {
      const uint32_t ct = cw[g], cq = cw[NWIN + g];
      const float* wb = reinterpret_cast<const float*>(vv) + (g >> 4) * 4;
      first_pass_x1(
          [&](int r) {
            const float wt = wb[64 * r + ((ct >> (2 * r)) & 3u)];
            const float wq = wb[NWIN * 4 + 64 * r + ((cq >> (2 * r)) & 3u)];
            return make_float2(g + 256 * r < T ? wt : 0.f, g + 256 * r < Q ? wq : 0.f);
          },
          G == 1, g, twLh, twLl, twNh, twNl, bw);
      gb();
      fft_pass16_tab<N, N / 16>(bw, tw16t, g);
      gb();
      fft_pass<16, N, N / 256, false>(bw, twNh, twNl, g, 256);
    }
    gb();
    // 3e. stage 2 per-bin step, each group over its own half: E = Y(m), H = Y(N-m)
    //     (partly unrolled: fully unrolled, its loads push the kernel past 128 registers)
    if (G == 0) {
      const int la = lp<LOG2N>(g);
      const int lb = lp<LOG2N>((256 - g) & 255);
#pragma unroll 3
      for (int it = 0; it <= N / 512; it++) {
        const int m = g + 256 * it;
        if (m >= N / 2) break;
        const int pa = la ^ lp<LOG2N>(256 * it);
        const int pb = g ? (lb ^ lp<LOG2N>(N - 256 * (it + 1))) : lp<LOG2N>((N - 256 * it) & (N - 1));
        float2 f, r;
        pair_bin_w(ZE[pa], ZE[pb], f, r);
        aFE[m] = cadd(aFE[m], f);
        aRE[m] = cadd(aRE[m], r);
      }
    } else {
      const int la = lp<LOG2N>(g);
#pragma unroll 3
      for (int it = 0; it < N / 512; it++) {
        const int m = g + 256 * it;
        if (m == N / 2 - 1) break;
        const int pa = la ^ lp<LOG2N>(256 * it);
        const int pb = pa ^ lp<LOG2N>(N - 1);
        float2 f, r;
        pair_bin_w(WO[pa], WO[pb], f, r);
        aFO[m] = cadd(aFO[m], f);
        aRO[m] = cadd(aRO[m], r);
      }
    }
    __syncthreads();

    // ---- 4. inverses: group 0 the forward strand into ZE, group 1 the
    //      reverse strand S_r(k) = W_L^((Q-1)k) i conj(2i R(k)) into WE; the two
    //      target-only bins are the same for both strands.  Sums and the pack
    //      carry factors 2 and 2: FindTop scales by 1/(4N). ----
    float2* buf = G ? WE : ZE;
    if (G == 0) {
      auto SF = [&](int k) -> float2 { return (k & 1) ? aFO[k >> 1] : aFE[k >> 1]; };
      hermitian_pack<LOG2L, 256>(ZE, both_bins<N>(SF), twLh, twLl, g, 1.0f);
    } else {
      hermitian_pack<LOG2L, 256>(
          WE, [&](int k, float2& a, float2& b) { reverse_bins<LOG2L>(k, Q, aFE, aFO, aRE, aRO, twLh, twLl, a, b); },
          twLh, twLl, g, 1.0f);
    }
    gb();
    fft_pass<16, N, 16, true>(buf, twNh, twNl, g, 256);
    gb();
    fft_pass16_inv_tab<N, 256>(buf, tw16t, g);
    gb();
    fft_pass<16, N, N, true>(buf, twNh, twNl, g, 256);
    gb();

    // ---- 5. FindTop, one strand per group ----
    find_top<LOG2L, 256, GroupBarrier>(P, P.pairs[pidx].flags, P.pairs[pidx].off_base, pidx, G, buf, g, s_warp[G], gb,
                                       1.0f / (float)(8 * N));
    if (tid == 0) s_take = take;
    __syncthreads();   // buffers and per-pair words are reused by the next pair
    p = np;
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// ---------------------------------------------------------------------------
// The spectra path at FFT 8192.  In a block of chunk pairs (a t_pair block of
// 24 x 24 chunks is 576 pairs of 48 distinct chunks) every chunk takes part in
// many pairs; the reference builds each chunk's signals once per block
// (HomologyByXCorrSlave.cc:284-299).  spec_kernel transforms each distinct
// chunk once in corr_pair2_kernel's channel basis -- u + i v (u = A - T,
// v = C - G) and w + 0 i (w = A + T), even-bin and odd-bin transforms -- and
// stores the spectra in bin order (128 KB per chunk, of w's real spectrum
// the bins the pair kernel reads; L2-resident for a batch of blocks);
// corr_spec_kernel then forms each pair's sums from the two chunks' spectra,
// u + i v at m and N - m and W at m, and runs the inverses and FindTop.  Its
// sums differ from corr_pair2_kernel's in rounding only (that kernel
// transforms the two sequences' w jointly), so the two agree on every
// FindTop offset outside the near-threshold lags.
// ---------------------------------------------------------------------------
size_t spec_bytes_per_chunk() { return (size_t)4 * 4096 * sizeof(float2); }

// ---------------------------------------------------------------------------
// corr_rcq_kernel<13>: both strands of an A/C/G/T pair whose query is at least
// 1024 bases and not a multiple of the entropy window (16).  There the
// reverse-complemented query's windows do not map onto the forward ones, so
// the reverse strand's query signal is its own (CCSignal over the reverse
// complement, as the reference builds it), and the spectra cannot be shared
// the way corr_pair2_kernel shares them.  The target is still transformed
// once for both strands (two per-strand CTAs transform it twice).  The
// channels go in corr_pair2_kernel's basis u = A - T, v = C - G, w = A + T
// (the reverse complement is A/C/G/T too, so its channels also sum to
// zero): group 0 transforms the target's u + i v and group 1 the forward
// query's (two transforms each), the forward sum takes
// f = conj(A) C + B conj(D); then group 0 transforms the reverse
// complement's even-bin half and group 1 its odd-bin half, and the reverse
// sum takes the same formula; then wt + i wq and wt + i wr, each split
// between the groups, add 4 conj(Wt) Wq and 4 conj(Wt) Wr (pair_bin_w).
// 10 forward and 2 inverse half-length transforms per pair (12 with the
// four channels), where two corr_kernel CTAs take 16 and 2.  The pairs
// are the FFT-8192 bucket's last ones, placed there by the host (its
// ragged query windows), or the list corr_spec_kernel (or, without a
// range, corr_pair2_kernel) hands on; CTAs stride over them.  A pair with a
// byte >= 128 is voided after the pass and one with other letters is handed
// on to the per-strand kernel.
// ---------------------------------------------------------------------------
size_t corr_rcq_smem_bytes() {
  return pair_base_smem_bytes() + 256 * sizeof(float)   // reverse-complement window weights
         + 256 * sizeof(float4)                          // its window values
         + 256 * sizeof(uint32_t);                       // its codes of positions g + 256 r
}

template <int LOG2L>
__global__ void __launch_bounds__(NT_PAIR2, 1) corr_rcq_kernel(const CorrParams P) {
  constexpr int L = 1 << LOG2L;
  constexpr int N = L >> 1;
  constexpr int LOG2N = LOG2L - 1;
  constexpr int WIN = L / 512;
  constexpr int NWIN = 256;
  constexpr int NH = N / 64;
  static_assert(N == 16 * NWIN && N == 4096 && WIN == 16, "thread g of a group owns positions g + 256 r, r < 16");

  extern __shared__ __align__(16) unsigned char smem[];
  float2* ZE = reinterpret_cast<float2*>(smem);   // z = t_c0 + i t_c1, even-bin transform
  float2* ZO = ZE + N;                            // z * W_L^n, odd-bin transform
  float2* WE = ZO + N;                            // w = q_c0 + i q_c1, then the reverse complement's
  float2* WO = WE + N;
  float2* aFE = WO + N;                           // 4 x forward-strand sum, bins 2m, m <= N/2
  float2* aFO = aFE + (N / 2 + 8);                // bins 2m+1
  float2* aRE = aFO + N / 2;                      // 4 x reverse-strand sum, bins 2m (m < N/2)
  float2* aRO = aRE + (N / 2 + 8);                // bins 2m+1 (m < N/2 - 1)
  float2* twNh = aRO + N / 2;
  float2* twNl = twNh + NH;
  float2* twLh = twNl + 64;
  float2* twLl = twLh + NH;
  uint8_t* st = reinterpret_cast<uint8_t*>(twLl + 64);
  uint8_t* sq = st + N;
  float* Et = reinterpret_cast<float*>(sq + N);
  float* Eq = Et + NWIN;
  float4* vv = reinterpret_cast<float4*>(Eq + NWIN);   // [sequence][window]: w by base code
  uint32_t* cw = reinterpret_cast<uint32_t*>(vv + 2 * NWIN);   // [sequence][g]
  float* Er = reinterpret_cast<float*>(cw + 2 * NWIN);        // reverse complement: window weights
  float4* vr = reinterpret_cast<float4*>(Er + NWIN);          // its w by base code
  uint32_t* cr = reinterpret_cast<uint32_t*>(vr + NWIN);      // its codes of positions g + 256 r
  __shared__ int s_cnt4[8];
  __shared__ unsigned s_flags;     // bit 0: a byte >= 128; bit 1: a byte other than A, C, G, T
  __shared__ double s_wmo[2][8];   // 0 - mean and 1 - mean per (sequence, channel)
  __shared__ Split3 s_wf[2][8];    // the same as three floats each
  __shared__ int s_warp[2][2 * 256 / 32];

  const int tid = threadIdx.x;
  const int G = tid >> 8;
  const int g = tid & 255;
  const GroupBarrier gb{1 + G, 256};
  // the list the spectra kernel filled, or the bucket's range of them
  const int count = P.fb2_list ? *P.fb2_cnt : P.rcq_count;
  auto pair_at = [&](int k) { return P.fb2_list ? P.fb2_list[k] : P.rcq_first + k; };

  for (int i = tid; i < NH; i += NT_PAIR2) {
    twNh[i] = P.tab.twN_hi[i];
    twLh[i] = P.tab.twL_hi[i];
  }
  if (tid < 64) {
    twNl[tid] = P.tab.twN_lo[tid];
    twLl[tid] = P.tab.twL_lo[tid];
  }
  if ((int)blockIdx.x < count) pair2_prefetch(P, pair_at(blockIdx.x), st, sq, tid);

  for (int p = blockIdx.x; p < count; p += gridDim.x) {
    const int pidx = pair_at(p);
    const int next = p + (int)gridDim.x < count ? pair_at(p + gridDim.x) : -1;
    const int T = P.pairs[pidx].tlen, Q = P.pairs[pidx].qlen;
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (tid < 8) s_cnt4[tid] = 0;
    if (tid == 0) s_flags = 0u;
    __syncthreads();   // the chunk bytes are in; the counters are zero

    // ---- 1. thread (G, g): bytes 16g..16g+15 of sequence G (entropy window
    //      g): 2-bit codes, base counts, window weight, as corr_pair2_kernel.
    //      The query's last reverse window (the reverse complement's
    //      positions 16k.. with fewer than 16 left) is weighed here from the
    //      bytes; its full windows after the barrier, from the codes. ----
    uint32_t* cwin = reinterpret_cast<uint32_t*>(vv);   // [sequence][window] codes; vv is free until step 3
    {
      const int len = G ? Q : T;
      const int valid = len - 16 * g;
      const uint8_t* sb = G ? sq : st;
      const uint4 v = *reinterpret_cast<const uint4*>(sb + 16 * g);
      const uint32_t x[4] = {v.x, v.y, v.z, v.w};
      {
        // byte checks, as corr_pair2_kernel's (a range of ragged query
        // windows is not checked before)
        auto nz = [](uint32_t y) { return (((y & 0x7f7f7f7fu) + 0x7f7f7f7fu) | y) & 0x80808080u; };
        uint32_t high = 0u, bad = 0u;
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const int vk = min(max(valid - 4 * k, 0), 4);
          const uint32_t m = vk >= 4 ? 0xffffffffu : (1u << (8 * vk)) - 1u;
          high |= x[k] & m & 0x80808080u;
          bad |= nz(x[k] ^ 0x41414141u) & nz(x[k] ^ 0x43434343u) & nz(x[k] ^ 0x47474747u) &
                 nz(x[k] ^ 0x54545454u) & m & 0x80808080u;   // bit 7: byte is not A, C, G or T
        }
        const unsigned fl = (high ? 1u : 0u) | (bad ? 2u : 0u);
        if (fl) atomicOr(&s_flags, fl);
      }
      uint32_t p0 = 0u, p1 = 0u, codes = 0u;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int vk = min(max(valid - 4 * k, 0), 4);
        const uint32_t m = vk >= 4 ? 0xffffffffu : (1u << (8 * vk)) - 1u;
        const uint32_t cd = ((x[k] >> 1) ^ (x[k] >> 2)) & 0x03030303u & m;
        p0 |= (((cd & 0x01010101u) * 0x10204080u) >> 28) << (4 * k);
        p1 |= ((((cd >> 1) & 0x01010101u) * 0x10204080u) >> 28) << (4 * k);
        const uint32_t c2 = cd | (cd >> 6);
        codes |= ((c2 & 0xfu) | ((c2 >> 12) & 0xf0u)) << (8 * k);
      }
      cwin[tid] = codes;
      const int nv = min(max(valid, 0), 16);
      const int nt = __popc(p0 & p1), nc = __popc(p0) - nt, ng = __popc(p1) - nt, na = nv - nc - ng - nt;
      auto partial = [&](const uint8_t* bytes, int n, bool rc) -> float {
        int a4 = 0, c4 = 0, g4 = 0, t4 = 0;
        for (int j = 0; j < n; j++) {
          const unsigned b = bytes[j];
          const uchar4 q = c_w4q[(rc ? c_rc[b] : b) & 127u];   // a byte >= 128 voids the pair
          a4 += q.x; c4 += q.y; g4 += q.z; t4 += q.w;
        }
        const double* et = P.tab.ent + n * (4 * WIN + 1);
        const double sv =
            __dadd_rn(__dadd_rn(__dadd_rn(__ldg(et + a4), __ldg(et + c4)), __ldg(et + g4)), __ldg(et + t4));
        const float E = __double2float_rn(-sv);
        return E < 0.f ? 0.f : E;
      };
      float E = 0.f;
      if (len < 1024) E = 1.f;
      else if (nv == 16) E = __ldg(&P.tab.ent_acgt[(na * (WIN + 1) + nc) * (WIN + 1) + ng]);
      else if (nv > 0) E = partial(sb + 16 * g, nv, false);
      (G ? Eq : Et)[g] = E;
      if (G == 1) {
        // reverse window k = g: the reverse complement's positions 16k..16k+15,
        // forward positions Q-16k-16..Q-16k-1; the last one is partial
        const int nr = min(Q - 16 * g, 16);
        if (nr > 0 && nr < 16) Er[g] = partial(sq, nr, true);   // forward positions 0..nr-1
        else if (nr <= 0) Er[g] = 0.f;
      }
      const uint32_t lo = __reduce_add_sync(0xffffffffu, (uint32_t)na | ((uint32_t)nc << 16));
      const uint32_t hi = __reduce_add_sync(0xffffffffu, (uint32_t)ng | ((uint32_t)nt << 16));
      if ((tid & 31) == 0) {
        atomicAdd(&s_cnt4[4 * G + 0], 4 * (int)(lo & 0xffffu));
        atomicAdd(&s_cnt4[4 * G + 1], 4 * (int)(lo >> 16));
        atomicAdd(&s_cnt4[4 * G + 2], 4 * (int)(hi & 0xffffu));
        atomicAdd(&s_cnt4[4 * G + 3], 4 * (int)(hi >> 16));
      }
    }
    __syncthreads();   // the chunk bytes are no longer read: the next pair's may come in
    if (next >= 0) pair2_prefetch(P, next, st, sq, tid);
    if (tid == 0) P.pair_flags[pidx] = P.pairs[pidx].flags & PF_FAST;
    // ---- 2. channel means (FP64); the codes of positions g + 256 r of the
    //      target, the query and the reverse complement (3 - the code of
    //      forward position Q-1-n); the reverse complement's full windows
    //      (its counts are the forward counts of the complement bases) ----
    if (tid < 8) {
      const int len = (tid >> 2) ? Q : T;
      mean_terms(s_cnt4[tid], len, s_wmo[0][tid], s_wmo[1][tid], s_wf[0][tid], s_wf[1][tid]);
    }
    {
      const uint32_t* cs = cwin + G * NWIN + (g >> 4);
      const int sh = 2 * (g & 15);
      uint32_t w = 0;
#pragma unroll
      for (int r = 0; r < 16; r++) w |= ((cs[16 * r] >> sh) & 3u) << (2 * r);
      cw[tid] = w;
    }
    const uint32_t* cq = cwin + NWIN;   // the query's codes per window
    if (G == 0) {
      uint32_t w = 0;
#pragma unroll
      for (int r = 0; r < 16; r++) {
        const int m = Q - 1 - (g + 256 * r);
        if (m >= 0) w |= (3u - ((cq[m >> 4] >> (2 * (m & 15))) & 3u)) << (2 * r);
      }
      cr[g] = w;
    } else if (Q - 16 * g >= 16) {
      const int a = Q - 16 * g - 16;   // forward positions a..a+15
      const int wa = a >> 4, sh = 2 * (a & 15);
      const uint32_t c16 = __funnelshift_r(cq[wa], wa + 1 < NWIN ? cq[wa + 1] : 0u, sh);
      const int nt = __popc(c16 & (c16 >> 1) & 0x55555555u), nc = __popc(c16 & 0x55555555u) - nt,
                ng = __popc(c16 & 0xaaaaaaaau) - nt, na = 16 - nc - ng - nt;
      // reverse complement: A <- T, C <- G, G <- C
      Er[g] = Q < 1024 ? 1.f : __ldg(&P.tab.ent_acgt[(nt * (WIN + 1) + ng) * (WIN + 1) + nc]);
      (void)na;
    }
    __syncthreads();

    // ---- 3. the channels in the basis u = s_A - s_T, v = s_C - s_G,
    //      w = s_A + s_T = -(s_C + s_G), as corr_pair2_kernel (the reverse
    //      complement is A/C/G/T too, its channel means the forward query's
    //      of the complement channels, so its channels also sum to zero).
    //      Stage 1: u + i v of the target (group 0) and the query (group 1),
    //      both halves, the forward per-bin step, then u + i v of the reverse
    //      complement (group 0 its even-bin half, group 1 its odd-bin half)
    //      and the reverse per-bin step.  Stage 2: wt + i wq, then wt + i wr,
    //      each split between the groups, with per-bin steps over each
    //      group's own half.  Ten half-length forward transforms per pair.
    // 3a. per-window signal values by base code: (u, v) of the target and
    //     query into the forward sums' space, of the reverse complement into
    //     the reverse sums' space (each overwritten only after its first
    //     pass); w into vv (target, query) and vr (reverse complement)
    float2* uvt = reinterpret_cast<float2*>(aFE);   // [sequence][window][code]
    float2* uvr = reinterpret_cast<float2*>(aRE);   // [window][code]
    auto tables = [&](float E, int k0, int k1, int k2, int k3, float2* uvo, float4* wo) {
      const float4 at = window_values(E, s_wf, s_wmo, k0, k3);   // A at 0, 1; T at 0, 1
      const float4 cg = window_values(E, s_wf, s_wmo, k1, k2);   // C at 0, 1; G at 0, 1
      const float u0 = __fsub_rn(at.x, at.z), v0 = __fsub_rn(cg.x, cg.z), w0 = __fadd_rn(at.x, at.z);
      float4* o = reinterpret_cast<float4*>(uvo);
      o[0] = make_float4(__fsub_rn(at.y, at.z), v0, u0, __fsub_rn(cg.y, cg.z));   // A, C
      o[1] = make_float4(u0, __fsub_rn(cg.x, cg.w), __fsub_rn(at.x, at.w), v0);   // G, T
      *wo = make_float4(__fadd_rn(at.y, at.z), w0, w0, __fadd_rn(at.x, at.w));
    };
    tables((G ? Eq : Et)[g], G * 4 + 0, G * 4 + 1, G * 4 + 2, G * 4 + 3, uvt + (G * NWIN + g) * 4, vv + G * NWIN + g);
    // the reverse complement's channel c has the forward query's mean of 3 - c
    if (G == 0) tables(Er[g], 4 + 3, 4 + 2, 4 + 1, 4 + 0, uvr + g * 4, vr + g);
    __syncthreads();
    // 3b. stage 1: u + i v of the target and the query, both halves
    {
      const uint32_t codes = cw[tid];
      const int len = G ? Q : T;
      const float2* ub = uvt + (G * NWIN + (g >> 4)) * 4;
      float2* bE = G ? WE : ZE;
      first_pass_x2(
          [&](int r) {
            const float2 z = ub[64 * r + ((codes >> (2 * r)) & 3u)];
            return g + 256 * r < len ? z : make_float2(0.f, 0.f);
          },
          g, twLh, twLl, twNh, twNl, bE, bE + N);
      gb();
      fft_pass16_x2<N, N / 16>(bE, bE + N, twNh, twNl, g);
      gb();
      fft_pass16_x2<N, N / 256>(bE, bE + N, twNh, twNl, g);
    }
    __syncthreads();
    // 3c. per-bin step of stage 1 against the target's spectra in ZE / ZO:
    //     f = conj(A) C + B conj(D) = 2 (conj(Ut) Xu + conj(Vt) Xv); the
    //     target-only bins N-1 and N are zero in this basis
    auto per_bin_uv = [&](const float2* VE, const float2* VO, float2* oE, float2* oO) {
      if (G == 0) {
        const int la = lp<LOG2N>(g);
        const int lb = lp<LOG2N>((256 - g) & 255);
#pragma unroll
        for (int it = 0; it <= N / 512; it++) {
          const int m = g + 256 * it;
          if (m > N / 2) break;
          const int pa = la ^ lp<LOG2N>(256 * it);
          const int pb = g ? (lb ^ lp<LOG2N>(N - 256 * (it + 1))) : lp<LOG2N>((N - 256 * it) & (N - 1));
          oE[m] = m == N / 2 ? make_float2(0.f, 0.f) : cadd(cmulc(VE[pa], ZE[pa]), cmulc(ZE[pb], VE[pb]));
        }
      } else {
        const int la = lp<LOG2N>(g);
#pragma unroll
        for (int it = 0; it < N / 512; it++) {
          const int m = g + 256 * it;
          const int pa = la ^ lp<LOG2N>(256 * it);
          const int pb = pa ^ lp<LOG2N>(N - 1);
          oO[m] = m == N / 2 - 1 ? make_float2(0.f, 0.f) : cadd(cmulc(VO[pa], ZO[pa]), cmulc(ZO[pb], VO[pb]));
        }
      }
    };
    per_bin_uv(WE, WO, aFE, aFO);
    __syncthreads();
    // 3d. u + i v of the reverse complement: the even-bin half in group 0
    //     (into WE), the odd-bin half in group 1 (into WO)
    {
      float2* b = G ? WO : WE;
      const uint32_t codes = cr[g];
      const float2* ub = uvr + (g >> 4) * 4;
      first_pass_x1(
          [&](int r) {
            const float2 z = ub[64 * r + ((codes >> (2 * r)) & 3u)];
            return g + 256 * r < Q ? z : make_float2(0.f, 0.f);
          },
          G == 1, g, twLh, twLl, twNh, twNl, b);
      gb();
      fft_pass<16, N, N / 16, false>(b, twNh, twNl, g, 256);
      gb();
      fft_pass<16, N, N / 256, false>(b, twNh, twNl, g, 256);
    }
    __syncthreads();
    // 3e. the reverse strand's per-bin step of stage 1
    per_bin_uv(WE, WO, aRE, aRO);
    gb();   // stage 2 overwrites what the group's per-bin step read (group 0 ZE, group 1 WO)
    // 3f. stage 2: wt + i wq, then wt + i wr; each group transforms its half
    //     and adds f = 2 Im(H E) - i (|E|^2 - |H|^2) = 4 conj(Wt) Wx over it
    float2* bw = G ? WO : ZE;
    const uint32_t ct = cw[g];
    const float* wt_tab = reinterpret_cast<const float*>(vv) + (g >> 4) * 4;
#pragma unroll 1
    for (int stg = 0; stg < 2; stg++) {
      const uint32_t cx = stg ? cr[g] : cw[NWIN + g];
      const float* wx_tab = stg ? reinterpret_cast<const float*>(vr) + (g >> 4) * 4
                                : reinterpret_cast<const float*>(vv) + NWIN * 4 + (g >> 4) * 4;
      first_pass_x1(
          [&](int r) {
            const float wt = wt_tab[64 * r + ((ct >> (2 * r)) & 3u)];
            const float wx = wx_tab[64 * r + ((cx >> (2 * r)) & 3u)];
            return make_float2(g + 256 * r < T ? wt : 0.f, g + 256 * r < Q ? wx : 0.f);
          },
          G == 1, g, twLh, twLl, twNh, twNl, bw);
      gb();
      fft_pass<16, N, N / 16, false>(bw, twNh, twNl, g, 256);
      gb();
      fft_pass<16, N, N / 256, false>(bw, twNh, twNl, g, 256);
      gb();
      float2* oE = stg ? aRE : aFE;
      float2* oO = stg ? aRO : aFO;
      if (G == 0) {
        const int la = lp<LOG2N>(g);
        const int lb = lp<LOG2N>((256 - g) & 255);
#pragma unroll 3
        for (int it = 0; it <= N / 512; it++) {
          const int m = g + 256 * it;
          if (m >= N / 2) break;
          const int pa = la ^ lp<LOG2N>(256 * it);
          const int pb = g ? (lb ^ lp<LOG2N>(N - 256 * (it + 1))) : lp<LOG2N>((N - 256 * it) & (N - 1));
          float2 f, r;
          pair_bin_w(ZE[pa], ZE[pb], f, r);
          oE[m] = cadd(oE[m], f);
        }
      } else {
        const int la = lp<LOG2N>(g);
#pragma unroll 3
        for (int it = 0; it < N / 512; it++) {
          const int m = g + 256 * it;
          if (m == N / 2 - 1) break;
          const int pa = la ^ lp<LOG2N>(256 * it);
          const int pb = pa ^ lp<LOG2N>(N - 1);
          float2 f, r;
          pair_bin_w(WO[pa], WO[pb], f, r);
          oO[m] = cadd(oO[m], f);
        }
      }
      gb();   // the next stage overwrites the group's buffer
    }
    __syncthreads();

    // ---- 4. inverses: group 0 the forward strand into ZE, group 1 the
    //      reverse strand into WE (bins N-1 and N: zero for both strands).
    //      Sums and the pack carry factors 4 and 2: FindTop scales by
    //      1/(8N). ----
    float2* buf = G ? WE : ZE;
    auto SF = [&](int k) -> float2 { return (k & 1) ? aFO[k >> 1] : aFE[k >> 1]; };
    auto SRc = [&](int k) -> float2 {
      if (k >= N - 1) return (k & 1) ? aFO[k >> 1] : aFE[k >> 1];
      return (k & 1) ? aRO[k >> 1] : aRE[k >> 1];
    };
    if (G == 0) hermitian_pack<LOG2L, 256>(ZE, both_bins<N>(SF), twLh, twLl, g, 1.0f);
    else hermitian_pack<LOG2L, 256>(WE, both_bins<N>(SRc), twLh, twLl, g, 1.0f);
    gb();
    fft_inverse<LOG2N, Plan<LOG2N>, Plan<LOG2N>::n - 1, GroupBarrier>(buf, twNh, twNl, g, 256, gb);
    // ---- 5. FindTop, one strand per group ----
    find_top<LOG2L, 256, GroupBarrier>(P, P.pairs[pidx].flags, P.pairs[pidx].off_base, pidx, G, buf, g, s_warp[G], gb,
                                       1.0f / (float)(8 * N));
    __syncthreads();   // buffers and per-pair words are reused by the next pair
    if (tid == 0 && s_flags) {
      // bytes outside the premise (rare): the pass above is void.  A byte
      // >= 128 voids the pair; other letters send it to the per-strand
      // kernel, which redoes its offsets and near-threshold lags.
      if (s_flags & 1u) {
        P.off_cnt[pidx * 2] = 0;
        P.off_cnt[pidx * 2 + 1] = 0;
        P.pair_flags[pidx] = PF_INVALID;
        if (P.strad_cnt) {
          P.strad_cnt[pidx * 2] = 0;
          P.strad_cnt[pidx * 2 + 1] = 0;
        }
      } else {
        P.fb_list[atomicAdd(P.fb_cnt, 1)] = pidx;
      }
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

static size_t spec_smem_bytes() {
  constexpr size_t N = 4096, NH = N / 64;
  return (4 * N + 2 * (NH + 64) + 16 * TW16_ROW) * sizeof(float2)   // 4 transforms, twiddles
         + N                                        // chunk bytes
         + 256 * sizeof(float)                      // entropy weight per window
         + 2 * 256 * sizeof(float4)                 // (u, v) by base code per window
         + 256 * sizeof(uint32_t)                   // 2-bit codes of positions g + 256 r
         + 256 * sizeof(float4);                    // w by base code per window
}

__device__ __forceinline__ void spec_prefetch(const SpecParams& S, int u, uint8_t* sb, int tid) {
  if (tid >= 256) return;   // 256 pieces of 16 bytes
  const ChunkDesc c = S.chunks[u];
  const int valid = min(max(c.len - 16 * tid, 0), 16);
  const uint8_t* src = S.pool + c.off + (valid > 0 ? 16 * tid : 0);
  const uint32_t dst = (uint32_t)__cvta_generic_to_shared(sb + 16 * tid);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid) : "memory");
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <int LOG2L>
__global__ void __launch_bounds__(NT_PAIR2, 1) spec_kernel(const SpecParams S) {
  constexpr int L = 1 << LOG2L;
  constexpr int N = L >> 1;
  constexpr int WIN = L / 512;
  constexpr int NWIN = 256;
  constexpr int NH = N / 64;
  static_assert(N == 4096, "thread g of a group owns positions g + 256 r, r < 16");
  extern __shared__ __align__(16) unsigned char smem[];
  float2* buf = reinterpret_cast<float2*>(smem);   // [channel pair][even, odd][N]
  float2* twNh = buf + 4 * N;
  float2* twNl = twNh + NH;
  float2* twLh = twNl + 64;
  float2* twLl = twLh + NH;
  float2* tw16t = twLl + 64;   // twiddles of the span-256 pass (build_tw16_table)
  uint8_t* sb = reinterpret_cast<uint8_t*>(tw16t + 16 * TW16_ROW);
  float* Es = reinterpret_cast<float*>(sb + N);
  float4* vv = reinterpret_cast<float4*>(Es + NWIN);     // (u, v) by base code per window
  uint32_t* cw = reinterpret_cast<uint32_t*>(vv + 2 * NWIN);
  float4* wv = reinterpret_cast<float4*>(cw + NWIN);      // w by base code per window
  __shared__ int s_cnt4[4];
  __shared__ unsigned s_flags;   // bit 0: a byte >= 128; bit 1: a byte other than A, C, G, T
  __shared__ int s_take;         // the CTA's next chunk
  __shared__ double s_wmo[2][8];
  __shared__ Split3 s_wf[2][8];

  const int tid = threadIdx.x;
  const int G = tid >> 8;   // signal: 0 u + i v, 1 w
  const int g = tid & 255;
  const GroupBarrier gb{1 + G, 256};
  for (int i = tid; i < NH; i += NT_PAIR2) {
    twNh[i] = S.tab.twN_hi[i];
    twLh[i] = S.tab.twL_hi[i];
  }
  if (tid < 64) {
    twNl[tid] = S.tab.twN_lo[tid];
    twLl[tid] = S.tab.twL_lo[tid];
  }
  if ((int)blockIdx.x < S.count) spec_prefetch(S, blockIdx.x, sb, tid);
  __syncthreads();
  build_tw16_table(tw16t, twNh, twNl, N / 256, tid);   // read after the first barrier of the loop
  // chunks in the order take_item gives, each taken one chunk ahead, as
  // corr_pair2_kernel takes its pairs
  const int SR = static_rounds(S.count);
  if (tid == 0) s_take = take_item(S.work, 1, SR);
  for (int u = blockIdx.x, r = 0; u < S.count; r++) {
    const int len = S.chunks[u].len;
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    if (tid < 4) s_cnt4[tid] = 0;
    if (tid == 0) s_flags = 0u;
    __syncthreads();
    const int nu = s_take;
    const int next = nu < S.count ? nu : -1;
    int take = 0;
    if (tid == 0) take = take_item(S.work, r + 2, SR);
    // thread g < 256 takes bytes 16g..16g+15, which are also entropy window g
    // (WIN = 16): byte checks, 2-bit codes, base counts and the window's
    // entropy weight from one load, as corr_pair2_kernel's prologue
    uint32_t* cwin = reinterpret_cast<uint32_t*>(vv);   // codes per window; vv is free until the window values
    if (tid < 256) {
      const int g = tid;
      const int valid = len - 16 * g;
      const uint4 v = *reinterpret_cast<const uint4*>(sb + 16 * g);
      const uint32_t x[4] = {v.x, v.y, v.z, v.w};
      auto nz = [](uint32_t y) { return (((y & 0x7f7f7f7fu) + 0x7f7f7f7fu) | y) & 0x80808080u; };
      uint32_t high = 0u, bad = 0u, p0 = 0u, p1 = 0u, codes = 0u;
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const int vk = min(max(valid - 4 * k, 0), 4);
        const uint32_t m = vk >= 4 ? 0xffffffffu : (1u << (8 * vk)) - 1u;
        high |= x[k] & m & 0x80808080u;
        bad |= nz(x[k] ^ 0x41414141u) & nz(x[k] ^ 0x43434343u) & nz(x[k] ^ 0x47474747u) & nz(x[k] ^ 0x54545454u) &
               m & 0x80808080u;
        const uint32_t cd = ((x[k] >> 1) ^ (x[k] >> 2)) & 0x03030303u & m;
        p0 |= (((cd & 0x01010101u) * 0x10204080u) >> 28) << (4 * k);
        p1 |= ((((cd >> 1) & 0x01010101u) * 0x10204080u) >> 28) << (4 * k);
        const uint32_t c2 = cd | (cd >> 6);
        codes |= ((c2 & 0xfu) | ((c2 >> 12) & 0xf0u)) << (8 * k);
      }
      cwin[g] = codes;
      const int nv = min(max(valid, 0), 16);
      const int nt = __popc(p0 & p1), nc = __popc(p0) - nt, ng = __popc(p1) - nt, na = nv - nc - ng - nt;
      float E = 0.f;
      if (len < 1024) {
        E = 1.f;
      } else if (nv == 16) {
        E = __ldg(&S.tab.ent_acgt[(na * (WIN + 1) + nc) * (WIN + 1) + ng]);
      } else if (nv > 0) {
        int a4 = 0, c4 = 0, g4 = 0, t4 = 0;
        for (int j = 0; j < nv; j++) {
          const uchar4 q = c_w4q[sb[16 * g + j] & 127u];   // a byte >= 128 voids the pair
          a4 += q.x; c4 += q.y; g4 += q.z; t4 += q.w;
        }
        const double* et = S.tab.ent + nv * (4 * WIN + 1);
        const double sv =
            __dadd_rn(__dadd_rn(__dadd_rn(__ldg(et + a4), __ldg(et + c4)), __ldg(et + g4)), __ldg(et + t4));
        E = __double2float_rn(-sv);
        if (E < 0.f) E = 0.f;
      }
      Es[g] = E;
      const uint32_t lo = __reduce_add_sync(0xffffffffu, (uint32_t)na | ((uint32_t)nc << 16));
      const uint32_t hi = __reduce_add_sync(0xffffffffu, (uint32_t)ng | ((uint32_t)nt << 16));
      const uint32_t fl = __reduce_or_sync(0xffffffffu, (high ? 1u : 0u) | (bad ? 2u : 0u));
      if ((tid & 31) == 0) {
        atomicAdd(&s_cnt4[0], 4 * (int)(lo & 0xffffu));
        atomicAdd(&s_cnt4[1], 4 * (int)(lo >> 16));
        atomicAdd(&s_cnt4[2], 4 * (int)(hi & 0xffffu));
        atomicAdd(&s_cnt4[3], 4 * (int)(hi >> 16));
        if (fl) atomicOr(&s_flags, fl);
      }
    }
    __syncthreads();   // the chunk bytes are no longer read
    if (next >= 0) spec_prefetch(S, next, sb, tid);
    const uint32_t flg = s_flags;
    if (flg) {
      if (tid == 0) S.chunk_flags[u] = ((flg & 1u) ? CF_HIGH : 0u) | CF_GENERIC;
      if (tid == 0) s_take = take;
      __syncthreads();   // cwin (in vv), the flags and the next chunk's index are reused
      u = nu;
      continue;
    }
    if (tid < 4) {
      mean_terms(s_cnt4[tid], len, s_wmo[0][tid], s_wmo[1][tid], s_wf[0][tid], s_wf[1][tid]);
    }
    if (tid >= 256) {   // the codes of positions g + 256 r, one word per g
      const int g = tid - 256;
      const uint32_t* cs = cwin + (g >> 4);
      const int sh = 2 * (g & 15);
      uint32_t w = 0;
#pragma unroll
      for (int r = 0; r < 16; r++) w |= ((cs[16 * r] >> sh) & 3u) << (2 * r);
      cw[g] = w;
    }
    __syncthreads();
    // group 0 transforms u + i v (u = A - T, v = C - G), group 1 w + 0 i
    // (w = A + T = -(C + G)): the signal values by base code per window from
    // the channel values float(entropy * (weight - mean)) (CrossCorr.cc:123)
    // with one FP32 add each, as corr_pair2_kernel forms them
    float2* bE = buf + 2 * G * N;
    float2* bO = bE + N;
    float2* uvt = reinterpret_cast<float2*>(vv);   // [window][code]
    {
      const float4 at = window_values(Es[g], s_wf, s_wmo, 0, 3);   // A at 0, 1; T at 0, 1
      const float w0 = __fadd_rn(at.x, at.z);
      if (G == 0) {
        const float4 cg = window_values(Es[g], s_wf, s_wmo, 1, 2);   // C at 0, 1; G at 0, 1
        const float u0 = __fsub_rn(at.x, at.z), v0 = __fsub_rn(cg.x, cg.z);
        float4* o = reinterpret_cast<float4*>(uvt + g * 4);
        o[0] = make_float4(__fsub_rn(at.y, at.z), v0, u0, __fsub_rn(cg.y, cg.z));   // A, C
        o[1] = make_float4(u0, __fsub_rn(cg.x, cg.w), __fsub_rn(at.x, at.w), v0);   // G, T
      } else {
        wv[g] = make_float4(__fadd_rn(at.y, at.z), w0, w0, __fadd_rn(at.x, at.w));
      }
    }
    gb();
    {
      const uint32_t codes = cw[g];
      const float2* ub = uvt + (g >> 4) * 4;
      const float* wb = reinterpret_cast<const float*>(wv) + (g >> 4) * 4;
      first_pass_x2(
          [&](int r) {
            const uint32_t k = (codes >> (2 * r)) & 3u;
            const float2 z = G ? make_float2(wb[64 * r + k], 0.f) : ub[64 * r + k];
            return g + 256 * r < len ? z : make_float2(0.f, 0.f);
          },
          g, twLh, twLl, twNh, twNl, bE, bO);
    }
    gb();
    fft_pass16_x2_tab<N, N / 16>(bE, bO, tw16t, g);
    gb();
    fft_pass16_x2<N, N / 256>(bE, bO, twNh, twNl, g);
    gb();
    // out in bin order: bin m of the even-bin transform at [2G][m], odd at
    // [2G + 1][m]; of w's spectrum (real signal: W(L - k) = conj W(k)) only
    // the bins the pair kernel reads, m <= N/2 of each half
    float2* out = S.spec + ((size_t)u * 4 + 2 * G) * N;
    const int la = lp<LOG2L - 1>(g);
#pragma unroll 4
    for (int it = 0; it < N / 256; it++) {
      const int m = g + 256 * it;
      if (G && m > N / 2) break;
      const int pa = la ^ lp<LOG2L - 1>(256 * it);
      out[m] = bE[pa];
      out[N + m] = bO[pa];
    }
    if (tid == 0) {
      S.chunk_flags[u] = 0u;
      s_take = take;
    }
    __syncthreads();
    u = nu;
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

static size_t corr_spec_smem_bytes() {
  constexpr size_t N = 4096, NH = N / 64;
  return (2 * N + 2 * N + 16 + 2 * (NH + 64) + 16 * TW16_ROW) * sizeof(float2);   // 2 inverses, F and R sums, twiddles
}

template <int LOG2L>
__global__ void __launch_bounds__(NT_PAIR2, 1) corr_spec_kernel(const CorrParams P) {
  constexpr int L = 1 << LOG2L;
  constexpr int N = L >> 1;
  constexpr int WIN = L / 512;
  constexpr int NH = N / 64;
  extern __shared__ __align__(16) unsigned char smem[];
  float2* ZE = reinterpret_cast<float2*>(smem);   // forward-strand inverse
  float2* WE = ZE + N;                            // reverse-strand inverse
  float2* aFE = WE + N;
  float2* aFO = aFE + (N / 2 + 8);
  float2* aRE = aFO + N / 2;
  float2* aRO = aRE + (N / 2 + 8);
  float2* twNh = aRO + N / 2;
  float2* twNl = twNh + NH;
  float2* twLh = twNl + 64;
  float2* twLl = twLh + NH;
  float2* tw16t = twLl + 64;   // twiddles of the span-256 inverse pass (build_tw16_table)
  __shared__ int s_warp[2][2 * 256 / 32];
  __shared__ int s_take;   // the CTA's next pair

  const int tid = threadIdx.x;
  const int G = tid >> 8;   // product: 0 even bins, 1 odd bins; then 0 forward strand, 1 reverse
  const int g = tid & 255;
  const GroupBarrier gb{1 + G, 256};
  for (int i = tid; i < NH; i += NT_PAIR2) {
    twNh[i] = P.tab.twN_hi[i];
    twLh[i] = P.tab.twL_hi[i];
  }
  if (tid < 64) {
    twNl[tid] = P.tab.twN_lo[tid];
    twLl[tid] = P.tab.twL_lo[tid];
  }
  __syncthreads();
  build_tw16_table(tw16t, twNh, twNl, N / 256, tid);   // read after the loop's barriers
  // pairs in the order take_item gives, each taken one pair ahead, as
  // corr_pair2_kernel takes them
  const int S = static_rounds(P.count);
  if (tid == 0) s_take = take_item(P.work, 1, S);
  __syncthreads();
  for (int p = blockIdx.x, r = 0; p < P.count; r++) {
    const int pidx = P.first + p;
    const int np = s_take;
    int take = 0;
    if (tid == 0) take = take_item(P.work, r + 2, S);
    const int tc = P.pair_chunk[2 * pidx], qc = P.pair_chunk[2 * pidx + 1];
    const int Q = P.pairs[pidx].qlen;
    const uint32_t fl = P.chunk_flags[tc] | P.chunk_flags[qc];
    if (fl || (Q >= 1024 && Q % WIN != 0) || P.dbg_sig) {   // the same for every thread
      if (tid == 0) {
        if (fl & CF_HIGH) {
          P.off_cnt[pidx * 2] = 0;
          P.off_cnt[pidx * 2 + 1] = 0;
          P.pair_flags[pidx] = PF_INVALID;
        } else if (P.fb2_list && !fl && !P.dbg_sig) {
          P.fb2_list[atomicAdd(P.fb2_cnt, 1)] = pidx;   // a ragged query window: corr_rcq_kernel takes it
        } else {
          P.fb_list[atomicAdd(P.fb_cnt, 1)] = pidx;
        }
      }
      if (tid == 0) s_take = take;
      __syncthreads();   // s_take is rewritten for the next pair
      p = np;
      continue;
    }
    if (tid == 0) P.pair_flags[pidx] = P.pairs[pidx].flags & PF_FAST;
    // ---- per-bin step from the stored spectra (u + i v both halves, W of
    //      the real signal w = A + T): with A, B, C, D the u + i v spectra of
    //      target and query at m and N-m,
    //        4 sum_c conj(T_c) Q_c = conj(A) C + B conj(D) + 4 conj(Wt) Wq
    //        4i sum_c T_c Q_comp(c) = -i (A conj(D) + conj(B) C) + 4i Wt Wq,
    //      and the target-only bins N-1 and N are zero (the basis of
    //      corr_pair2_kernel, which forms W from a joint transform) ----
    const float2* __restrict__ Ts = P.spec + (size_t)tc * 4 * N;
    const float2* __restrict__ Qs = P.spec + (size_t)qc * 4 * N;
    auto bin = [](float2 A, float2 B, float2 C, float2 D, float2 Wt, float2 Wq, float2& f, float2& r) {
      const float2 s = cadd(cmulc(A, D), cmulc(C, B));
      const float2 fw = cmulc(Wq, Wt), rw = cmul(Wt, Wq);
      f = cadd(cadd(cmulc(C, A), cmulc(B, D)), make_float2(4.f * fw.x, 4.f * fw.y));
      r = cadd(make_float2(s.y, -s.x), make_float2(-4.f * rw.y, 4.f * rw.x));
    };
    if (G == 0) {
#pragma unroll 3
      for (int it = 0; it <= N / 512; it++) {
        const int m = g + 256 * it;
        if (m > N / 2) break;
        if (m == N / 2) {
          aFE[m] = make_float2(0.f, 0.f);
          continue;
        }
        const int mb = (N - m) & (N - 1);
        float2 f, r;
        bin(__ldg(Ts + m), __ldg(Ts + mb), __ldg(Qs + m), __ldg(Qs + mb), __ldg(Ts + 2 * N + m),
            __ldg(Qs + 2 * N + m), f, r);
        aFE[m] = f;
        aRE[m] = r;
      }
    } else {
#pragma unroll 4
      for (int it = 0; it < N / 512; it++) {
        const int m = g + 256 * it;
        if (m == N / 2 - 1) {
          aFO[m] = make_float2(0.f, 0.f);
          continue;
        }
        const int mb = N - 1 - m;
        float2 f, r;
        bin(__ldg(Ts + N + m), __ldg(Ts + N + mb), __ldg(Qs + N + m), __ldg(Qs + N + mb), __ldg(Ts + 3 * N + m),
            __ldg(Qs + 3 * N + m), f, r);
        aFO[m] = f;
        aRO[m] = r;
      }
    }
    __syncthreads();
    // ---- inverses and FindTop, as corr_pair2_kernel ----
    float2* buf = G ? WE : ZE;
    if (G == 0) {
      auto SF = [&](int k) -> float2 { return (k & 1) ? aFO[k >> 1] : aFE[k >> 1]; };
      hermitian_pack<LOG2L, 256>(ZE, both_bins<N>(SF), twLh, twLl, g, 1.0f);
    } else {
      hermitian_pack<LOG2L, 256>(
          WE, [&](int k, float2& a, float2& b) { reverse_bins<LOG2L>(k, Q, aFE, aFO, aRE, aRO, twLh, twLl, a, b); },
          twLh, twLl, g, 1.0f);
    }
    gb();
    fft_pass<16, N, 16, true>(buf, twNh, twNl, g, 256);
    gb();
    fft_pass16_inv_tab<N, 256>(buf, tw16t, g);
    gb();
    fft_pass<16, N, N, true>(buf, twNh, twNl, g, 256);
    gb();
    find_top<LOG2L, 256, GroupBarrier>(P, P.pairs[pidx].flags, P.pairs[pidx].off_base, pidx, G, buf, g, s_warp[G], gb,
                                       1.0f / (float)(8 * N));
    if (tid == 0) s_take = take;
    __syncthreads();
    p = np;
  }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
cudaError_t prepare_scan_kernels();
cudaError_t upload_scan_constants(const unsigned char* rc256, const uchar4* w4q128, const double* w4d);

template <int LOG2L, int NT = NT_CORR>
static cudaError_t set_corr_attrs() {
  return cudaFuncSetAttribute(corr_kernel<LOG2L, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)corr_smem_bytes(LOG2L));
}

// The per-strand kernel at FFT length 2^log2L with nt threads per strand
// (512; 256 up to 8192; 128 up to 4096), grid (x, 2).
static cudaError_t launch_strand(int log2L, int nt, dim3 grid, const CorrParams& p, cudaStream_t s) {
  const size_t sm = corr_smem_bytes(log2L);
#define XC_STRAND(LG, NTV)                                  \
  if (log2L == LG && nt == NTV) {                           \
    corr_kernel<LG, NTV><<<grid, NTV, sm, s>>>(p);          \
    return cudaGetLastError();                              \
  }
  XC_STRAND(10, 512) XC_STRAND(10, 256) XC_STRAND(10, 128)
  XC_STRAND(11, 512) XC_STRAND(11, 256) XC_STRAND(11, 128)
  XC_STRAND(12, 512) XC_STRAND(12, 256) XC_STRAND(12, 128)
  XC_STRAND(13, 512) XC_STRAND(13, 256)
  XC_STRAND(14, 512) XC_STRAND(15, 512)
#undef XC_STRAND
  return cudaErrorInvalidValue;
}

bool strand_threads_ok(int log2L, int nt) {
  return nt == 512 || (nt == 256 && log2L <= 13) || (nt == 128 && log2L <= 12);
}

cudaError_t prepare_kernels() {
  cudaError_t e = cudaFuncSetAttribute(corr_pair_kernel<PAIR_LOG2L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)corr_pair_smem_bytes(PAIR_LOG2L));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(corr_pair2_kernel<PAIR_LOG2L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)corr_pair2_smem_bytes());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(corr_rcq_kernel<PAIR_LOG2L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)corr_rcq_smem_bytes());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(spec_kernel<PAIR_LOG2L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)spec_smem_bytes());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(corr_spec_kernel<PAIR_LOG2L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)corr_spec_smem_bytes());
  if (e != cudaSuccess) return e;
  if ((e = set_corr_attrs<10>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<11>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<12>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<13>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<10, 256>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<11, 256>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<12, 256>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<13, 256>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<10, 128>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<11, 128>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<12, 128>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<14>()) != cudaSuccess) return e;
  if ((e = set_corr_attrs<15>()) != cudaSuccess) return e;
  return prepare_scan_kernels();
}

cudaError_t launch_corr(int log2L, const CorrParams& p, int npairs, cudaStream_t s) {
  if (npairs <= 0) return cudaSuccess;
  dim3 grid(npairs, 2);
  const int nt = strand_threads_ok(log2L, p.strand_threads) ? p.strand_threads : NT_CORR;
  if (p.fb_list) {
    // both strands per CTA, corr_rcq_kernel over the ragged query windows
    // (fb2_list), then corr_kernel over the pairs handed back: one wave of
    // CTAs striding over each list (the counts start at zero)
    if (log2L != PAIR_LOG2L) return cudaErrorInvalidValue;
    static const int sms = [] {
      int dev = 0, n = 152;
      if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
      return n;
    }();
    CorrParams q = p;
    q.count = npairs;
    if (p.pair_form == 2) {   // persistent: one CTA per SM strides over the pairs
      // (the bucket's ragged query windows, when given as a range, come last
      // and go to corr_rcq_kernel alone)
      q.count = npairs - (p.fb2_list ? 0 : p.rcq_count);
      if (q.count > 0)
        corr_pair2_kernel<PAIR_LOG2L><<<std::min(q.count, sms), NT_PAIR2, corr_pair2_smem_bytes(), s>>>(q);
      if (p.fb2_list || p.rcq_count > 0)   // the pairs with a ragged query window
        corr_rcq_kernel<PAIR_LOG2L><<<std::min(p.fb2_list ? npairs : p.rcq_count, sms), NT_PAIR2,
                                      corr_rcq_smem_bytes(), s>>>(q);
    } else {
      q.fb2_list = nullptr;
      q.rcq_count = 0;
      corr_pair_kernel<PAIR_LOG2L><<<npairs, NT_PAIR, corr_pair_smem_bytes(PAIR_LOG2L), s>>>(q);
    }
    grid.x = std::min(npairs, sms * (NT_CORR / nt));
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_strand(log2L, nt, grid, p, s);
}

cudaError_t launch_corr_spec(const SpecParams& sp, const CorrParams& p, int npairs, cudaStream_t s) {
  if (npairs <= 0) return cudaSuccess;
  static const int sms = [] {
    int dev = 0, n = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
  }();
  if (!p.fb_list || !p.pair_chunk) return cudaErrorInvalidValue;
  if (sp.count > 0) spec_kernel<PAIR_LOG2L><<<std::min(sp.count, sms), NT_PAIR2, spec_smem_bytes(), s>>>(sp);
  CorrParams q = p;
  q.count = npairs;
  corr_spec_kernel<PAIR_LOG2L><<<std::min(npairs, sms), NT_PAIR2, corr_spec_smem_bytes(), s>>>(q);
  if (p.fb2_list)   // the pairs with a ragged query window it handed on
    corr_rcq_kernel<PAIR_LOG2L><<<std::min(npairs, sms), NT_PAIR2, corr_rcq_smem_bytes(), s>>>(q);
  // the pairs handed back: one wave of per-strand CTAs striding over the list
  CorrParams h = p;
  h.pair_chunk = nullptr;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int nt = strand_threads_ok(PAIR_LOG2L, p.strand_threads) ? p.strand_threads : NT_CORR;
  return launch_strand(PAIR_LOG2L, nt, dim3(std::min(npairs, sms * (NT_CORR / nt)), 2), h, s);
}

cudaError_t upload_constants(const unsigned char* rc256, const uchar4* w4q128, const double* w4d) {
  cudaError_t e = upload_constants_here(rc256, w4q128, w4d);
  if (e != cudaSuccess) return e;
  return upload_scan_constants(rc256, w4q128, w4d);
}

}  // namespace xc
