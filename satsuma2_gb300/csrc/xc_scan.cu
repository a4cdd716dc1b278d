// Scan and finalize kernels of the satsuma2 cross-correlation path (sm_103a).
//
//   scan_kernel<log2 L>  one CTA of 128 threads per (chunk pair, strand):
//                        SeqAnalyzer::DoOne over every FindTop offset, then
//                        FilterMatches on the raw segments.
//     A/C/G/T pairs, in rounds of 128 diagonals (longest first):
//       pass 1 (thread = diagonal): on 2-bit bitplanes, 32 equality bits per
//         word op, a branch-free screen marks the words holding a 4-check
//         block whose 49-position span holds >= 19 equal bases (the eight
//         blocks of a word tested at once in byte lanes);
//       items: the marked words of the round laid out contiguously per
//         diagonal by a prefix sum, processed one per thread (phase AB): the
//         word's 32 exact window bits, four byte lanes at once; the bit of
//         the check before the word from the same equality words; falls and
//         closing ends of runs, queued as (item, bit) with one atomic per
//         warp (items that overrun the queue run in place after it);
//       phase C (thread = segment): run start from the same word or by
//         looking back, equal-base count, FP32 probability screen, exact FP64
//         GetMatchProbability / PrintMatch for survivors.
//     Other pairs (N, IUPAC, unknown letters): the reference's byte-table
//       DoOne per lane and the exact double sums.
//   finalize kernels     order each strand's results as the reference appends
//                        them and pack them densely.
#include "xc_device.cuh"

namespace xc {

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
  static constexpr int MW = (TW + 31) / 32;  // marked-word mask entries per diagonal
  // Marked-block items of one pass-2 sub-range and the segment queue (4 bytes
  // each; item indices fit 12 bits).  The queue shares its bytes with the
  // chunk byte arrays, which only the byte-table path fills.
  static constexpr int ICAP = 1280;   // items (8 bytes each: word, passing bits)
  static constexpr int QCAP = 2048;
  // Survivors of the probability screen awaiting the FP64 tail, after the
  // queue: 64, or as many as the rest of the byte region holds.
  static constexpr int SVB = 28;   // bytes per survivor (Surv)
  static constexpr int SVCAP = 2 * N > QCAP * 4 + 64 * SVB ? (2 * N - QCAP * 4) / SVB : 64;
  static constexpr size_t region = (size_t)QCAP * 4 + (size_t)SVCAP * SVB > 2 * (size_t)N
                                       ? (size_t)QCAP * 4 + (size_t)SVCAP * SVB
                                       : 2 * (size_t)N;
  static constexpr size_t bytes = region +
      (size_t)(2 * TWP + (TW + 1) + 2 * QWP + (TW + 1) + OFF_CHUNK + MW * NT_SCAN + 2 * ICAP + NT_SCAN) * 4 +
      (size_t)OFF_CHUNK * 2;
};

size_t scan_smem_bytes(int log2L) {
  switch (log2L) {
    case 10: return ScanGeom<10>::bytes;
    case 11: return ScanGeom<11>::bytes;
    case 12: return ScanGeom<12>::bytes;
    case 13: return ScanGeom<13>::bytes;
    case 14: return ScanGeom<14>::bytes;
    case 15: return ScanGeom<15>::bytes;
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
__device__ __forceinline__ int gc_count(const uint2* b, const int* pref, int a, int e) {
  const int wa = a >> 5, we = e >> 5;
  const uint2 x = b[wa], y = b[we];
  const int ga = pref[wa] + __popc((x.x ^ x.y) & lowmask(a & 31));
  const int ge = pref[we] + __popc((y.x ^ y.y) & lowmask(e & 31));
  return ge - ga;
}

__device__ __forceinline__ int warp_incl_sum(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// Warp-cooperative exclusive prefix of per-word G/C counts -> pref[0..nw].
__device__ __forceinline__ void gc_prefix(const uint2* b, int* pref, int nw, int lane) {
  int run = 0;
  for (int w0 = 0; w0 < nw; w0 += 32) {
    const int w = w0 + lane;
    const int c = w < nw ? __popc(b[w].x ^ b[w].y) : 0;
    const int incl = warp_incl_sum(c, lane);
    if (w < nw) pref[w] = run + incl - c;
    run += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (lane == 0) pref[nw] = run;
}

// 2-bit code planes of len bytes at g (16-byte aligned, readable up to the
// next 16-byte boundary) into words 0..nw-1 of p (plane 0 in .x, plane 1 in
// .y: the two words of a position range come in one 8-byte access),
// positions >= len zero.
// Each lane loads 16 bytes, forms four codes per 32-bit word
// ((b>>1 ^ b>>2) & 3, A=0 C=1 G=2 T=3), gathers their plane bits with one
// multiply per word, and lanes 2j, 2j+1 join their 16 bits into one word.
// Every thread of the CTA calls it.
__device__ __forceinline__ void build_planes(const uint8_t* __restrict__ g, int len, uint2* p, int nw, int tid) {
  for (int c0 = 0; c0 < 2 * nw; c0 += NT_SCAN) {
    const int c = c0 + tid;
    uint32_t m0 = 0u, m1 = 0u;
    if (c < 2 * nw && 16 * c < len) {
      const uint4 v = *reinterpret_cast<const uint4*>(g + 16 * c);
      const uint32_t x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int k = 0; k < 4; k++) {
        const uint32_t cd = ((x[k] >> 1) ^ (x[k] >> 2)) & 0x03030303u;
        m0 |= (((cd & 0x01010101u) * 0x10204080u) >> 28) << (4 * k);          // bit 0 of byte j -> bit j
        m1 |= ((((cd >> 1) & 0x01010101u) * 0x10204080u) >> 28) << (4 * k);
      }
      const int valid = len - 16 * c;
      if (valid < 16) {
        m0 &= (1u << valid) - 1u;
        m1 &= (1u << valid) - 1u;
      }
    }
    const uint32_t h0 = __shfl_down_sync(0xffffffffu, m0, 1), h1 = __shfl_down_sync(0xffffffffu, m1, 1);
    if (!(tid & 1) && c < 2 * nw) p[c >> 1] = make_uint2(m0 | (h0 << 16), m1 | (h1 << 16));
  }
}

// Per-nibble popcount of a 32-bit word.
__device__ __forceinline__ uint32_t nib_popc(uint32_t x) {
  x = x - ((x >> 1) & 0x55555555u);
  return (x & 0x33333333u) + ((x >> 2) & 0x33333333u);
}

// Pass-1 screen of one word (equality words e2, e1, e0 of the word and the
// two before it; check u of the word has the window of positions u-45..u,
// bits u+19..u+64 of e2:e1:e0).  True when some block of four checks
// 4b..4b+3 (b < 8) has >= MIN_HITS equal bases in its 49-position span, a
// necessary condition for any of its checks to pass.  The span counts are
// c(b) = c(0) + sum_{k<b} (entering nibble k - leaving nibble k), formed for
// all eight blocks at once in byte lanes: even blocks 2j in one word, odd
// blocks 2j+1 in another, each count biased by 128 - MIN_HITS so that bit 7
// of its byte is the test.  Every byte stays within 0..255 (counts <= 49,
// nibble differences biased by 4, prefix sums <= 48).  Returns the test bits
// (nonzero: some block passes) and in edge those of blocks 0 and 7.
__device__ __forceinline__ uint32_t screen_word(uint32_t e2, uint32_t e1, uint32_t e0, uint32_t& edge) {
  const uint32_t pl = nib_popc(__funnelshift_r(e2, e1, 19));   // nibble k: bits 19+4k.. leaving
  const uint32_t pe = nib_popc(e0 >> 4);                        // nibble k: bits 68+4k.. entering
  const uint32_t de = (pe & 0x0f0f0f0fu) + 0x04040404u - (pl & 0x0f0f0f0fu);                 // 4 + d(2j)
  const uint32_t dd = ((pe >> 4) & 0x0f0f0f0fu) + 0x04040404u - ((pl >> 4) & 0x0f0f0f0fu);   // 4 + d(2j+1)
  const uint32_t sx = (de + dd) * 0x01010100u;   // byte j: sum_{i<j} (8 + d(2i) + d(2i+1))
  const uint32_t c0 = __popc(e2 >> 19) + __popc(e1) + __popc(e0 & 15u);
  const uint32_t x = sx + (c0 + (128 - MIN_HITS)) * 0x01010101u - 0x18100800u;   // 128 - 19 + c(2j)
  const uint32_t x2 = x + de - 0x04040404u;                                        // 128 - 19 + c(2j+1)
  edge = (x & 0x80u) | (x2 & 0x80000000u);
  return (x | x2) & 0x80808080u;
}

// Pass-1 mark of one word: screen_word's test, except that a word whose
// blocks 0 and 7 fail it and whose positions under checks 4..27 (the 69
// positions of bits 23..91 of e2:e1:e0) hold fewer than word_floor equal
// bases stays unmarked.  A passing check passes its block's test, so no run
// of passing checks crosses such a word's edges; every run inside it makes
// a segment within those 69 positions, and word_floor is the least run
// floor (run_hits_floor), so none of its segments could pass the
// probability screen.  Marked words still hold every check of every run
// that crosses a word edge, which the run tracking of phases AB and C
// relies on.
__device__ __forceinline__ uint32_t mark_word(uint32_t e2, uint32_t e1, uint32_t e0, int word_floor) {
  uint32_t edge;
  const uint32_t m = screen_word(e2, e1, e0, edge);
  const int h69 = __popc(e2 >> 23) + __popc(e1) + __popc(e0 & 0x0fffffffu);
  return (edge || (m && h69 >= word_floor)) ? 1u : 0u;
}

// Pass-1 mark with the floors on, without the full screen: a word is marked
// when block 0 or block 7 passes the block test (their spans are bits
// 19..67 and 47..95 of e2:e1:e0, the counts screen_word forms for them) or
// its 69 inner positions hold at least word_floor equal bases.  That marks
// every word mark_word marks and some more (words at the floor none of
// whose blocks passes), whose exact window bits in phase AB hold no passing
// check; it costs about half of screen_word's instructions.  With the
// floors off (word_floor 0) it would mark every word: mark_word then.
__device__ __forceinline__ uint32_t mark_word_floor(uint32_t e2, uint32_t e1, uint32_t e0, int word_floor) {
  const int p1 = __popc(e1);
  const int h69 = __popc(e2 >> 23) + p1 + __popc(e0 & 0x0fffffffu);
  const int c0 = __popc(e2 >> 19) + p1 + __popc(e0 & 15u);
  const int c7 = __popc(e1 >> 15) + __popc(e0);
  return (max(c0, c7) >= MIN_HITS || h69 >= word_floor) ? 1u : 0u;
}

// Exact window bits of one word: bit u set when check u's window holds
// >= MIN_HITS equal bases.  Four byte lanes (checks 8j + s) step s = 0..7
// together: count(u+1) = count(u) + bit u+65 - bit u+19 of e2:e1:e0.  Each
// lane holds its count plus 128 - MIN_HITS, so bit 7 is the test; biased
// counts stay within 109..155, so no lane borrows from or carries into the
// next, and bit 7 of lane j moves to bit 8j + s with one shift and a mask.
__device__ __forceinline__ uint32_t exact_word(uint32_t e2, uint32_t e1, uint32_t e0) {
  const uint64_t U = ((uint64_t)e1 << 32) | e2;
  uint32_t w = ((uint32_t)(__popcll(U >> 19) + __popc(e0 & 1u)) |
                (uint32_t)(__popcll(U >> 27) + __popc(e0 & 0x1ffu)) << 8 |
                (uint32_t)(__popcll(U >> 35) + __popc(e0 & 0x1ffffu)) << 16 |
                (uint32_t)(__popcll(U >> 43) + __popc(e0 & 0x1ffffffu)) << 24) +
               (128 - MIN_HITS) * 0x01010101u;
  const uint32_t lv = __funnelshift_r(e2, e1, 19);   // bit 8j+s: leaves after check 8j+s
  const uint32_t en = e0 >> 1;                       // bit 8j+s: enters at check 8j+s+1
  uint32_t g = 0;
#pragma unroll
  for (int s = 0; s < 8; s++) {
    if (s) w = w + ((en >> (s - 1)) & 0x01010101u) - ((lv >> (s - 1)) & 0x01010101u);
    g |= (w >> (7 - s)) & (0x01010101u << s);
  }
  return g;
}

// A segment that passed the FP32 probability screen, waiting for the FP64
// tail (GetMatchProbabilityEx and the record write).
struct Surv {
  int key, pos, s0, len, hits, gT, gQ;
};
static_assert(sizeof(Surv) == 28, "ScanGeom::SVB");

template <int LOG2L>
__global__ void __launch_bounds__(NT_SCAN, SCAN_CTAS_PER_SM) scan_kernel(const ScanParams P) {
  using Gm = ScanGeom<LOG2L>;
  constexpr int L = Gm::L, N = Gm::N, TW = Gm::TW, TWP = Gm::TWP, QPAD = Gm::QPAD, QWP = Gm::QWP;
  constexpr int ICAP = Gm::ICAP, QCAP = Gm::QCAP, NWARP = NT_SCAN / 32;
  constexpr unsigned FULL = 0xffffffffu;
  extern __shared__ __align__(16) unsigned char smem[];
  uint8_t* st = smem;
  uint8_t* sq = st + N;
  uint32_t* queue = reinterpret_cast<uint32_t*>(smem);   // bitplane path only: item | bit << 12
  Surv* surv = reinterpret_cast<Surv*>(smem + (size_t)Gm::QCAP * 4);   // bitplane path only
  uint2* tb = reinterpret_cast<uint2*>(smem + Gm::region);   // target planes (zero padded)
  uint2* qb = tb + TWP;                                       // query planes, QPAD zero words first
  int* tgp = reinterpret_cast<int*>(qb + QWP);
  int* qgp = tgp + (TW + 1);
  int* offs = qgp + (TW + 1);
  uint32_t* wmask = reinterpret_cast<uint32_t*>(offs + OFF_CHUNK);    // [MW][NT_SCAN] pass-1 marked words
  uint32_t* items = wmask + Gm::MW * NT_SCAN;                         // [ICAP] diag | word << 7
  uint32_t* gbits = items + ICAP;                                     // [ICAP] passing checks of the word
  int* dpos = reinterpret_cast<int*>(gbits + ICAP);                   // [NT_SCAN] offsets of the round
  uint16_t* order = reinterpret_cast<uint16_t*>(dpos + NT_SCAN);
  __shared__ int s_hist[64];
  __shared__ int s_wsum[NWARP];
  __shared__ int s_next, s_res, s_qn, s_nsv;
  __shared__ int s_cy_start[2];
  __shared__ uint32_t s_floor[8];   // P.run_floor

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int pidx = P.first + blockIdx.x;
  const int strand = blockIdx.y;
  const int slot = pidx * 2 + strand;
  // Small batches split each strand over gridDim.z CTAs: CTA z takes the
  // rounds (and byte-table groups) z, z + split, ...; results then take their
  // slot from the strand's counter in global memory, zeroed by the launcher.
  const int split = gridDim.z, zi = blockIdx.z;
  const PairDesc D = P.pairs[pidx];
  const uint32_t pflags = P.pair_flags[pidx];
  const int cnt = P.off_cnt[slot];
  if ((pflags & PF_INVALID) || cnt <= 0) {
    if (tid == 0 && split == 1) P.res_cnt[slot] = 0;
    return;
  }
  const int T = D.tlen, Q = D.qlen;
  const bool generic = (pflags & PF_GENERIC) != 0;
  const uint8_t* __restrict__ gt = P.pool + D.t_off;
  const uint8_t* __restrict__ gq = P.pool + D.q_off;

  if (tid == 0) {
    s_res = 0;
    s_qn = 0;
    s_nsv = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s_floor[k] = P.run_floor[k];
  }
  if (generic) {
    // chunk bytes; strand 1 reverse-complements the query (DNAVector.cc:482-500)
    for (int i = tid; i < N; i += NT_SCAN) {
      st[i] = i < T ? gt[i] : 0;
      unsigned c = 0;
      if (i < Q) {
        const unsigned raw = strand ? gq[Q - 1 - i] : gq[i];
        c = strand ? c_rc[raw] : raw;
      }
      sq[i] = (uint8_t)c;
    }
  } else {
    // 2-bit codes as two bitplanes straight from the pool, bit u of word w =
    // position 32w+u.  The pair is all A/C/G/T, whose complement flips both
    // code bits.  Strand 1 builds the query's forward planes in the (here
    // unused) byte region first and reads them backwards.
    if (tid < QPAD) qb[tid] = make_uint2(0u, 0u);
    build_planes(gt, T, tb, TWP, tid);
    if (!strand) {
      build_planes(gq, Q, qb + QPAD, QWP - QPAD, tid);
    } else {
      uint2* f = reinterpret_cast<uint2*>(smem);
      build_planes(gq, Q, f, TW + 2, tid);
      __syncthreads();
      // word w of the reverse complement: forward positions Q-32-32w ..
      // Q-1-32w, bit-reversed and complemented; positions past Q are zero
      for (int w = tid; w < QWP - QPAD; w += NT_SCAN) {
        const int lim = Q - 32 * w;   // valid bits of the word
        uint32_t r0 = 0u, r1 = 0u;
        if (lim > 0) {
          const int s0 = lim - 32;  // forward start, > -32
          uint32_t g0, g1;
          if (s0 >= 0) {
            const int fw = s0 >> 5, sh = s0 & 31;
            const uint2 a = f[fw], b2 = f[fw + 1];
            g0 = __funnelshift_r(a.x, b2.x, sh);
            g1 = __funnelshift_r(a.y, b2.y, sh);
          } else {
            g0 = f[0].x << -s0;
            g1 = f[0].y << -s0;
          }
          const uint32_t m = lowmask(lim);
          r0 = ~__brev(g0) & m;
          r1 = ~__brev(g1) & m;
        }
        qb[QPAD + w] = make_uint2(r0, r1);
      }
    }
    __syncthreads();
    if (warp == 0) gc_prefix(tb, tgp, TW, lane);
    if (warp == 1) gc_prefix(qb + QPAD, qgp, TW, lane);
  }
  __syncthreads();

  const int* __restrict__ olist = P.off_list + D.off_base + (size_t)strand * L;

  // Equality bits of target positions [32w, 32w+32) on diagonal pos.
  auto eword = [&](int pos, int w) -> uint32_t {
    if (w < 0) return 0u;
    const int qo = 32 * w + pos + 32 * QPAD;
    const int qw = qo >> 5, sh = qo & 31;
    const uint2 a = qb[qw], b = qb[qw + 1], t = tb[w];
    const uint32_t q0 = __funnelshift_r(a.x, b.x, sh);
    const uint32_t q1 = __funnelshift_r(a.y, b.y, sh);
    return ~((t.x ^ q0) | (t.y ^ q1));
  };
  // Equal bases of segment [s0, s1) on diagonal pos.  (A version streaming
  // one query word per target word measured 17% slower over the whole scan.)
  auto seg_hits = [&](int pos, int s0, int s1) -> int {
    int h = 0;
    const int wa = s0 >> 5, wb = (s1 - 1) >> 5;
    for (int w = wa; w <= wb; w++) {
      uint32_t m = 0xffffffffu;
      if (w == wa) m &= ~lowmask(s0 & 31);
      if (w == wb) m &= lowmask(((s1 - 1) & 31) + 1);
      h += __popc(eword(pos, w) & m);
    }
    return h;
  };
  // eword(pos, w - 2), eword(pos, w - 1), eword(pos, w) for w >= 1, sharing
  // the four query words they read.
  auto ewords3 = [&](int pos, int w, uint32_t& e2, uint32_t& e1, uint32_t& e0) {
    const int qo = 32 * (w - 2) + pos + 32 * QPAD;
    const int qw = qo >> 5, sh = qo & 31;
    const uint2 q0 = qb[qw], q1 = qb[qw + 1], q2 = qb[qw + 2], q3 = qb[qw + 3];
    const uint2 t1 = tb[w - 1], t0 = tb[w];
    if (w >= 2) {
      const uint2 t2 = tb[w - 2];
      e2 = ~((t2.x ^ __funnelshift_r(q0.x, q1.x, sh)) | (t2.y ^ __funnelshift_r(q0.y, q1.y, sh)));
    } else {
      e2 = 0u;
    }
    e1 = ~((t1.x ^ __funnelshift_r(q1.x, q2.x, sh)) | (t1.y ^ __funnelshift_r(q1.y, q2.y, sh)));
    e0 = ~((t0.x ^ __funnelshift_r(q2.x, q3.x, sh)) | (t0.y ^ __funnelshift_r(q2.y, q3.y, sh)));
  };

  // GetMatchProbabilityEx (AlignProbability.cc:107-125) in FP64, no FMA, or
  // the ProbTable lookup, and the record of a segment that passes.
  auto score = [&](int key, int pos, int s0, int len, double matches, double gcT, double gcQ) {
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
    const int k = split == 1 ? atomicAdd(&s_res, 1) : atomicAdd(&P.res_cnt[slot], 1);
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

  // One DoOne segment [s0, s1) on offset pos (CrossCorr.cc:693,713) through
  // FilterMatches (HomologyByXCorrSlave.cc:171-212).  hits: exact equal-base
  // count for A/C/G/T pairs (ignored on the generic path).  A/C/G/T segments
  // that pass the FP32 screen wait in the survivor buffer, scored after phase
  // C by one thread each (the FP64 pipe's cost is per warp instruction,
  // whatever the active lanes); a full buffer scores in place.
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
    if (!generic) {
      const int gT = gc_count(tb, tgp, s0, s1);
      const int gQ = gc_count(qb + QPAD, qgp, s0 + pos, s1 + pos);
      if (!P.ptable) {
        // FP32 screen on the z-score (pm*N - hits) / sd: reject only past a
        // threshold set on the host with a margin far beyond FP32 error;
        // anything else goes to the exact test.  With A = gQ gT + (N-gQ)(N-gT),
        // pm N = A / 2N and sd^2 = A (2N^2 - A) / 4N^3, so the test is
        // D = A - 2N hits > z sqrt(A (2N^2 - A) / N), squared without
        // divisions (A = 0: sd = 0, left to the exact test).
        const int A = gQ * gT + (len - gQ) * (len - gT);
        if (A > 0) {
          const float D = (float)(A - 2 * len * hits);
          const float Lf = D * D * (float)len;
          const float R = P.screen_z * P.screen_z * (float)A * (float)(2 * len * len - A);
          if (P.screen_z >= 0.f ? (D > 0.f && Lf > R) : (D >= 0.f || Lf < R)) return;
        }
      }
      const int v = atomicAdd(&s_nsv, 1);
      if (v < Gm::SVCAP) {
        surv[v] = Surv{key, pos, s0, len, hits, gT, gQ};
      } else {
        score(key, pos, s0, len, (double)hits, (double)gT, (double)gQ);
      }
      return;
    }
    // GetMatchProbabilityEx's sums, in its order (AlignProbability.cc:79-95).
    double matches = 0.0, gcT = 0.0, gcQ = 0.0;
    for (int i = 0; i < len; i++) {
      const int a = st[s0 + i], b = sq[s0 + pos + i];
      matches = __dadd_rn(matches, __ldg(&P.eq[a * 128 + b]));
      gcT = __dadd_rn(gcT, __ldg(&P.gcw[a]));
      gcQ = __dadd_rn(gcQ, __ldg(&P.gcw[b]));
    }
    score(key, pos, s0, len, matches, gcT, gcQ);
  };

  int rbase = 0, gbase = 0;   // rounds and byte-table groups of the earlier chunks
  for (int c0 = 0; c0 < cnt; c0 += OFF_CHUNK) {
    const int nc = min(OFF_CHUNK, cnt - c0);
    if (tid < 64) s_hist[tid] = 0;
    __syncthreads();
    // Longest diagonals first: the threads of a round and the lanes of a warp
    // get diagonals of similar length.
    for (int k = tid; k < nc; k += NT_SCAN) {
      const int o = olist[c0 + k];
      offs[k] = o;
      const int b = 63 - (int)(((long long)diag_len(o - N, T, Q) * 64) / N);
      atomicAdd(&s_hist[b], 1);
    }
    __syncthreads();
    if (warp == 0) {
      const int v0 = s_hist[lane], v1 = s_hist[lane + 32];
      const int i0 = warp_incl_sum(v0, lane);
      const int tot0 = __shfl_sync(FULL, i0, 31);
      const int i1 = warp_incl_sum(v1, lane);
      s_hist[lane] = i0 - v0;
      s_hist[lane + 32] = tot0 + i1 - v1;
    }
    __syncthreads();
    // Stable placement, in offset-index order within a length bucket: when a
    // strand is split over several CTAs each builds this order itself, and
    // they must agree on it (an atomic placement order may differ between
    // CTAs, so a diagonal could fall to two CTAs' rounds or to none).  Groups
    // of NT_SCAN indices in order; within a group, warp by warp; within a
    // warp, lanes with the same bucket ranked by lane.
    for (int kb = 0; kb < nc; kb += NT_SCAN) {
      const int k = kb + tid;
      const bool have = k < nc;
      const int b = have ? 63 - (int)(((long long)diag_len(offs[k] - N, T, Q) * 64) / N) : -1;
      const unsigned peers = __match_any_sync(FULL, b);
      const unsigned below = peers & ((1u << lane) - 1u);
      const bool leader = (32 - __clz((int)peers)) - 1 == lane;   // highest lane of the peers
#pragma unroll
      for (int w = 0; w < NWARP; w++) {
        int p = 0;
        if (warp == w && have) {
          p = s_hist[b] + __popc(below);
          order[p] = (uint16_t)k;
        }
        __syncwarp();
        if (warp == w && have && leader) s_hist[b] += __popc(peers);
        __syncthreads();
      }
    }
    if (tid == 0) s_next = 0;
    __syncthreads();

    if (generic) {
      // A warp takes 32 consecutive (similar-length) diagonals at a time.
      const int gfirst = ((zi - gbase) % split + split) % split;   // first group of this CTA
      for (;;) {
        int k0 = 0;
        if (lane == 0) k0 = 32 * (gfirst + split * atomicAdd(&s_next, 1));
        k0 = __shfl_sync(FULL, k0, 0);
        if (k0 >= nc) break;
        if (k0 + lane < nc) {
          const int li = order[k0 + lane];
          const int pos = offs[li] - N;
          const int key = c0 + li;
          const int i0 = max(0, -pos);
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
        }
        __syncwarp();
      }
      gbase += (nc + 31) / 32;
      __syncthreads();
      continue;
    }

    // A/C/G/T: window sums are 100 x equal-base counts, so a window passes
    // when it holds >= 19 equal bases.  Check positions c run from i0+46 to
    // iend-1; window(c) = [c-45, c]; a segment is a maximal run of passing
    // checks [a..b], emitted as [a-45, b+1) (or [a-45, iend) at the end).
    const int rfirst = ((zi - rbase) % split + split) % split;   // first round of this CTA
    rbase += (nc + NT_SCAN - 1) / NT_SCAN;
    for (int r0 = NT_SCAN * rfirst; r0 < nc; r0 += NT_SCAN * split) {
      const int k = r0 + tid;
      const bool have = k < nc;
      const int pos = have ? offs[order[k]] - N : 0;
      dpos[tid] = pos;
      const int i0 = max(0, -pos);
      const int iend = min(T - 1, Q - pos);
      const int cfirst = i0 + 46, clast = iend - 1;
      const bool valid = have && clast >= cfirst;
      const int wfirst = cfirst >> 5, wlast = clast >> 5;

      // ---- pass 1 (thread = diagonal): one bit per word, 32 words per entry
      //      of wmask[q >> 5][tid]; no check of an unmarked word can pass.
      int nb = 0;
      if (valid) {
        // The query word pair of target word w is (w + qd, w + qd + 1) at bit
        // shift sh: one new query word per step.
        const int qd = (pos + 32 * QPAD) >> 5, sh = (pos + 32 * QPAD) & 31;
        const bool floor_on = P.word_floor > 0;   // off: every screened word is marked (mark_word)
        uint32_t e2 = eword(pos, wfirst - 2), e1 = eword(pos, wfirst - 1);
        const uint2* qp = qb + wfirst + qd;
        const uint2* tp = tb + wfirst;
        uint2 a = qp[0];
        const int nw = wlast - wfirst + 1;
        for (int q0 = 0; q0 < nw; q0 += 32) {
          const int m = min(32, nw - q0);
          uint32_t acc = 0;
#pragma unroll 4
          for (int q = 0; q < m; q++) {
            const uint2 nx = qp[q0 + q + 1], tw = tp[q0 + q];
            const uint32_t e0 = ~((tw.x ^ __funnelshift_r(a.x, nx.x, sh)) | (tw.y ^ __funnelshift_r(a.y, nx.y, sh)));
            a = nx;
            const uint32_t mk = floor_on ? mark_word_floor(e2, e1, e0, P.word_floor) : mark_word(e2, e1, e0, 0);
            acc = __funnelshift_r(acc, mk, 1);   // in at bit 31
            e2 = e1;
            e1 = e0;
          }
          acc >>= 32 - m;   // bit q: word q0 + q
          wmask[(q0 >> 5) * NT_SCAN + tid] = acc;
          nb += __popc(acc);
        }
      }
      // item index of this diagonal's first marked word: CTA exclusive scan
      const int nincl = warp_incl_sum(nb, lane);
      if (lane == 31) s_wsum[warp] = nincl;
      if (tid == 0) s_cy_start[1] = -1;   // no run open into the first sub-range
      __syncthreads();
      int ibase = nincl - nb, total = 0;
#pragma unroll
      for (int x = 0; x < NWARP; x++) {
        const int v = s_wsum[x];
        ibase += x < warp ? v : 0;
        total += v;
      }

      // ---- pass 2 over sub-ranges of at most ICAP items (one per marked
      //      word).  A sub-range may split a diagonal: its last item (word,
      //      bits, open-run start) is carried into the next one.
      int par = 0;
      for (int g0 = 0; g0 < total; g0 += ICAP, par ^= 1) {
        const int n = min(ICAP, total - g0);
        const int g1 = g0 + n;
        if (nb && ibase < g1 && ibase + nb > g0) {
          int kk = ibase;
          const int nq = (wlast - wfirst + 32) >> 5;
          for (int q32 = 0; q32 < nq && kk < g1; q32++) {
            uint32_t ent = wmask[q32 * NT_SCAN + tid];
            const int c = __popc(ent);
            if (kk + c <= g0) {
              kk += c;
              continue;
            }
            while (ent && kk < g1) {
              const int bi = __ffs(ent) - 1;
              ent &= ent - 1;
              if (kk >= g0) items[kk - g0] = (uint32_t)tid | ((uint32_t)(32 * q32 + bi) << 7);
              kk++;
            }
          }
        }
        __syncthreads();

        // ---- phase AB (thread = item): the word's exact window bits, the bit
        //      of the check before it, and the falls and closing ends of its
        //      runs, queued as (item, bit) descriptors.  The check before the
        //      word (bit 31 of the previous word) is tested from the same
        //      equality words: its window is bits 18..63 of e2:e1, and a
        //      passing check lies in a marked word, so a run crossing into the
        //      word always comes from the item before it (or the carry). ----
        constexpr uint32_t IT_PREV = 1u << 31;    // items[i]: the check before the word passes
        constexpr uint32_t IT_DEFER = 1u << 30;   // items[i]: its segments did not fit the queue
        constexpr uint32_t NO_SEG = 0xffffffffu;  // queue slot of a deferred item
        const int cy = par ^ 1;   // carry slot written by the previous sub-range
        // falls and closing end of item i (word bits g, previous-check bit pb)
        auto runs_of = [&](uint32_t it, uint32_t g, uint32_t pb, uint32_t& fall, bool& close) {
          const int d = (int)(it & 127u), wr = (int)((it >> 7) & 1023u);
          const int p = dpos[d];
          const int cf = max(0, -p) + 46, cl = min(T - 1, Q - p) - 1;
          const int cw = 32 * ((cf >> 5) + wr);
          const int lo = max(cf - cw, 0), hi = min(cl - cw, 31);
          const uint32_t vm = (0xffffffffu >> (31 - hi)) & (0xffffffffu << lo);
          fall = ~g & ((g << 1) | pb) & vm;
          // a run still open at the word's last valid check ends at the
          // diagonal's end or at the first check of an unmarked next word
          close = ((g >> hi) & 1u) &&
                  (cw + hi == cl || !((wmask[((wr + 1) >> 5) * NT_SCAN + d] >> ((wr + 1) & 31)) & 1u));
        };
        // check position where the run holding bit u-1 of item i began
        auto run_start = [&](int i, uint32_t g, int u) -> int {
          uint32_t rb = g & ~((g << 1) | (items[i] >> 31)) & lowmask(u);
          while (!rb) {
            if (--i < 0) return s_cy_start[cy];
            g = gbits[i];
            rb = g & ~((g << 1) | (items[i] >> 31));
          }
          const uint32_t it = items[i];
          const int d = (int)(it & 127u), wr = (int)((it >> 7) & 1023u);
          return 32 * (((max(0, -dpos[d]) + 46) >> 5) + wr) + (31 - __clz((int)rb));
        };
        // segment ending at bit u (0..31: a fall; 32: the closing end) of item i
        auto segment = [&](int i, int u) {
          const uint32_t it = items[i];
          const int d = (int)(it & 127u), wr = (int)((it >> 7) & 1023u);
          const uint32_t g = gbits[i];
          const int p = dpos[d];
          const int cf = max(0, -p) + 46, ie = min(T - 1, Q - p), cl = ie - 1;
          const int cw = 32 * ((cf >> 5) + wr);
          int s1 = cw + u, ub = u;
          if (u == 32) {
            const int hi = min(cl - cw, 31);
            s1 = cw + hi == cl ? ie : cw + 32;
            ub = hi + 1;
          }
          const int s0 = run_start(i, g, ub) - 45;
          if (s0 < 1 || s1 <= s0) {   // cannot happen: a run start precedes its end
            atomicOr(P.err, 4);
            return;
          }
          emit(c0 + order[r0 + d], p, s0, s1, seg_hits(p, s0, s1));
        };
        for (int ib = 0; ib < n; ib += NT_SCAN) {
          const int i = ib + tid;
          uint32_t fall = 0;
          bool close = false;
          if (i < n) {
            const uint32_t it = items[i];
            const int d = (int)(it & 127u), wr = (int)((it >> 7) & 1023u);
            const int p = dpos[d];
            const int cf = max(0, -p) + 46, cl = min(T - 1, Q - p) - 1;
            const int w = (cf >> 5) + wr;
            uint32_t e2, e1, e0;
            ewords3(p, w, e2, e1, e0);
            const int lo = max(cf - 32 * w, 0), hi = min(cl - 32 * w, 31);
            const uint32_t g = exact_word(e2, e1, e0) & (0xffffffffu >> (31 - hi)) & (0xffffffffu << lo);
            const uint32_t pb =
                (32 * w - 1 >= cf && __popcll((((uint64_t)e1 << 32) | e2) >> 18) >= MIN_HITS) ? 1u : 0u;
            gbits[i] = g;
            items[i] = it | (pb ? IT_PREV : 0u);
            runs_of(it, g, pb, fall, close);
            // A run that starts and ends inside this word (checks a..b, r of
            // them) makes the segment [a-45, b+1) of length r + 45, positions
            // that bits a+19..b+64 of e2:e1:e0 cover, so its equal-base count
            // is one popcount here.  Below the floor for r no G+C composition
            // lets it pass the probability screen, so the segment is dropped
            // here instead of queued.
            if (fall | close) {
              const uint32_t rise = g & ~((g << 1) | pb);   // first checks of runs
              const uint64_t U = ((uint64_t)e1 << 32) | e2;
              const uint8_t* fl = reinterpret_cast<const uint8_t*>(s_floor);
              auto hopeless = [&](int b) -> bool {
                const uint32_t rs = rise & (0xffffffffu >> (31 - b));
                if (!rs) return false;   // the run began in an earlier word
                const int a = 31 - __clz((int)rs);
                const int h = __popcll(U >> (a + 19)) + __popc(e0 & (0xffffffffu >> (31 - b)));
                return h < (int)fl[b - a];
              };
              uint32_t f = fall & ~1u;   // bit 0: the run ended in the word before
              while (f) {
                const int u = __ffs(f) - 1;
                f &= f - 1;
                if (hopeless(u - 1)) fall &= ~(1u << u);
              }
              if (close && hopeless(hi)) close = false;
            }
          }
          const int nseg = __popc(fall) + (close ? 1 : 0);
          const int sincl = warp_incl_sum(nseg, lane);
          int q = 0;
          if (lane == 31 && sincl) q = atomicAdd(&s_qn, sincl);
          q = __shfl_sync(FULL, q, 31) + sincl - nseg;
          if (nseg && q + nseg > QCAP) {
            // does not fit: the item's segments run in place after the barrier
            for (int x = q; x < min(q + nseg, QCAP); x++) queue[x] = NO_SEG;
            items[i] |= IT_DEFER;
          } else {
            while (fall) {
              const int u = __ffs(fall) - 1;
              fall &= fall - 1;
              queue[q++] = (uint32_t)i | ((uint32_t)u << 12);
            }
            if (close) queue[q] = (uint32_t)i | (32u << 12);
          }
        }
        __syncthreads();

        // ---- the run open at the sub-range's end, carried into the next ----
        if (tid == 0) {
          const uint32_t g = gbits[n - 1];
          s_cy_start[par] = (g >> 31) ? run_start(n - 1, g, 32) : -1;
        }

        // ---- phase C (thread = segment): run start, equal-base count,
        //      FilterMatches; then the deferred items in place. ----
        const int qn = min(s_qn, QCAP);
        for (int e = tid; e < qn; e += NT_SCAN) {
          const uint32_t sg = queue[e];
          if (sg != NO_SEG) segment((int)(sg & 4095u), (int)(sg >> 12));
        }
        if (s_qn > QCAP) {
          for (int i = tid; i < n; i += NT_SCAN) {
            const uint32_t it = items[i];
            if (!(it & IT_DEFER)) continue;
            uint32_t fall;
            bool close;
            runs_of(it, gbits[i], it >> 31, fall, close);
            while (fall) {
              const int u = __ffs(fall) - 1;
              fall &= fall - 1;
              segment(i, u);
            }
            if (close) segment(i, 32);
          }
        }
        __syncthreads();
        // ---- the FP64 tail of the screen's survivors, one thread each ----
        const int nsv = min(s_nsv, Gm::SVCAP);
        for (int k = tid; k < nsv; k += NT_SCAN) {
          const Surv v = surv[k];
          score(v.key, v.pos, v.s0, v.len, (double)v.hits, (double)v.gT, (double)v.gQ);
        }
        __syncthreads();
        if (tid == 0) {
          s_qn = 0;
          s_nsv = 0;
        }
      }
      __syncthreads();
    }
  }
  if (tid == 0 && split == 1) P.res_cnt[slot] = s_res;
}

// ---------------------------------------------------------------------------
// Finalize: dense, ordered results
// ---------------------------------------------------------------------------
// dense_base[i] = sum_{j<i} min(cnt[j], slots); dense_base[n] = total.  One
// CTA: each thread sums a run of ceil(n/1024) consecutive slots, one block
// scan of the run sums, then each thread writes its run's bases.
__global__ void __launch_bounds__(1024) count_scan_kernel(const int* __restrict__ cnt, int n, int slots,
                                                          int* __restrict__ base) {
  __shared__ int s_w[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int per = (n + 1023) / 1024;
  const int lo = min(tid * per, n), hi = min(lo + per, n);
  int sum = 0;
  for (int i = lo; i < hi; i++) sum += min(cnt[i], slots);
  int incl = sum;
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
  int run = s_w[warp] + incl - sum;
  for (int i = lo; i < hi; i++) {
    base[i] = run;
    run += min(cnt[i], slots);
  }
  if (tid == 1023) base[n] = run;   // the last thread's run ends at the total
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
static cudaError_t set_scan_attrs() {
  cudaError_t e = cudaFuncSetAttribute(scan_kernel<LOG2L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)scan_smem_bytes(LOG2L));
  if (e != cudaSuccess) return e;
  // several CTAs per SM: ask for the largest shared-memory carveout
  return cudaFuncSetAttribute(scan_kernel<LOG2L>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

cudaError_t prepare_scan_kernels() {
  cudaError_t e;
  if ((e = set_scan_attrs<10>()) != cudaSuccess) return e;
  if ((e = set_scan_attrs<11>()) != cudaSuccess) return e;
  if ((e = set_scan_attrs<12>()) != cudaSuccess) return e;
  if ((e = set_scan_attrs<13>()) != cudaSuccess) return e;
  if ((e = set_scan_attrs<14>()) != cudaSuccess) return e;
  return set_scan_attrs<15>();
}

cudaError_t launch_scan(int log2L, const ScanParams& p, int npairs, cudaStream_t s) {
  if (npairs <= 0) return cudaSuccess;
  // Fewer strands than a wave of CTAs: split them, up to 4 ways.
  static const int sms = [] {
    int dev = 0, n = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
  }();
  int split = 1;
  while (split < 4 && 2 * npairs * split * 2 <= SCAN_CTAS_PER_SM * sms) split *= 2;
  if (split > 1) {
    const cudaError_t e = cudaMemsetAsync(p.res_cnt + 2 * (size_t)p.first, 0, 2 * (size_t)npairs * sizeof(int), s);
    if (e != cudaSuccess) return e;
  }
  const dim3 grid(npairs, 2, split);
  const size_t sm = scan_smem_bytes(log2L);
  switch (log2L) {
    case 10: scan_kernel<10><<<grid, NT_SCAN, sm, s>>>(p); break;
    case 11: scan_kernel<11><<<grid, NT_SCAN, sm, s>>>(p); break;
    case 12: scan_kernel<12><<<grid, NT_SCAN, sm, s>>>(p); break;
    case 13: scan_kernel<13><<<grid, NT_SCAN, sm, s>>>(p); break;
    case 14: scan_kernel<14><<<grid, NT_SCAN, sm, s>>>(p); break;
    case 15: scan_kernel<15><<<grid, NT_SCAN, sm, s>>>(p); break;
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

cudaError_t upload_scan_constants(const unsigned char* rc256, const uchar4* w4q128, const double* w4d) {
  return upload_constants_here(rc256, w4q128, w4d);
}

}  // namespace xc
