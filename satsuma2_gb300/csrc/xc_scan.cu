// Scan and finalize kernels of the satsuma2 cross-correlation path (sm_103a).
//
//   scan_kernel<log2 L>  one CTA per (chunk pair, strand): DoOne's ungapped
//                        46-wide window scan of every FindTop offset on 2-bit
//                        bitplanes (32 positions per word op, 8-position window
//                        screening), then FilterMatches on the raw segments: an
//                        FP32 screen of the match probability and the exact FP64
//                        GetMatchProbability / PrintMatch tail for survivors.
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
  // Raw-segment queue of the bitplane path (8 bytes per segment).  It reuses
  // the byte arrays, which that path no longer reads once the planes exist.
  static constexpr int QCAP = 2048;
  static constexpr size_t region = (size_t)QCAP * 8 > 2 * (size_t)N ? (size_t)QCAP * 8 : 2 * (size_t)N;
  static constexpr int FW = (TW + 7) / 8;   // 32-bit flag entries per thread (4 bits per word)
  static constexpr size_t bytes =
      (size_t)(2 * TWP + (TW + 1) + 2 * QWP + (TW + 1) + OFF_CHUNK + FW * NT_SCAN) * 4 + OFF_CHUNK * 2 + region;
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
  uint32_t* bflags = reinterpret_cast<uint32_t*>(offs + OFF_CHUNK);   // [FW][NT_SCAN] block masks of pass 1
  uint16_t* order = reinterpret_cast<uint16_t*>(bflags + Gm::FW * NT_SCAN);
  uint8_t* st = reinterpret_cast<uint8_t*>(order + OFF_CHUNK);
  uint8_t* sq = st + N;
  uint2* queue = reinterpret_cast<uint2*>(st);   // bitplane path only, after the planes are built
  constexpr int QCAP = Gm::QCAP;
  __shared__ int s_hist[64];
  __shared__ int s_next;
  __shared__ int s_res;
  __shared__ int s_qn;

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
  if (tid == 0) {
    s_res = 0;
    s_qn = 0;
  }
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
    // Bitplane path: queue a raw segment (chunk-local offset index, start,
    // length, equal-base count) for the converged drain below; handle it in
    // place only when the queue is full.
    auto push = [&](int key, int pos, int s0, int s1, int hits) {
      const int qi = atomicAdd(&s_qn, 1);
      if (qi < QCAP)
        queue[qi] = make_uint2((uint32_t)(key - c0) | ((uint32_t)s0 << 16),
                               (uint32_t)(s1 - s0) | ((uint32_t)hits << 16));
      else
        emit(key, pos, s0, s1, hits);
    };
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

    // A warp takes 32 consecutive (similar-length) diagonals at a time and
    // finishes them together, so its lanes stay converged.
    auto process = [&](int k) {
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
        return;
      }
      // A/C/G/T: window sums are 100 x equal-base counts, so a window passes
      // when it holds >= 19 equal bases.  Check positions c run from i0+46 to
      // iend-1; window(c) = [c-45, c]; a segment is a maximal run of passing
      // checks [a..b], emitted as [a-45, b+1) (or [a-45, iend) at the end).
      const int cfirst = i0 + 46, clast = iend - 1;
      if (clast < cfirst) return;
      const int wfirst = cfirst >> 5, wlast = clast >> 5;
      auto eword = [&](int w) -> uint32_t {
        if (w < 0) return 0u;
        const int qo = 32 * w + pos + 32 * QPAD;
        const int qw = qo >> 5, sh = qo & 31;
        const uint32_t q0 = __funnelshift_r(qb0[qw], qb0[qw + 1], sh);
        const uint32_t q1 = __funnelshift_r(qb1[qw], qb1[qw + 1], sh);
        return ~((tb0[w] ^ q0) | (tb1[w] ^ q1));
      };
      // Valid check positions of word w as a bit mask.
      auto validmask = [&](int w) -> uint32_t {
        const int lo = max(cfirst - 32 * w, 0), hi = min(clast - 32 * w, 31);
        return (0xffffffffu >> (31 - hi)) & (0xffffffffu << lo);
      };
      // Pass 1, branch-free: per word a 4-bit mask of the 8-position blocks
      // whose 53-position span [c0-45, c0+8) holds >= 19 equal bases; no
      // window inside any other block can pass.  Masks go to shared memory,
      // eight words per 32-bit entry, entries interleaved across threads.
      {
        uint32_t e2 = eword(wfirst - 2), e1 = eword(wfirst - 1);
        uint32_t acc = 0;
        for (int w = wfirst; w <= wlast; w++) {
          const uint32_t e0 = eword(w);
          const uint64_t U = ((uint64_t)e1 << 32) | e2;
          const uint32_t vm = validmask(w);
          uint32_t f = 0;
#pragma unroll
          for (int sb = 0; sb < 4; sb++) {
            const int a = 8 * sb + 19;
            const int c53 = __popcll(U >> a) + __popc(e0 & lowmask(a - 11));
            f |= (uint32_t)((c53 >= MIN_HITS) && ((vm >> (8 * sb)) & 0xffu)) << sb;
          }
          const int q = w - wfirst;
          acc |= f << (4 * (q & 7));
          if ((q & 7) == 7 || w == wlast) {
            bflags[(q >> 3) * NT_SCAN + tid] = acc;
            acc = 0;
          }
          e2 = e1;
          e1 = e0;
        }
      }
      // Pass 2, sparse: exact windows only in flagged blocks, then runs of
      // passing checks.  A run is contiguous, so every word it covers is
      // flagged and visited in order; its equal-base count is the rising
      // window's count plus the bits after it.
      const int nq = wlast - wfirst + 1;
      bool open = false;
      int start = 0, runcnt = 0, accpos = 0, lastw = -4;
      uint32_t e2 = 0, e1 = 0, e0 = 0;
      // One flat loop over this lane's flagged words (a cursor skips empty
      // entries), so a warp runs max-over-lanes of the flagged-word count
      // rather than that maximum per 8-word entry.
      const int nq8 = (nq + 7) >> 3;
      int q8 = 0;
      uint32_t fw = bflags[tid];
      for (;;) {
        while (fw == 0 && ++q8 < nq8) fw = bflags[q8 * NT_SCAN + tid];
        if (fw == 0) break;
        {
          const int nib = (__ffs(fw) - 1) >> 2;
          const uint32_t f = (fw >> (4 * nib)) & 15u;
          fw &= ~(15u << (4 * nib));
          const int w = wfirst + q8 * 8 + nib;
          if (open && w != lastw + 1) {
            // the run ended at the first check of the unflagged word lastw+1
            push(key, pos, start, 32 * (lastw + 1), runcnt);
            open = false;
          }
          if (w == lastw + 1) {
            e2 = e1;
            e1 = e0;
            e0 = eword(w);
          } else if (w == lastw + 2) {
            e2 = e0;
            e1 = eword(w - 1);
            e0 = eword(w);
          } else {
            e2 = eword(w - 2);
            e1 = eword(w - 1);
            e0 = eword(w);
          }
          lastw = w;
          const uint64_t U = ((uint64_t)e1 << 32) | e2;
          const uint32_t vm = validmask(w);
          uint32_t g = 0;
#pragma unroll
          for (int sb = 0; sb < 4; sb++) {
            if (!((f >> sb) & 1u)) continue;
#pragma unroll
            for (int u = 8 * sb; u < 8 * sb + 8; u++) {
              const int wc = __popcll(U >> (u + 19)) + __popc(e0 & lowmask(u + 1));
              g |= (uint32_t)(wc >= MIN_HITS) << u;
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
              runcnt = __popcll(U >> (u + 19)) + __popc(e0 & lowmask(u + 1));   // window count at the rise
              accpos = u + 1;
              open = true;
            } else {
              runcnt += __popc(e0 & lowmask(u) & ~lowmask(accpos));
              push(key, pos, start, 32 * w + u, runcnt);
              open = false;
            }
          }
          if (open) {
            if (w == wlast) {
              const int ue = iend - 32 * w;   // 1..32
              push(key, pos, start, iend, runcnt + __popc(e0 & lowmask(ue) & ~lowmask(accpos)));
              open = false;
            } else {
              runcnt += __popc(e0 & ~lowmask(accpos));
              accpos = 0;
            }
          }
        }
      }
      if (open) push(key, pos, start, 32 * (lastw + 1), runcnt);
    };
    for (;;) {
      int k0 = 0;
      if (lane == 0) k0 = atomicAdd(&s_next, 32);
      k0 = __shfl_sync(0xffffffffu, k0, 0);
      if (k0 >= nc) break;
      if (k0 + lane < nc) process(k0 + lane);
      __syncwarp();
    }
    __syncthreads();
    // Drain the queued segments with every thread (converged warps).
    if (!generic) {
      const int qn = min(s_qn, QCAP);
      for (int e = tid; e < qn; e += NT_SCAN) {
        const uint2 g = queue[e];
        const int key = (int)(g.x & 0xffffu), s0 = (int)(g.x >> 16);
        const int len = (int)(g.y & 0xffffu), hits = (int)(g.y >> 16);
        emit(c0 + key, offs[key] - N, s0, s0 + len, hits);
      }
      __syncthreads();
      if (tid == 0) s_qn = 0;
      __syncthreads();
    }
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
static cudaError_t set_scan_attrs() {
  return cudaFuncSetAttribute(scan_kernel<LOG2L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)scan_smem_bytes(LOG2L));
}

cudaError_t prepare_scan_kernels() {
  cudaError_t e;
  if ((e = set_scan_attrs<10>()) != cudaSuccess) return e;
  if ((e = set_scan_attrs<11>()) != cudaSuccess) return e;
  if ((e = set_scan_attrs<12>()) != cudaSuccess) return e;
  if ((e = set_scan_attrs<13>()) != cudaSuccess) return e;
  return set_scan_attrs<14>();
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

cudaError_t upload_scan_constants(const unsigned char* rc256, const uchar4* w4q128, const double* w4d) {
  return upload_constants_here(rc256, w4q128, w4d);
}

}  // namespace xc
