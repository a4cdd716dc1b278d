// Test infrastructure only: a C-callable harness around the reference's own
// CPU implementation of the cross-correlation path (satsuma2 analysis/ and
// extern/RealFFT/), linked from the unmodified reference sources by
// oracle/build_ref.sh into oracle/_ref/libsatsuma_ref.so.  Only tests/, the
// golden-fixture generator, __graft_entry__.smoke() and bench.py's CPU
// baseline may load it; the product never does.
//
// The per-pair glue (Align + FilterMatches + RCQuery) lives inside the slave's
// main translation unit in the reference (analysis/HomologyByXCorrSlave.cc:
// 56-60, 168-253), so it cannot be linked; ref_align_pair() below restates those
// lines and calls the reference library for everything else.

// Standard headers first, so that the access override below only touches the
// reference's own classes.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>
#include <math.h>
#include <string.h>

// FindTop/DoOne are private members of SeqAnalyzer; the harness reaches them
// directly so that each stage can be pinned separately.
#define private public
#include "analysis/CrossCorr.h"
#include "analysis/AlignProbability.h"
#include "analysis/ProbTable.h"
#include "analysis/DNAVector.h"
#undef private

#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// Same field order and padding as t_result (analysis/WorkQueue.h:23-33).
struct RefResult {
  unsigned long query_id, target_id, query_size, qstart, tstart, len;
  bool reverse;
  double prob;
  double ident;
};
static_assert(sizeof(RefResult) == 72, "t_result layout");

DNAVector make_dna(const char* s, int n) {
  DNAVector d;
  d.resize(n);
  for (int i = 0; i < n; i++) d[i] = s[i];
  return d;
}

// HomologyByXCorrSlave.cc:56-60
int rc_query(int offset, int start, int len, int chunkSize, int qLen) {
  (void)len;
  return start + qLen - offset - chunkSize;
}

}  // namespace

extern "C" {

// CCSignal::SetSequence (CrossCorr.cc:179-206) at signal length L; out[c*L+k].
void ref_signal(const char* seq, int len, int L, float* out) {
  DNAVector d = make_dna(seq, len);
  CCSignal s;
  s.SetSequence(d, L);
  for (int c = 0; c < 4; c++) {
    const std::vector<float>& v = s.Get(c);
    memcpy(out + (size_t)c * L, v.data(), sizeof(float) * L);
  }
}

// DNAVector::ReverseComplement (DNAVector.cc:482-500).
void ref_rc(const char* seq, int len, char* out) {
  DNAVector d = make_dna(seq, len);
  d.ReverseComplement();
  for (int i = 0; i < len; i++) out[i] = d[i];
}

// CrossCorrelation::CrossCorrelate (CrossCorr.cc:386-403) of the signals of t and q.
void ref_xcorr(const char* t, int tlen, const char* q, int qlen, int L, float* out) {
  DNAVector dt = make_dna(t, tlen), dq = make_dna(q, qlen);
  CCSignal st, sq;
  st.SetSequence(dt, L);
  sq.SetSequence(dq, L);
  CrossCorrelation xc;
  std::vector<float> r;
  xc.CrossCorrelate(r, st, sq);
  memcpy(out, r.data(), sizeof(float) * L);
}

// SeqAnalyzer::FindTop (CrossCorr.cc:878-944).
int ref_findtop(const float* xc, int L, double cutoff, int* out, int cap) {
  SeqAnalyzer sa;
  std::vector<float> v(xc, xc + L);
  std::vector<int> top;
  sa.FindTop(top, v, cutoff);
  int n = (int)top.size();
  for (int i = 0; i < n && i < cap; i++) out[i] = top[i];
  return n;
}

// SeqAnalyzer::DoOne (CrossCorr.cc:667-724); segs[3*i] = tStart, qStart, len.
int ref_doone(const char* t, int tlen, const char* q, int qlen, int pos, int* segs, int cap) {
  DNAVector dt = make_dna(t, tlen), dq = make_dna(q, qlen);
  SeqAnalyzer sa;
  vecSeqMatch m;
  sa.DoOne(m, dq, dt, pos);
  int n = m.size();
  for (int i = 0; i < n && i < cap; i++) {
    segs[3 * i + 0] = m[i].GetStartTarget();
    segs[3 * i + 1] = m[i].GetStartQuery();
    segs[3 * i + 2] = m[i].GetLength();
  }
  return n;
}

// GetMatchProbabilityEx (AlignProbability.cc:62-126).
double ref_match_prob(const char* t, int tlen, const char* q, int qlen, int ts, int qs, int len,
                      double target_total, double* ident) {
  DNAVector dt = make_dna(t, tlen), dq = make_dna(q, qlen);
  double id = 0;
  double p = GetMatchProbabilityEx(id, dt, dq, ts, qs, len, target_total);
  if (ident) *ident = id;
  return p;
}

// PrintMatch(..., bSilent=true) (CrossCorr.cc:967-1037).
double ref_print_ident(const char* t, int tlen, const char* q, int qlen, int ts, int qs, int len) {
  DNAVector dt = make_dna(t, tlen), dq = make_dna(q, qlen);
  SeqMatch m(ts, qs, len, 0.);
  return PrintMatch(dq, dt, m, true);
}

// DNA_EqualAmb / DNA_Equal / codec weights (DNAVector.cc:13-58, 351-403).
double ref_equal_amb(int a, int b) { return DNA_EqualAmb((char)a, (char)b); }
double ref_equal(int a, int b) { return DNA_Equal((char)a, (char)b); }
void ref_codec(int l, double* w4) {
  w4[0] = DNA_A((char)l); w4[1] = DNA_C((char)l); w4[2] = DNA_G((char)l); w4[3] = DNA_T((char)l);
}

// ProbTable (ProbTable.cc:7-140).
void* ref_probtable_new(double target_size, double cutoff) { return new ProbTable(target_size, cutoff); }
void ref_probtable_free(void* p) { delete (ProbTable*)p; }
// Dumps m_table rows 1..511 (row 0 is never filled by Setup) as 512*2048 doubles.
void ref_probtable_dump(void* p, double* out) {
  ProbTable* pt = (ProbTable*)p;
  for (int i = 0; i < 512; i++)
    for (int j = 0; j < 2048; j++)
      out[(size_t)i * 2048 + j] = (i < (int)pt->m_table.size() && j < (int)pt->m_table[i].size())
                                       ? pt->m_table[i][j] : -1.0;
}
double ref_probtable_prob(void* p, const char* t, int tlen, const char* q, int qlen, int ts, int qs,
                          int len, double* ident) {
  DNAVector dt = make_dna(t, tlen), dq = make_dna(q, qlen);
  double id = 0;
  double r = ((ProbTable*)p)->GetMatchProbability(id, dt, dq, ts, qs, len);
  if (ident) *ident = id;
  return r;
}

// One chunk pair through HomologyByXCorr::Align + FilterMatches
// (HomologyByXCorrSlave.cc:168-253), both strands.  Signals are built exactly
// as create_signals does (:254-268): signal length = fft_len for target, query
// and the reverse-complemented query.
//
// offs/n_offs: FindTop offsets per strand (strand s at offs + s*off_cap).
// segs/n_segs: raw DoOne segments per strand (3 ints each, at segs + s*3*seg_cap).
// Returns the number of t_result records (written up to cap).
int ref_align_pair(const char* t, int tlen, int t_chunk_start, unsigned long target_id,
                   const char* q, int qlen, int q_chunk_start, unsigned long query_id,
                   unsigned long query_size, int fft_len, double cutoff, int min_len,
                   double min_prob, double target_total, int query_chunk, void* probtable,
                   void* out, int cap,
                   int* offs, int* n_offs, int off_cap,
                   int* segs, int* n_segs, int seg_cap,
                   float* xc_out) {
  DNAVector dt = make_dna(t, tlen), dq = make_dna(q, qlen);
  DNAVector drc = dq;
  drc.ReverseComplement();
  CCSignal st, sq, srq;
  st.SetSequence(dt, fft_len);
  sq.SetSequence(dq, fft_len);
  srq.SetSequence(drc, fft_len);

  RefResult* res = (RefResult*)out;
  int nres = 0;
  CrossCorrelation xc;
  SeqAnalyzer sa;
  sa.SetTopCutoff(cutoff);
  for (int strand = 0; strand < 2; strand++) {
    const DNAVector& qs = strand ? drc : dq;
    std::vector<float> r;
    xc.CrossCorrelate(r, st, strand ? srq : sq);
    if (xc_out) memcpy(xc_out + (size_t)strand * fft_len, r.data(), sizeof(float) * fft_len);
    if (offs && n_offs) {
      std::vector<float> v = r;
      std::vector<int> top;
      sa.FindTop(top, v, cutoff);
      n_offs[strand] = (int)top.size();
      for (int i = 0; i < (int)top.size() && i < off_cap; i++) offs[strand * off_cap + i] = top[i];
    }
    vecSeqMatch m;
    sa.MatchUp(m, qs, dt, r);
    if (segs && n_segs) {
      n_segs[strand] = m.size();
      for (int i = 0; i < m.size() && i < seg_cap; i++) {
        int* sp = segs + (size_t)strand * 3 * seg_cap + 3 * i;
        sp[0] = m[i].GetStartTarget();
        sp[1] = m[i].GetStartQuery();
        sp[2] = m[i].GetLength();
      }
    }
    // FilterMatches (HomologyByXCorrSlave.cc:168-219)
    for (int j = 0; j < m.size(); j++) {
      if (m[j].GetLength() < min_len) continue;
      int len = m[j].GetLength();
      int tStart = t_chunk_start + m[j].GetStartTarget();
      int qStart;
      if (!strand)
        qStart = q_chunk_start + m[j].GetStartQuery();
      else
        qStart = rc_query(q_chunk_start, m[j].GetStartQuery(), len, query_chunk, (int)query_size);
      double prob, ident;
      if (probtable) {
        prob = ((ProbTable*)probtable)->GetMatchProbability(ident, dt, qs, m[j].GetStartTarget(),
                                                            m[j].GetStartQuery(), len);
        if (prob < min_prob) continue;
      } else {
        prob = GetMatchProbability(dt, qs, m[j].GetStartTarget(), m[j].GetStartQuery(), len,
                                   target_total);
        if (prob < min_prob) continue;
        ident = PrintMatch(qs, dt, m[j], true);
      }
      if (nres < cap) {
        RefResult& rr = res[nres];
        memset(&rr, 0, sizeof(rr));
        rr.query_id = query_id;
        rr.target_id = target_id;
        rr.query_size = query_size;
        rr.qstart = qStart;
        rr.tstart = tStart;
        rr.len = len;
        rr.reverse = strand != 0;
        rr.prob = prob;
        rr.ident = ident;
      }
      nres++;
    }
  }
  return nres;
}

}  // extern "C"
