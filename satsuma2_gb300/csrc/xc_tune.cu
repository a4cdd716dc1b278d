// Autotuner of the correlation stage: for each FFT length it times the
// kernel forms the library is built with on a synthetic batch and keeps the
// fastest in the context.
//
// The forms differ in threads per transform and pairs per CTA, and compute
// bit-identical results (the same butterflies and sums in the same order), so
// the choice changes speed only:
//   FFT 1024..4096   per-strand kernel with 512, 256 or 128 threads per strand
//                    (transform groups of 256, 128 or 64 threads; 2, 4 or 8
//                    CTAs per SM).  FFTReal's single fixed pass structure
//                    (extern/RealFFT/FFTReal.hpp:429-458) is what this choice
//                    replaces: a short transform on a wide CTA leaves most of
//                    its threads idle in every pass.
//   FFT 8192         the persistent 512-thread both-strands kernel, the
//                    1024-thread one-CTA-per-pair form, or the per-strand
//                    kernel alone (512 or 256 threads).
//   FFT 16384, 32768 one form (512 threads).
// The table is plain text, one line per length, which xc_apply_tuning (or
// SATSUMA2_GB300_TUNING at xc_create) reads back.
#include "satsuma2_xcorr.h"
#include "xc_runtime.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace xc {

namespace {

struct Rng {   // xorshift64*
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 1) {}
  uint64_t next() {
    s ^= s >> 12;
    s ^= s << 25;
    s ^= s >> 27;
    return s * 0x2545F4914F6CDD1Dull;
  }
  int below(int n) { return (int)(next() % (uint64_t)n); }
};

// n chunk pairs of len bases each: a random target, and a query holding an
// 85%-identity copy of a random target segment (reverse-complemented for
// every other pair) in random flanks -- the shape of the benchmark batches.
void synth_pairs(int n, int len, uint64_t seed, std::vector<std::string>& seqs, std::vector<xc_pair>& pairs) {
  static const char acgt[4] = {'A', 'C', 'G', 'T'};
  Rng r(seed);
  seqs.assign(2 * (size_t)n, std::string());
  pairs.assign(n, xc_pair{});
  for (int i = 0; i < n; i++) {
    std::string& t = seqs[2 * i];
    std::string& q = seqs[2 * i + 1];
    t.resize(len);
    q.resize(len);
    for (int k = 0; k < len; k++) t[k] = acgt[r.below(4)];
    for (int k = 0; k < len; k++) q[k] = acgt[r.below(4)];
    const int hl = len / 8 + r.below(len / 2);
    const int ts = r.below(len - hl + 1), qs = r.below(len - hl + 1);
    for (int k = 0; k < hl; k++) {
      char b = t[ts + k];
      if (i & 1) {   // reverse complement
        const char c = t[ts + hl - 1 - k];
        b = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : 'A';
      }
      if (r.below(100) < 15) b = acgt[r.below(4)];
      q[qs + k] = b;
    }
    xc_pair& p = pairs[i];
    p.tseq = t.data();
    p.tlen = len;
    p.qseq = q.data();
    p.qlen = len;
    p.query_size = (unsigned long)len;
  }
}

// Median correlation-stage time (ms) of the packed batch under the context's
// current choices: two warm runs, then five timed ones.
int time_corr(Ctx* c, Batch* b, cudaStream_t s, float* ms) {
  std::vector<float> v;
  for (int k = 0; k < 7; k++) {
    int r = batch_run(c, b, s, false, true);
    if (r != XC_OK) return r;
    if (cudaEventSynchronize(b->ev[3]) != cudaSuccess) return XC_ERR_CUDA;
    float st = 0.f;
    if (cudaEventElapsedTime(&st, b->ev[0], b->ev[1]) != cudaSuccess) return XC_ERR_CUDA;
    if (k >= 2) v.push_back(st);
  }
  std::sort(v.begin(), v.end());
  *ms = v[v.size() / 2];
  return XC_OK;
}

}  // namespace

int apply_tuning_text(Ctx* c, const char* text) {
  const char* line = text;
  while (line && *line) {
    const char* end = strchr(line, '\n');
    const std::string l(line, end ? (size_t)(end - line) : strlen(line));
    line = end ? end + 1 : nullptr;
    int L = 0;
    if (sscanf(l.c_str(), "fft_len=%d", &L) != 1) continue;
    int lg = 0;
    while ((1 << lg) < L) lg++;
    if ((1 << lg) != L || lg < MIN_LOG2L || lg > MAX_LOG2L) return XC_ERR_ARG;
    const char* st = strstr(l.c_str(), "strand_threads=");
    if (st) {
      int nt = 0;
      if (sscanf(st, "strand_threads=%d", &nt) != 1 || !strand_threads_ok(lg, nt)) return XC_ERR_ARG;
      c->strand_threads[lg] = nt;
    }
    const char* pf = strstr(l.c_str(), "pair_form=");
    if (pf && lg == PAIR_LOG2L) {
      int f = -1;
      if (sscanf(pf, "pair_form=%d", &f) != 1 || f < 0 || f > 2) return XC_ERR_ARG;
      if (f == 0) c->pair_kernel = false;
      else c->pair_form = f;   // (the both-strands kernel stays off where the context found it unusable)
    }
  }
  return XC_OK;
}

}  // namespace xc

using namespace xc;

extern "C" {

int xc_tune(xc_ctx* c, char* table, size_t cap, size_t* table_len) {
  if (!c) return XC_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  const xc_params saved = c->prm;
  const bool pair_usable = c->pair_kernel;
  std::string out;
  int r = XC_OK;
  cudaStream_t s = c->stream;
  for (int lg = MIN_LOG2L; lg <= PAIR_LOG2L && r == XC_OK; lg++) {
    const int L = 1 << lg;
    const int n = lg == PAIR_LOG2L ? 1536 : 2048;
    std::vector<std::string> seqs;
    std::vector<xc_pair> pairs;
    synth_pairs(n, L / 2, 1000 + lg, seqs, pairs);
    c->prm.fft_len = L;
    Batch* b = new_batch(c);
    r = batch_pack(c, b, pairs.data(), pairs.size(), s);
    struct Cand {
      const char* name;
      bool pair;
      int form, nt;
    };
    std::vector<Cand> cands;
    if (lg == PAIR_LOG2L) {
      if (pair_usable) {
        cands.push_back({"pair_form=2", true, 2, 512});
        cands.push_back({"pair_form=1", true, 1, 512});
      }
      cands.push_back({"strand512", false, 0, 512});
      cands.push_back({"strand256", false, 0, 256});
    } else {
      for (int nt : {512, 256, 128})
        if (strand_threads_ok(lg, nt)) cands.push_back({nt == 512 ? "strand512" : nt == 256 ? "strand256" : "strand128", false, 0, nt});
    }
    float best = 1e30f;
    int bi = -1;
    std::string detail;
    for (size_t k = 0; k < cands.size() && r == XC_OK; k++) {
      c->pair_kernel = cands[k].pair;
      if (cands[k].pair) c->pair_form = cands[k].form;
      c->strand_threads[lg] = cands[k].nt;
      float ms = 0.f;
      r = time_corr(c, b, s, &ms);
      char buf[64];
      snprintf(buf, sizeof(buf), "%s%s: %.4f", k ? ", " : "", cands[k].name, ms);
      detail += buf;
      if (r == XC_OK && ms < best) {
        best = ms;
        bi = (int)k;
      }
    }
    if (r == XC_OK) cudaStreamSynchronize(s);
    delete b;
    if (r != XC_OK || bi < 0) break;
    const Cand& w = cands[bi];
    c->pair_kernel = lg == PAIR_LOG2L ? w.pair : pair_usable;
    if (w.pair) c->pair_form = w.form;
    c->strand_threads[lg] = w.nt;
    char line[256];
    if (lg == PAIR_LOG2L)
      snprintf(line, sizeof(line), "fft_len=%d pair_form=%d strand_threads=%d corr_ms=%.4f pairs=%d (%s)\n", L,
               w.pair ? w.form : 0, w.nt, best, n, detail.c_str());
    else
      snprintf(line, sizeof(line), "fft_len=%d strand_threads=%d corr_ms=%.4f pairs=%d (%s)\n", L, w.nt, best, n,
               detail.c_str());
    out += line;
  }
  c->prm = saved;
  if (r != XC_OK) {
    c->pair_kernel = pair_usable;
    return r;
  }
  if (table_len) *table_len = out.size();
  if (table) {
    if (cap < out.size() + 1) return XC_ERR_CAPACITY;
    memcpy(table, out.c_str(), out.size() + 1);
  }
  return XC_OK;
}

int xc_apply_tuning(xc_ctx* c, const char* table) {
  if (!c || !table) return XC_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  return apply_tuning_text(c, table);
}

}  // extern "C"
