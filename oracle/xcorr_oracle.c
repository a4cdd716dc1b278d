/*
 * TEST INFRASTRUCTURE ONLY -- the CPU oracle for the satsuma2 cross-correlation
 * path.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * --impl reference legs may load it, and only as the checker or the timed CPU
 * baseline.  The product (satsuma2_gb300) never links or calls it.
 *
 * A plain-C restatement of the reference algorithm, one function per reference
 * routine, each citing the file:line it follows (paths relative to the
 * satsuma2 source tree).  It is pinned against the reference itself: tests
 * compare it with oracle/_ref/libsatsuma_ref.so (the reference sources compiled
 * in place) and with golden vectors generated from that library and from the
 * unmodified reference slave binary (tests/golden/).
 *
 * Differences from the reference, on purpose:
 *  - the cross-correlation is computed in FP64 (own radix-2 FFT) instead of
 *    FFTReal's FP32; it is the "FP64 oracle" the GPU's FP32 result is held to.
 *    Offsets picked from it can differ from the reference's only where the
 *    reference's FP32 value straddles the cutoff.
 *  - inputs outside 7-bit ASCII are rejected (the reference indexes a
 *    [128][128] table with them, which is undefined behaviour).
 *
 * Compile with -ffp-contract=off: the reference is built for x86-64 without
 * FMA, and GCC on aarch64 would otherwise fuse a*b+c.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------------- */
/* DNA codec: DNACodec::DNACodec (analysis/DNAVector.cc:13-58)              */
/* ---------------------------------------------------------------------- */
static double W[4][256];
static unsigned char RC[256];
static int SCORE[128][128];      /* LookupMatch::precalc_scores, CrossCorr.cc:547-553 */
static double EQ[128][128];      /* DNA_Equal, DNAVector.cc:390-403 */
static int codec_ready = 0;
static pthread_mutex_t codec_mu = PTHREAD_MUTEX_INITIALIZER;

static void codec_set(int l, double a, double c, double g, double t, int rc) {
  W[0][l] = a; W[1][l] = c; W[2][l] = g; W[3][l] = t; RC[l] = (unsigned char)rc;
}

/* DNA_EqualAmb (DNAVector.cc:372-387) */
static double equal_amb(int l1, int l2) {
  if (l1 == l2 && l1 != 'N') return 1.;
  double a = W[0][l1] * W[0][l2];
  double c = W[1][l1] * W[1][l2];
  double g = W[2][l1] * W[2][l2];
  double t = W[3][l1] * W[3][l2];
  double sum = a + c + g + t;
  return sum + 0.;
}

/* DNA_Equal (DNAVector.cc:390-403) */
static double equal_w(int l1, int l2) {
  double a = W[0][l1] * W[0][l2];
  double c = W[1][l1] * W[1][l2];
  double g = W[2][l1] * W[2][l2];
  double t = W[3][l1] * W[3][l2];
  double sum = a + c + g + t;
  return sum + 0.;
}

void orc_init(void) {
  pthread_mutex_lock(&codec_mu);
  if (!codec_ready) {
    const double third = 1. / 3.;
    memset(W, 0, sizeof(W));
    memset(RC, 0, sizeof(RC));
    codec_set('A', 1., 0., 0., 0., 'T');
    codec_set('C', 0., 1., 0., 0., 'G');
    codec_set('G', 0., 0., 1., 0., 'C');
    codec_set('T', 0., 0., 0., 1., 'A');
    codec_set('K', 0., 0., 0.5, 0.5, 'M');
    codec_set('M', 0.5, 0.5, 0., 0., 'K');
    codec_set('R', 0.5, 0., 0.5, 0., 'Y');
    codec_set('Y', 0., 0.5, 0., 0.5, 'R');
    codec_set('S', 0., 0.5, 0.5, 0., 'S');
    codec_set('W', 0.5, 0., 0., 0.5, 'W');
    codec_set('B', 0., third, third, third, 'V');
    codec_set('V', third, third, third, 0., 'B');
    codec_set('H', third, third, 0., third, 'D');
    codec_set('D', third, 0., third, third, 'H');
    codec_set('-', 0., 0., 0., 0., '-');
    codec_set('N', 0.25, 0.25, 0.25, 0.25, 'N');
    codec_set('X', 0.25, 0.25, 0.25, 0.25, 'X');
    for (int i = 0; i < 128; i++)
      for (int j = 0; j < 128; j++) {
        SCORE[i][j] = (int)(equal_amb(i, j) * 100.0 + 0.5);
        EQ[i][j] = equal_w(i, j);
      }
    codec_ready = 1;
  }
  pthread_mutex_unlock(&codec_mu);
}

void orc_codec(int l, double* w4) { orc_init(); for (int c = 0; c < 4; c++) w4[c] = W[c][l & 255]; }
int orc_rc_letter(int l) { orc_init(); return RC[l & 255]; }
int orc_score(int a, int b) { orc_init(); return SCORE[a & 127][b & 127]; }
double orc_equal(int a, int b) { orc_init(); return EQ[a & 127][b & 127]; }

/* 0 when every byte is 7-bit ASCII, else -1. */
static int check_ascii(const unsigned char* s, int n) {
  for (int i = 0; i < n; i++) if (s[i] & 0x80) return -1;
  return 0;
}

/* DNAVector::ReverseComplement (DNAVector.cc:482-500): letters without a
 * complement in the codec become byte 0, as in the reference. */
void orc_rc(const char* in, int n, char* out) {
  orc_init();
  const unsigned char* s = (const unsigned char*)in;
  for (int i = 0; i < n; i++) out[i] = (char)RC[s[n - 1 - i]];
}

/* ---------------------------------------------------------------------- */
/* CCSignal (analysis/CrossCorr.cc:28-206)                                  */
/* ---------------------------------------------------------------------- */

/* Ent (CrossCorr.cc:28-33) */
static double ent(double p) {
  if (p < 0.001) return 0;
  return p * log(p) / 0.69314718056;
}

/* CCSignal::ComputeEntropy (CrossCorr.cc:35-93); e has L entries, zeroed. */
static void compute_entropy(const unsigned char* s, int len, int L, float* e) {
  if (len < 1024) {
    for (int i = 0; i < L; i++) e[i] = 1.f;
    return;
  }
  int win = L / 512;
  for (int i = 0; i < len; i += win) {
    double a = 0, c = 0, g = 0, t = 0;
    int k = 0;
    for (int j = i; j < i + win; j++) {
      if (j >= len) break;
      k++;
      a += W[0][s[j]];
      c += W[1][s[j]];
      g += W[2][s[j]];
      t += W[3][s[j]];
    }
    a /= (double)k;
    c /= (double)k;
    g /= (double)k;
    t /= (double)k;
    double sv = ent(a) + ent(c) + ent(g) + ent(t);
    for (int j = i; j < i + k; j++) {
      e[j] = (float)(-sv);
      if (e[j] < 0.) e[j] = 0.;
    }
  }
}

/* CCSignal::SetSequence (CrossCorr.cc:179-206) with SeqToPCM (:97-134):
 * out[c*L + k], channels A,C,G,T; zeros beyond len. Returns -1 on bad input. */
int orc_signal(const char* seq, int len, int L, float* out) {
  orc_init();
  const unsigned char* s = (const unsigned char*)seq;
  if (len < 0 || len > L || L < 1 || check_ascii(s, len)) return -1;
  float* e = (float*)calloc((size_t)L, sizeof(float));
  if (!e) return -2;
  compute_entropy(s, len, L, e);
  memset(out, 0, sizeof(float) * 4 * (size_t)L);
  for (int c = 0; c < 4; c++) {
    double sum = 0;
    for (int i = 0; i < len; i++) sum += W[c][s[i]];
    double off = sum / (double)len;
    float* o = out + (size_t)c * L;
    for (int i = 0; i < len; i++) o[i] = (float)((double)e[i] * (W[c][s[i]] - off));
  }
  free(e);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* FP64 cross-correlation with the reference's spectral treatment           */
/* (CrossCorrelation::CrossCorrelate / DoOne, CrossCorr.cc:386-507)         */
/* ---------------------------------------------------------------------- */

typedef struct { double re, im; } cplx;

/* In-place iterative radix-2 complex FFT, sign -1 (forward) or +1. */
static void fft64(cplx* a, int n, int sign) {
  for (int i = 1, j = 0; i < n; i++) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) { cplx t = a[i]; a[i] = a[j]; a[j] = t; }
  }
  for (int len = 2; len <= n; len <<= 1) {
    int h = len >> 1;
    for (int k = 0; k < h; k++) {
      double ang = sign * 2.0 * M_PI * (double)k / (double)len;
      double wr = cos(ang), wi = sin(ang);
      for (int i = k; i < n; i += len) {
        cplx u = a[i], v = a[i + h];
        double vr = v.re * wr - v.im * wi, vi = v.re * wi + v.im * wr;
        a[i].re = u.re + vr; a[i].im = u.im + vi;
        a[i + h].re = u.re - vr; a[i + h].im = u.im - vi;
      }
    }
  }
}

/* Spectra of two real signals x, y (length L) via one complex FFT:
 * X[k], Y[k] for k = 0..L/2 (standard e^{-j...} convention). */
static void two_real_spectra(const float* x, const float* y, int L, cplx* buf, cplx* X, cplx* Y) {
  for (int i = 0; i < L; i++) { buf[i].re = x ? x[i] : 0.0; buf[i].im = y ? y[i] : 0.0; }
  fft64(buf, L, -1);
  for (int k = 0; k <= L / 2; k++) {
    cplx zk = buf[k & (L - 1)], zn = buf[(L - k) & (L - 1)];
    /* X = (Z[k] + conj Z[L-k]) / 2 ; Y = (Z[k] - conj Z[L-k]) / (2j) */
    X[k].re = 0.5 * (zk.re + zn.re); X[k].im = 0.5 * (zk.im - zn.im);
    Y[k].re = 0.5 * (zk.im + zn.im); Y[k].im = -0.5 * (zk.re - zn.re);
  }
}

/*
 * Sum over the four channels of the reference's per-channel correlation, in
 * FP64.  Per channel the reference forms, in FFTReal's layout, conj(T)*Q on
 * bins 1..N-2 (CrossCorr.cc:482-492), T(0)*Q(0) on bin 0 (:480), and leaves
 * bins N-1 and N (Nyquist) holding the target's own spectrum; then inverse,
 * 1/L rescale (:493-494) and a half rotation o[i] = x[(i+N) mod L] (:500-505).
 * In the standard negative-exponent convention that is, with r = IDFT(S)/L:
 *   S(k) = conj(T(k)) Q(k), k = 1..N-2;  S(0) = T(0)Q(0);
 *   S(N-1) = T(N-1);  S(N) = T(N);  S(L-k) = conj S(k).
 * xc must hold L doubles.
 */
static void xcorr64_sig(const float* ts, const float* qs, int L, double* xc) {
  int N = L / 2;
  cplx* buf = (cplx*)malloc(sizeof(cplx) * L);
  cplx* T = (cplx*)malloc(sizeof(cplx) * (N + 1));
  cplx* Q = (cplx*)malloc(sizeof(cplx) * (N + 1));
  cplx* S = (cplx*)calloc((size_t)N + 1, sizeof(cplx));
  for (int c = 0; c < 4; c++) {
    two_real_spectra(ts + (size_t)c * L, qs + (size_t)c * L, L, buf, T, Q);
    for (int k = 0; k <= N; k++) {
      double sr, si;
      if (k == 0) { sr = T[0].re * Q[0].re; si = 0; }
      else if (k >= N - 1) { sr = T[k].re; si = T[k].im; }
      else { sr = T[k].re * Q[k].re + T[k].im * Q[k].im; si = T[k].re * Q[k].im - T[k].im * Q[k].re; }
      S[k].re += sr; S[k].im += si;
    }
  }
  /* Hermitian extension and inverse */
  for (int k = 0; k < L; k++) {
    if (k <= N) buf[k] = S[k];
    else { buf[k].re = S[L - k].re; buf[k].im = -S[L - k].im; }
  }
  buf[N].im = 0;  /* Nyquist bin of a real signal has no imaginary part */
  buf[0].im = 0;
  fft64(buf, L, +1);
  for (int i = 0; i < L; i++) xc[i] = buf[(i + N) & (L - 1)].re / (double)L;
  free(buf); free(T); free(Q); free(S);
}

/* Signals of t and q at length L, then xcorr64_sig. */
int orc_xcorr64(const char* t, int tlen, const char* q, int qlen, int L, double* xc) {
  float* ts = (float*)malloc(sizeof(float) * 4 * (size_t)L);
  float* qs = (float*)malloc(sizeof(float) * 4 * (size_t)L);
  int rc = orc_signal(t, tlen, L, ts);
  if (!rc) rc = orc_signal(q, qlen, L, qs);
  if (!rc) xcorr64_sig(ts, qs, L, xc);
  free(ts); free(qs);
  return rc;
}

/* ---------------------------------------------------------------------- */
/* SeqAnalyzer (analysis/CrossCorr.cc:557-724, 878-944)                     */
/* ---------------------------------------------------------------------- */

/* SeqAnalyzer::FindTop (CrossCorr.cc:878-944); envelope size 256 (:562).
 * Returns the count; writes up to cap indices. */
int orc_findtop(const double* xc, int L, double cutoff, int* out, int cap) {
  const int envSize = 256;
  int nPoints = L / envSize;
  if (nPoints == 0) nPoints = 1;
  double* env = (double*)calloc((size_t)nPoints, sizeof(double));
  for (int i = 0; i < L; i++) {
    float xf = (float)xc[i];
    double d = (double)(float)(xf * xf);  /* float product, as xc[i]*xc[i] on floats */
    if (nPoints > 8) env[i / envSize] += d;
  }
  for (int b = 0; b < nPoints; b++) env[b] = sqrt(env[b] / (double)envSize);
  int n = 0;
  for (int i = 0; i < L; i++) {
    if (xc[i] > env[i / envSize] * cutoff + 1.0) {
      if (n < cap) out[n] = i;
      n++;
    }
  }
  free(env);
  return n;
}

/* Same on FP32 input (the reference's own xc type). */
int orc_findtop_f32(const float* xc, int L, double cutoff, int* out, int cap) {
  double* d = (double*)malloc(sizeof(double) * L);
  for (int i = 0; i < L; i++) d[i] = xc[i];
  int n = orc_findtop(d, L, cutoff, out, cap);
  free(d);
  return n;
}

/* Envelope threshold per index (for straddle classification). */
void orc_thresholds(const double* xc, int L, double cutoff, double* thr) {
  const int envSize = 256;
  int nPoints = L / envSize;
  if (nPoints == 0) nPoints = 1;
  double* env = (double*)calloc((size_t)nPoints, sizeof(double));
  for (int i = 0; i < L; i++) {
    float xf = (float)xc[i];
    if (nPoints > 8) env[i / envSize] += (double)(float)(xf * xf);
  }
  for (int b = 0; b < nPoints; b++) env[b] = sqrt(env[b] / (double)envSize);
  for (int i = 0; i < L; i++) thr[i] = env[i / envSize] * cutoff + 1.0;
  free(env);
}

/* SeqAnalyzer::DoOne, OPTIM_DOONE variant (CrossCorr.cc:667-724) with
 * m_minLen 45 and m_minIdent 0.42 (:557-563) and LookupMatch scale 100.
 * segs[3*i] = tStart, qStart, len.  Returns the count. */
int orc_doone(const char* tch, int T, const char* qch, int Q, int pos, int* segs, int cap) {
  orc_init();
  const unsigned char* t = (const unsigned char*)tch;
  const unsigned char* q = (const unsigned char*)qch;
  const int mlen = 45;
  const int minMatches = (int)((double)mlen * 0.42 * (double)100);
  int match = 0, lastStart = -1, n = 0, cnt = 0;
  for (int i = 0; i < T; i++) {
    int j = i + pos;
    if (j < 0) continue;
    if (j >= Q || i + 1 >= T) {
      if (lastStart != -1) {
        if (cnt < cap) { segs[3*cnt] = lastStart; segs[3*cnt+1] = lastStart + pos; segs[3*cnt+2] = i - lastStart; }
        cnt++;
      }
      break;
    }
    match += SCORE[t[i] & 127][q[j] & 127];
    if (n > mlen) {
      match -= SCORE[t[i - mlen - 1] & 127][q[j - mlen - 1] & 127];
      if (match > minMatches) {
        if (lastStart == -1) lastStart = i - mlen;
      } else {
        if (lastStart != -1) {
          if (cnt < cap) { segs[3*cnt] = lastStart; segs[3*cnt+1] = lastStart + pos; segs[3*cnt+2] = i - lastStart; }
          cnt++;
        }
        lastStart = -1;
      }
    }
    n++;
  }
  return cnt;
}

int orc_min_matches(void) { return (int)((double)45 * 0.42 * (double)100); }

/* ---------------------------------------------------------------------- */
/* Match probability (analysis/AlignProbability.cc:11-126)                  */
/* ---------------------------------------------------------------------- */

static double cdf_(double x, double m, double s) { return 0.5 * (1. + erf((x - m) / s / 1.414213562)); }
static double sigma_(double p, int N) { return sqrt(p * (1. - p) * (double)N); }
static double gc_adjust(double gc, int N, double gc_target) {
  double at_target = 1. - gc_target;
  double r = gc * gc_target;
  r += (double)(N - gc) * at_target;
  return r / (double)N / 2.;
}

/* GetMatchProbabilityEx (AlignProbability.cc:62-126) */
double orc_match_prob(const char* tch, const char* qch, int ts, int qs, int length,
                      double targetSize, double* ident_out) {
  orc_init();
  const unsigned char* t = (const unsigned char*)tch + ts;
  const unsigned char* q = (const unsigned char*)qch + qs;
  double gcT = 0, gcQ = 0, matches = 0;
  for (int i = 0; i < length; i++) {
    matches += EQ[t[i] & 127][q[i] & 127];
    gcT += W[1][t[i]] + W[2][t[i]];
    gcQ += W[1][q[i]] + W[2][q[i]];
  }
  double ident = matches / (double)length;
  if (ident_out) *ident_out = ident;
  double p_match = gc_adjust(gcQ, length, gcT / (double)length);
  double s = sigma_(p_match, length);
  double m = p_match * (double)length;
  double x = (double)length * ident;
  double cdf = cdf_(m, x, s);
  double expect = cdf * targetSize;
  return exp(-expect);
}

/* PrintMatch(..., bSilent=true, bNuc=true) identity (CrossCorr.cc:967-1037) */
double orc_print_ident(const char* tch, const char* qch, int ts, int qs, int length) {
  orc_init();
  const unsigned char* t = (const unsigned char*)tch;
  const unsigned char* q = (const unsigned char*)qch;
  double matches = 0;
  for (int i = ts; i < ts + length; i++) {
    int j = qs + i - ts;
    matches += EQ[q[j] & 127][t[i] & 127];
  }
  return matches / (double)length;
}

/* ---------------------------------------------------------------------- */
/* ProbTable (analysis/ProbTable.cc:7-165)                                  */
/* ---------------------------------------------------------------------- */
#define PT_ROWS 512
#define PT_LEN 2048

/* ProbTable::GetMatchProbabilityRaw (ProbTable.cc:143-165) */
static double pt_raw(int length, double ident, double ident_expect, double targetSize) {
  double p_match = ident_expect;
  double s = sigma_(p_match, length);
  double m = p_match * (double)length;
  double x = (double)length * ident;
  double cdf = cdf_(m, x, s);
  return exp(-cdf * targetSize);
}

typedef struct { double size, cutoff; double* table; int lo, hi; } pt_job;

static void* pt_worker(void* arg) {
  pt_job* jb = (pt_job*)arg;
  for (int i = jb->lo; i < jb->hi; i++) {
    double ident_expect = (double)i / ((double)PT_ROWS - 1);
    double* t = jb->table + (size_t)i * PT_LEN;
    t[0] = 2.;
    for (int j = 1; j < PT_LEN; j++) {
      double mn, mx, mid;
      for (mn = 0, mx = 1; mx - mn > 0.00000001;) {
        mid = (mx + mn) / 2.0;
        if (pt_raw(j, mid, ident_expect, jb->size)) mx = mid;
        else mn = mid;
      }
      t[j] = (mx + mn) / 2.0;
    }
  }
  return 0;
}

/* ProbTable::Setup (ProbTable.cc:15-56): rows 1..511 of 2048 cutoffs (row 0
 * unused, filled with -1).  Note the reference tests the raw probability as a
 * boolean (nonzero), not against the cutoff.  table: PT_ROWS*PT_LEN doubles. */
void orc_probtable_build(double targetSize, double cutoff, double* table, int nthreads) {
  (void)cutoff;
  for (int j = 0; j < PT_LEN; j++) table[j] = -1.0;
  if (nthreads < 1) nthreads = 1;
  pthread_t th[64];
  pt_job jobs[64];
  if (nthreads > 64) nthreads = 64;
  int rows = PT_ROWS - 1;
  for (int w = 0; w < nthreads; w++) {
    jobs[w].size = targetSize; jobs[w].cutoff = cutoff; jobs[w].table = table;
    jobs[w].lo = 1 + rows * w / nthreads; jobs[w].hi = 1 + rows * (w + 1) / nthreads;
    pthread_create(&th[w], 0, pt_worker, &jobs[w]);
  }
  for (int w = 0; w < nthreads; w++) pthread_join(th[w], 0);
}

/* ProbTable::GetMatchProbability (ProbTable.cc:105-140) with IsGood (:58-69).
 * Row 0 of the reference table is an empty vector, so an expectation index of
 * 0 reads out of bounds there; here it is treated as "not good". */
double orc_probtable_prob(const double* table, double cutoff, const char* tch, const char* qch,
                          int ts, int qs, int length, double* ident_out) {
  orc_init();
  const unsigned char* t = (const unsigned char*)tch + ts;
  const unsigned char* q = (const unsigned char*)qch + qs;
  double gcT = 0, gcQ = 0, matches = 0;
  for (int i = 0; i < length; i++) {
    matches += EQ[t[i] & 127][q[i] & 127];
    gcT += W[1][t[i]] + W[2][t[i]];
    gcQ += W[1][q[i]] + W[2][q[i]];
  }
  double ident = matches / (double)length;
  if (ident_out) *ident_out = ident;
  double p_match = gc_adjust(gcQ, length, gcT / (double)length);
  int index = (int)(p_match * (PT_ROWS - 1));
  if (index <= 0 || index >= PT_ROWS) return 0.;
  int l = length >= PT_LEN ? PT_LEN - 1 : length;
  return ident >= table[(size_t)index * PT_LEN + l] ? cutoff : 0.;
}

/* ---------------------------------------------------------------------- */
/* One chunk pair: HomologyByXCorr::Align + FilterMatches                   */
/* (analysis/HomologyByXCorrSlave.cc:56-60, 168-253)                        */
/* ---------------------------------------------------------------------- */

/* Same layout as t_result (analysis/WorkQueue.h:23-33). */
typedef struct {
  uint64_t query_id, target_id, query_size, qstart, tstart, len;
  unsigned char reverse;
  double prob, ident;
} orc_result;

typedef struct {
  const char* tseq; int tlen; int t_chunk_start; uint64_t target_id;
  const char* qseq; int qlen; int q_chunk_start; uint64_t query_id; uint64_t query_size;
  int fast;
} orc_pair;

typedef struct {
  double cutoff, cutoff_fast, min_prob, target_total;
  int min_len, t_chunk, q_chunk, fft_len;
  const double* probtable;   /* NULL: GetMatchProbability; else table mode */
  double probtable_cutoff;   /* ProbTable's own cutoff (-min_prob) */
} orc_params;

/* One pair, both strands, with the FP64 correlation.  xc_in, if given,
 * supplies 2*L precomputed correlation values to pick offsets from instead
 * (e.g. the reference's own FP32 values); offs_in/n_offs_in, if given, supply
 * the FindTop offsets per strand directly (strand s at offs_in + s*offs_in_cap).
 * Optional outputs as in the reference harness.  Returns the result count. */
int orc_align_pair(const orc_params* P, const orc_pair* pr, const float* xc_in,
                   const int* offs_in, const int* n_offs_in, int offs_in_cap,
                   orc_result* out, int cap,
                   int* offs, int* n_offs, int off_cap,
                   int* segs, int* n_segs, int seg_cap,
                   double* xc_out) {
  orc_init();
  int L = P->fft_len > 0 ? P->fft_len : 2 * P->t_chunk;
  if (pr->tlen > L || pr->qlen > L || pr->tlen < 0 || pr->qlen < 0) return -1;
  if (check_ascii((const unsigned char*)pr->tseq, pr->tlen) ||
      check_ascii((const unsigned char*)pr->qseq, pr->qlen)) return -1;
  char* rcq = (char*)malloc((size_t)pr->qlen + 1);
  orc_rc(pr->qseq, pr->qlen, rcq);
  float* ts = (float*)malloc(sizeof(float) * 4 * (size_t)L);
  float* qs = (float*)malloc(sizeof(float) * 4 * (size_t)L);
  double* xc = (double*)malloc(sizeof(double) * L);
  int* top = (int*)malloc(sizeof(int) * L);
  int scap = 1 << 16;
  int* sg = (int*)malloc(sizeof(int) * 3 * scap);
  orc_signal(pr->tseq, pr->tlen, L, ts);
  double cutoff = pr->fast ? P->cutoff_fast : P->cutoff;
  int nres = 0;
  for (int strand = 0; strand < 2; strand++) {
    const char* q = strand ? rcq : pr->qseq;
    int nt;
    if (offs_in && n_offs_in) {
      nt = n_offs_in[strand];
      for (int i = 0; i < nt; i++) top[i] = offs_in[strand * offs_in_cap + i];
    } else {
      if (xc_in) {
        for (int i = 0; i < L; i++) xc[i] = xc_in[(size_t)strand * L + i];
      } else {
        orc_signal(q, pr->qlen, L, qs);
        xcorr64_sig(ts, qs, L, xc);
      }
      if (xc_out) memcpy(xc_out + (size_t)strand * L, xc, sizeof(double) * L);
      nt = orc_findtop(xc, L, cutoff, top, L);
    }
    if (offs && n_offs) {
      n_offs[strand] = nt;
      for (int i = 0; i < nt && i < off_cap; i++) offs[strand * off_cap + i] = top[i];
    }
    /* SeqAnalyzer::MatchUp (CrossCorr.cc:583-605) */
    int ns = 0;
    for (int i = 0; i < nt; i++) {
      int pos = top[i] - L / 2;
      int room = scap - ns;
      int c = orc_doone(pr->tseq, pr->tlen, q, pr->qlen, pos, sg + 3 * ns, room);
      if (c > room) {   /* low-complexity chunks: grow the segment buffer and redo */
        while (scap - ns < c) scap *= 2;
        int* g = (int*)realloc(sg, sizeof(int) * 3 * (size_t)scap);
        if (!g) break;
        sg = g;
        c = orc_doone(pr->tseq, pr->tlen, q, pr->qlen, pos, sg + 3 * ns, scap - ns);
      }
      ns += c;
    }
    if (segs && n_segs) {
      n_segs[strand] = ns;
      for (int i = 0; i < ns && i < seg_cap; i++)
        memcpy(segs + (size_t)strand * 3 * seg_cap + 3 * i, sg + 3 * i, 3 * sizeof(int));
    }
    /* FilterMatches (HomologyByXCorrSlave.cc:168-219) */
    for (int j = 0; j < ns; j++) {
      int st = sg[3 * j], sq = sg[3 * j + 1], len = sg[3 * j + 2];
      if (len < P->min_len) continue;
      int tStart = pr->t_chunk_start + st;
      int qStart = strand ? sq + (int)pr->query_size - pr->q_chunk_start - P->q_chunk
                          : pr->q_chunk_start + sq;
      double prob, ident;
      if (P->probtable) {
        prob = orc_probtable_prob(P->probtable, P->probtable_cutoff, pr->tseq, q, st, sq, len, &ident);
        if (prob < P->min_prob) continue;
      } else {
        prob = orc_match_prob(pr->tseq, q, st, sq, len, P->target_total, 0);
        if (prob < P->min_prob) continue;
        ident = orc_print_ident(pr->tseq, q, st, sq, len);
      }
      if (nres < cap) {
        orc_result* r = &out[nres];
        memset(r, 0, sizeof(*r));
        r->query_id = pr->query_id;
        r->target_id = pr->target_id;
        r->query_size = pr->query_size;
        r->qstart = (uint64_t)(int64_t)qStart;
        r->tstart = (uint64_t)(int64_t)tStart;
        r->len = (uint64_t)(int64_t)len;
        r->reverse = (unsigned char)strand;
        r->prob = prob;
        r->ident = ident;
      }
      nres++;
    }
  }
  free(rcq); free(ts); free(qs); free(xc); free(top); free(sg);
  return nres;
}

/* ---------------------------------------------------------------------- */
/* Multi-threaded batch driver for the timed CPU baseline                   */
/* ---------------------------------------------------------------------- */
typedef struct {
  const orc_params* P; const orc_pair* pairs; int n; int* next; pthread_mutex_t* mu;
  long long results;
} batch_job;

static void* batch_worker(void* arg) {
  batch_job* jb = (batch_job*)arg;
  orc_result buf[4096];
  for (;;) {
    pthread_mutex_lock(jb->mu);
    int i = (*jb->next)++;
    pthread_mutex_unlock(jb->mu);
    if (i >= jb->n) break;
    int r = orc_align_pair(jb->P, &jb->pairs[i], 0, 0, 0, 0, buf, 4096, 0, 0, 0, 0, 0, 0, 0);
    if (r > 0) jb->results += r;
  }
  return 0;
}

/* Runs n pairs on nthreads host threads; returns the total result count. */
long long orc_align_batch(const orc_params* P, const orc_pair* pairs, int n, int nthreads) {
  orc_init();
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  batch_job jobs[256];
  int next = 0;
  pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
  for (int w = 0; w < nthreads; w++) {
    jobs[w].P = P; jobs[w].pairs = pairs; jobs[w].n = n; jobs[w].next = &next; jobs[w].mu = &mu;
    jobs[w].results = 0;
    pthread_create(&th[w], 0, batch_worker, &jobs[w]);
  }
  long long tot = 0;
  for (int w = 0; w < nthreads; w++) { pthread_join(th[w], 0); tot += jobs[w].results; }
  return tot;
}
