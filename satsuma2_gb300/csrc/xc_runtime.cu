// Host runtime of libsatsuma2_gb300.so: device tables, batch packing,
// launch sequencing (graph-captured), result assembly and the C ABI declared in
// include/satsuma2_xcorr.h.
#include "satsuma2_xcorr.h"
#include "xc_internal.h"
#include "xc_runtime.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

static_assert(sizeof(xc_result) == 72, "xc_result must match t_result (72 bytes)");
static_assert(sizeof(xc_block) == 28, "xc_block must match t_pair (28 bytes)");

namespace xc {

// ---------------------------------------------------------------------------
// DNA codec: DNACodec::DNACodec (analysis/DNAVector.cc:13-58)
// ---------------------------------------------------------------------------
struct Codec {
  double w[4][256];
  unsigned char rc[256];
  Codec() {
    memset(w, 0, sizeof(w));
    memset(rc, 0, sizeof(rc));
    const double third = 1. / 3.;
    set('A', 1., 0., 0., 0., 'T');
    set('C', 0., 1., 0., 0., 'G');
    set('G', 0., 0., 1., 0., 'C');
    set('T', 0., 0., 0., 1., 'A');
    set('K', 0., 0., 0.5, 0.5, 'M');
    set('M', 0.5, 0.5, 0., 0., 'K');
    set('R', 0.5, 0., 0.5, 0., 'Y');
    set('Y', 0., 0.5, 0., 0.5, 'R');
    set('S', 0., 0.5, 0.5, 0., 'S');
    set('W', 0.5, 0., 0., 0.5, 'W');
    set('B', 0., third, third, third, 'V');
    set('V', third, third, third, 0., 'B');
    set('H', third, third, 0., third, 'D');
    set('D', third, 0., third, third, 'H');
    set('-', 0., 0., 0., 0., '-');
    set('N', 0.25, 0.25, 0.25, 0.25, 'N');
    set('X', 0.25, 0.25, 0.25, 0.25, 'X');
  }
  void set(int l, double a, double c, double g, double t, int r) {
    w[0][l] = a; w[1][l] = c; w[2][l] = g; w[3][l] = t; rc[l] = (unsigned char)r;
  }
  // DNA_Equal (DNAVector.cc:390-403)
  double equal(int a, int b) const {
    double s = w[0][a] * w[0][b];
    s = s + w[1][a] * w[1][b];
    s = s + w[2][a] * w[2][b];
    s = s + w[3][a] * w[3][b];
    return s + 0.;
  }
  // DNA_EqualAmb (DNAVector.cc:372-387)
  double equal_amb(int a, int b) const {
    if (a == b && a != 'N') return 1.;
    return equal(a, b);
  }
};

static const Codec& codec() {
  static Codec c;
  return c;
}

static int cuda_err(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return XC_OK;
  fprintf(stderr, "satsuma2_gb300: %s: %s\n", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? XC_ERR_NOMEM : XC_ERR_CUDA;
}
#define XC_CHECK(call)                                        \
  do {                                                        \
    int _r = cuda_err((call), #call);                         \
    if (_r != XC_OK) return _r;                               \
  } while (0)

static int build_tables(Ctx* c) {
  for (int lg = MIN_LOG2L; lg <= MAX_LOG2L; lg++) {
    const int L = 1 << lg, N = L / 2, win = L / 512;
    // Two-level twiddle tables: W_M^m = hi[m >> 6] * lo[m & 63], M = N and L,
    // each entry computed in double and rounded once.
    const int NH = N / 64;
    std::vector<float2> tw(2 * (NH + 64));
    auto w = [](double num, double den) {
      const double a = -2.0 * M_PI * num / den;
      return make_float2((float)cos(a), (float)sin(a));
    };
    for (int i = 0; i < NH; i++) {
      tw[i] = w(64.0 * i, N);
      tw[NH + 64 + i] = w(64.0 * i, L);
    }
    for (int i = 0; i < 64; i++) {
      tw[NH + i] = w(i, N);
      tw[2 * NH + 64 + i] = w(i, L);
    }
    // Ent(p) for p = (a4/4)/k (CrossCorr.cc:28-33,80-84), same double ops.
    const int row = 4 * win + 1;
    std::vector<double> ent((size_t)(win + 1) * row, 0.0);
    for (int k = 1; k <= win; k++)
      for (int a4 = 0; a4 <= 4 * k; a4++) {
        double p = (double)a4 * 0.25;
        p /= (double)k;
        ent[(size_t)k * row + a4] = p < 0.001 ? 0.0 : p * log(p) / 0.69314718056;
      }
    // Weight of a full window holding a A, c C, g G, t T (ComputeEntropy,
    // CrossCorr.cc:80-91): -(Ent(a/w) + Ent(c/w) + Ent(g/w) + Ent(t/w)) in
    // that order, rounded to float, clamped at 0 -- the kernel's own double
    // steps, done once here.
    const int W1 = win + 1;
    std::vector<float> eacgt((size_t)W1 * W1 * W1, 0.f);
    for (int a = 0; a <= win; a++)
      for (int cc = 0; a + cc <= win; cc++)
        for (int g = 0; a + cc + g <= win; g++) {
          const int tt = win - a - cc - g;
          const double* er = &ent[(size_t)win * row];
          const double sv = ((er[4 * a] + er[4 * cc]) + er[4 * g]) + er[4 * tt];
          float E = (float)(-sv);
          if (E < 0.f) E = 0.f;
          eacgt[((size_t)a * W1 + cc) * W1 + g] = E;
        }
    if (lg == PAIR_LOG2L) {
      // corr_pair_kernel takes a reverse-strand window (the complement bases
      // of a forward window: t A, g C, c G, a T) at the forward window's weight
      bool sym = true;
      for (int a = 0; a <= win; a++)
        for (int cc = 0; a + cc <= win; cc++)
          for (int g = 0; a + cc + g <= win; g++) {
            const int tt = win - a - cc - g;
            sym = sym && eacgt[((size_t)a * W1 + cc) * W1 + g] == eacgt[((size_t)tt * W1 + g) * W1 + cc];
          }
      // SATSUMA2_GB300_PAIR_KERNEL: "0" one corr_kernel CTA per strand for
      // every pair, "1" the 1024-thread both-strands kernel, else (default)
      // the persistent 512-thread one
      const char* env = getenv("SATSUMA2_GB300_PAIR_KERNEL");
      c->pair_kernel = sym && !(env && env[0] == '0');
      c->pair_form = (env && env[0] == '1') ? 1 : 2;
      // SATSUMA2_GB300_SPECTRA=0: no spectra path (every pair transforms its chunks)
      const char* es = getenv("SATSUMA2_GB300_SPECTRA");
      c->spec_reuse = !(es && es[0] == '0');
    }
    DevTables& t = c->tab[lg];
    XC_CHECK(cudaMalloc(&t.tw, tw.size() * sizeof(float2)));
    XC_CHECK(cudaMalloc(&t.ent, ent.size() * sizeof(double)));
    XC_CHECK(cudaMalloc(&t.ent_acgt, eacgt.size() * sizeof(float)));
    XC_CHECK(cudaMemcpy(t.tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice));
    XC_CHECK(cudaMemcpy(t.ent, ent.data(), ent.size() * sizeof(double), cudaMemcpyHostToDevice));
    XC_CHECK(cudaMemcpy(t.ent_acgt, eacgt.data(), eacgt.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  const Codec& cd = codec();
  std::vector<int8_t> score(128 * 128);
  std::vector<double> eq(128 * 128), gcw(128);
  for (int a = 0; a < 128; a++) {
    for (int b = 0; b < 128; b++) {
      score[a * 128 + b] = (int8_t)(int)(cd.equal_amb(a, b) * 100.0 + 0.5);   // CrossCorr.cc:547-553
      eq[a * 128 + b] = cd.equal(a, b);
    }
    gcw[a] = cd.w[1][a] + cd.w[2][a];   // DNA_C + DNA_G (AlignProbability.cc:88)
  }
  XC_CHECK(cudaMalloc(&c->d_score, score.size()));
  XC_CHECK(cudaMalloc(&c->d_eq, eq.size() * sizeof(double)));
  XC_CHECK(cudaMalloc(&c->d_gcw, gcw.size() * sizeof(double)));
  XC_CHECK(cudaMemcpy(c->d_score, score.data(), score.size(), cudaMemcpyHostToDevice));
  XC_CHECK(cudaMemcpy(c->d_eq, eq.data(), eq.size() * sizeof(double), cudaMemcpyHostToDevice));
  XC_CHECK(cudaMemcpy(c->d_gcw, gcw.data(), gcw.size() * sizeof(double), cudaMemcpyHostToDevice));
  // Constant-memory codec: RC table, quarter-unit weights, double weights.
  uchar4 w4q[128];
  double wd[4 * 128];
  for (int a = 0; a < 128; a++) {
    unsigned char q[4];
    for (int ch = 0; ch < 4; ch++) {
      const double v = cd.w[ch][a] * 4.0;
      q[ch] = (v == std::floor(v)) ? (unsigned char)v : 0;   // one-third letters take the double path
      wd[ch * 128 + a] = cd.w[ch][a];
    }
    w4q[a] = make_uchar4(q[0], q[1], q[2], q[3]);
  }
  XC_CHECK(upload_constants(cd.rc, w4q, wd));
  return XC_OK;
}

// ProbTable::Setup (ProbTable.cc:15-56): 511 rows of 2047 bisection cutoffs,
// built on the host with the same double arithmetic, across host threads.
static void build_probtable(double size, std::vector<double>& tab) {
  tab.assign(512 * 2048, -1.0);
  auto raw = [size](int length, double ident, double ident_expect) {
    const double p = ident_expect;
    const double s = sqrt(p * (1. - p) * (double)length);
    const double m = p * (double)length;
    const double x = (double)length * ident;
    const double cdf = 0.5 * (1. + erf((m - x) / s / 1.414213562));
    return exp(-(cdf * size));
  };
  auto rows = [&](int lo, int hi) {
    for (int i = lo; i < hi; i++) {
      const double ie = (double)i / ((double)512 - 1);
      double* t = &tab[(size_t)i * 2048];
      t[0] = 2.;
      for (int j = 1; j < 2048; j++) {
        double mn = 0, mx = 1, mid;
        while (mx - mn > 0.00000001) {
          mid = (mx + mn) / 2.0;
          if (raw(j, mid, ie) != 0.0) mx = mid;
          else mn = mid;
        }
        t[j] = (mx + mn) / 2.0;
      }
    }
  };
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned w = 0; w < nt; w++)
    th.emplace_back(rows, 1 + (int)(511 * w / nt), 1 + (int)(511 * (w + 1) / nt));
  for (auto& t : th) t.join();
}

// ---------------------------------------------------------------------------
// Batches
// ---------------------------------------------------------------------------
static int log2_of(int L) {
  int l = 0;
  while ((1 << l) < L) l++;
  return (1 << l) == L ? l : -1;
}

int pair_log2L(const xc_params& p, const xc_pair& q) {
  int L;
  if (p.fft_len > 0) L = p.fft_len;
  else if (p.fft_len == 0) L = 2 * p.t_chunk;
  else {
    const int m = std::max(q.tlen, q.qlen);
    L = 1024;
    while (L < 2 * m) L *= 2;
  }
  return log2_of(L);
}

template <class T>
static int dev_grow(T*& ptr, size_t& cap, size_t need) {
  if (need <= cap && ptr) return XC_OK;
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  cap = 0;
  size_t n = std::max<size_t>(need, 1);
  n += n / 4;
  XC_CHECK(cudaMalloc(&ptr, n * sizeof(T)));
  cap = n;
  return XC_OK;
}

template <class T>
static int host_grow(T*& ptr, size_t& cap, size_t need) {
  if (need <= cap && ptr) return XC_OK;
  if (ptr) cudaFreeHost(ptr);
  ptr = nullptr;
  cap = 0;
  size_t n = std::max<size_t>(need, 1);
  n += n / 4;
  XC_CHECK(cudaHostAlloc(&ptr, n * sizeof(T), cudaHostAllocDefault));
  cap = n;
  return XC_OK;
}

// Worker threads kept for the host-side copies of batch_pack: the calling
// thread and up to 15 workers split one job's index range into chunks.  A
// thread that starts a job while another job runs does its own range.
class HostPool {
 public:
  static HostPool& get() {
    static HostPool* p = new HostPool();   // never destroyed: workers may outlive static destructors
    return *p;
  }
  void run(size_t n, size_t grain, const std::function<void(size_t, size_t)>& f) {
    const size_t chunks = std::min<size_t>(workers_ + 1, (n + grain - 1) / std::max<size_t>(grain, 1));
    std::unique_lock<std::mutex> busy(run_mu_, std::defer_lock);
    if (chunks <= 1 || !busy.try_lock()) {
      f(0, n);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &f;
      n_ = n;
      chunks_ = chunks;
      next_ = 0;
      left_ = chunks;
      gen_.fetch_add(1, std::memory_order_release);
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return left_ == 0; });
    job_ = nullptr;
  }

 private:
  HostPool() {
    const unsigned hc = std::thread::hardware_concurrency();
    workers_ = std::max(1u, std::min(16u, hc ? hc : 1u)) - 1;
    for (unsigned i = 0; i < workers_; i++) std::thread([this] { loop(); }).detach();
  }
  // A worker polls for the next job for a while (SPIN_US) before it sleeps:
  // the sub-batches of one call arrive a few hundred microseconds apart, and
  // a wake-up from the condition variable costs tens of microseconds.
  static constexpr int SPIN_US = 200;
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      const auto t0 = std::chrono::steady_clock::now();
      for (int i = 0; gen_.load(std::memory_order_acquire) == seen; i++) {
        if ((i & 255) == 255 &&
            std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(SPIN_US)) {
          std::unique_lock<std::mutex> lk(mu_);
          cv_.wait(lk, [&] { return gen_.load(std::memory_order_acquire) != seen; });
          break;
        }
      }
      seen = gen_.load(std::memory_order_acquire);
      work();
    }
  }
  void work() {   // takes chunks of the current job until none is left
    for (;;) {
      const std::function<void(size_t, size_t)>* f;
      size_t k, n, ch;
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (!job_ || next_ >= chunks_) return;
        k = next_++;
        f = job_;
        n = n_;
        ch = chunks_;
      }
      (*f)(n * k / ch, n * (k + 1) / ch);
      std::lock_guard<std::mutex> lk(mu_);
      if (--left_ == 0) done_cv_.notify_all();
    }
  }
  unsigned workers_ = 0;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(size_t, size_t)>* job_ = nullptr;
  size_t n_ = 0, chunks_ = 0, next_ = 0, left_ = 0;
  std::atomic<uint64_t> gen_{0};
};

static void parallel_for(size_t n, size_t grain, const std::function<void(size_t, size_t)>& f) {
  HostPool::get().run(n, grain, f);
}

Batch::~Batch() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph_exec_timed) cudaGraphExecDestroy(graph_exec_timed);
  for (auto& e : ev)
    if (e) cudaEventDestroy(e);
  if (fork_ev) cudaEventDestroy(fork_ev);
  if (join_ev) cudaEventDestroy(join_ev);
  if (side) cudaStreamDestroy(side);
  cudaFree(d_pool); cudaFree(d_desc); cudaFree(d_off); cudaFree(d_offcnt); cudaFree(d_flags);
  cudaFree(d_res); cudaFree(d_rescnt); cudaFree(d_ovf); cudaFree(d_misc); cudaFree(d_base);
  cudaFree(d_dense); cudaFree(d_dbg); cudaFree(d_dbg_sig); cudaFree(d_dbg_xc); cudaFree(d_acc); cudaFree(d_fb); cudaFree(d_fb2);
  cudaFree(d_stradcnt); cudaFree(d_strad);
  cudaFree(d_chunks); cudaFree(d_pairchunk); cudaFree(d_spec); cudaFree(d_chunkflags);
  cudaFreeHost(h_pool); cudaFreeHost(h_desc); cudaFreeHost(h_base); cudaFreeHost(h_dense);
  cudaFreeHost(h_misc); cudaFreeHost(h_ovf); cudaFreeHost(h_flags);
}

// Packs pairs into the batch's pinned staging and device buffers (async H2D
// on stream).  Pairs are bucketed by FFT length; device order = bucket order.
int batch_pack(Ctx* c, Batch* b, const xc_pair* pairs, size_t n, cudaStream_t stream) {
  if (n > (size_t)INT32_MAX / 4) return XC_ERR_ARG;
  b->n = (int)n;
  b->rb_pending = false;
  b->meta.assign(pairs, pairs + n);
  b->order.resize(n);
  b->log2L.resize(n);
  int counts[MAX_LOG2L + 1] = {0};
  for (size_t i = 0; i < n; i++) {
    const xc_pair& p = pairs[i];
    if (p.tlen < 0 || p.qlen < 0 || (p.tlen && !p.tseq) || (p.qlen && !p.qseq)) return XC_ERR_ARG;
    const int lg = pair_log2L(c->prm, p);
    if (lg < MIN_LOG2L || lg > MAX_LOG2L) return XC_ERR_UNSUPPORTED;
    if (p.tlen > (1 << lg) / 2 || p.qlen > (1 << lg) / 2) return XC_ERR_INPUT;
    b->log2L[i] = lg;
    counts[lg]++;
  }
  // bucket order; in the FFT-8192 bucket the pairs whose query is >= 1024
  // bases and not a multiple of the 16-base entropy window come last, a
  // range corr_rcq_kernel takes without the both-strands kernel
  auto ragged_q = [](const xc_pair& p) { return p.qlen >= 1024 && p.qlen % 16 != 0; };
  int ragged = 0;
  for (size_t i = 0; i < n; i++)
    if (b->log2L[i] == PAIR_LOG2L && ragged_q(pairs[i])) ragged++;
  b->ragged = ragged;
  b->buckets.clear();
  int start = 0;
  int fill[MAX_LOG2L + 1];
  int fill_ragged = 0;
  for (int lg = MIN_LOG2L; lg <= MAX_LOG2L; lg++) {
    fill[lg] = start;
    if (lg == PAIR_LOG2L) fill_ragged = start + counts[lg] - ragged;
    if (counts[lg]) b->buckets.push_back({lg, start, counts[lg]});
    start += counts[lg];
  }
  for (size_t i = 0; i < n; i++) {
    const int lg = b->log2L[i];
    b->order[lg == PAIR_LOG2L && ragged_q(pairs[i]) ? fill_ragged++ : fill[lg]++] = (int)i;
  }
  if (b->buckets.size() > 1 && !b->side) {   // made here, outside any stream capture
    XC_CHECK(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
    XC_CHECK(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
    XC_CHECK(cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming));
  }
  // pool and offset-list layout; a chunk that several pairs pass by the same
  // pointer and length (a block's target and query chunks) is stored once.
  // The distinct chunks of the FFT-8192 bucket are numbered as they appear
  // (the spectra path's chunk table; every empty chunk is one entry).
  std::vector<uint64_t> toff(n), qoff(n);
  uint64_t pool = 0, offl = 0;
  b->desc_host.resize(n);
  struct Src {
    const char* p;
    int len;
    uint64_t off;
    int cid;   // chunk index in the FFT-8192 bucket's table, -1 before its first use there
  };
  std::vector<Src> uniq;
  uniq.reserve(2 * n);
  size_t hsize = 16;
  while (hsize < 4 * n) hsize *= 2;
  b->ht.assign(hsize, HashSlot{nullptr, 0, 0});   // open addressing, linear probing
  const bool want_spec = c->pair_kernel && c->spec_reuse;
  b->chunk_host.clear();
  b->pair_chunk_host.assign(want_spec ? 2 * (size_t)n : 0, 0);
  int empty_cid = -1;
  auto place = [&](const char* ptr, int len, bool bucket8192, int* cid) -> uint64_t {
    if (len == 0) {
      if (bucket8192) {
        if (empty_cid < 0) {
          empty_cid = (int)b->chunk_host.size();
          b->chunk_host.push_back({(uint32_t)0, 0});
        }
        *cid = empty_cid;
      }
      return pool;
    }
    size_t h = (((uint64_t)(uintptr_t)ptr * 0x9E3779B97F4A7C15ull) ^ (uint64_t)len * 0xC2B2AE3D27D4EB4Full) >> 20;
    int u = -1;
    for (;; h++) {
      HashSlot& sl = b->ht[h & (hsize - 1)];
      if (!sl.p) {   // new chunk
        u = (int)uniq.size();
        sl.p = ptr;
        sl.len = len;
        sl.uid = (uint32_t)u;
        uniq.push_back({ptr, len, pool, -1});
        pool += ((uint64_t)len + 15) & ~15ull;
        break;
      }
      if (sl.p == ptr && sl.len == len) {
        u = (int)sl.uid;
        break;
      }
    }
    Src& e = uniq[u];
    if (bucket8192) {
      if (e.cid < 0) {
        e.cid = (int)b->chunk_host.size();
        b->chunk_host.push_back({(uint32_t)e.off, len});
      }
      *cid = e.cid;
    }
    return e.off;
  };
  for (size_t d = 0; d < n; d++) {
    const xc_pair& p = pairs[b->order[d]];
    const int lg = b->log2L[b->order[d]];
    const bool sp = want_spec && lg == PAIR_LOG2L;
    int ct = 0, cq = 0;
    toff[d] = place(p.tseq, p.tlen, sp, &ct);
    qoff[d] = place(p.qseq, p.qlen, sp, &cq);
    if (sp) {
      b->pair_chunk_host[2 * d] = ct;
      b->pair_chunk_host[2 * d + 1] = cq;
    }
    PairDesc& D = b->desc_host[d];
    D.t_off = (uint32_t)toff[d];
    D.q_off = (uint32_t)qoff[d];
    D.tlen = p.tlen;
    D.qlen = p.qlen;
    D.log2L = lg;
    D.flags = p.fast ? PF_FAST : 0u;
    D.off_base = (uint32_t)offl;
    D.pad = 0;
    offl += 2ull << lg;
  }
  if (pool >= (1ull << 32) || offl >= (1ull << 32)) return XC_ERR_ARG;
  const size_t nslots = 2 * n;
  const size_t slots = (size_t)b->slots;
  int r;
  if ((r = host_grow(b->h_pool, b->cap_h_pool, pool + 16)) != XC_OK) return r;
  if ((r = host_grow(b->h_desc, b->cap_h_desc, n)) != XC_OK) return r;
  if ((r = dev_grow(b->d_pool, b->cap_pool, pool + 16)) != XC_OK) return r;
  if ((r = dev_grow(b->d_desc, b->cap_desc, n)) != XC_OK) return r;
  if ((r = dev_grow(b->d_off, b->cap_off, offl)) != XC_OK) return r;
  if ((r = dev_grow(b->d_offcnt, b->cap_offcnt, nslots)) != XC_OK) return r;
  if ((r = dev_grow(b->d_flags, b->cap_flags, n)) != XC_OK) return r;
  if ((r = dev_grow(b->d_res, b->cap_res, nslots * slots)) != XC_OK) return r;
  if ((r = dev_grow(b->d_rescnt, b->cap_rescnt, nslots)) != XC_OK) return r;
  if ((r = dev_grow(b->d_ovf, b->cap_ovf, (size_t)b->ovf_cap)) != XC_OK) return r;
  if ((r = dev_grow(b->d_misc, b->cap_misc, 8)) != XC_OK) return r;
  if ((r = dev_grow(b->d_fb, b->cap_fb, n)) != XC_OK) return r;
  if ((r = dev_grow(b->d_fb2, b->cap_fb2, n)) != XC_OK) return r;   // sized for any later batch of n
  if ((r = dev_grow(b->d_stradcnt, b->cap_stradcnt, nslots)) != XC_OK) return r;
  if ((r = dev_grow(b->d_strad, b->cap_strad, nslots * STRAD_CAP)) != XC_OK) return r;
  if ((r = dev_grow(b->d_base, b->cap_base, nslots + 1)) != XC_OK) return r;
  if ((r = dev_grow(b->d_dense, b->cap_dense, nslots * slots)) != XC_OK) return r;
  size_t acc = 0;
  for (int lg = MAX_SMEM_LOG2L + 1; lg <= MAX_LOG2L; lg++) acc = std::max(acc, (size_t)counts[lg] * 2 * acc_stride(lg));
  if (acc && (r = dev_grow(b->d_acc, b->cap_acc, acc)) != XC_OK) return r;
  if ((r = host_grow(b->h_base, b->cap_h_base, nslots + 1)) != XC_OK) return r;
  if ((r = host_grow(b->h_misc, b->cap_h_misc, 4)) != XC_OK) return r;
  b->pool_bytes = pool;
  b->unique_bytes = pool;
  // gather the distinct chunks into pinned staging (threads for large batches)
  uint8_t* hp = b->h_pool;
  parallel_for(uniq.size(), 128, [&](size_t lo, size_t hi) {   // chunks of >= 128 chunks (0.5 MB)
    for (size_t u = lo; u < hi; u++) memcpy(hp + uniq[u].off, uniq[u].p, (size_t)uniq[u].len);
  });
  memcpy(b->h_desc, b->desc_host.data(), n * sizeof(PairDesc));
  XC_CHECK(cudaMemcpyAsync(b->d_pool, b->h_pool, pool, cudaMemcpyHostToDevice, stream));
  XC_CHECK(cudaMemcpyAsync(b->d_desc, b->h_desc, n * sizeof(PairDesc), cudaMemcpyHostToDevice, stream));
  b->h2d_bytes = pool + n * sizeof(PairDesc);
  // spectra path for the FFT-8192 bucket when its pairs share chunks
  b->spec = false;
  b->spec_chunks = 0;
  for (const Bucket& bk : b->buckets) {
    if (bk.log2L != PAIR_LOG2L || !want_spec) continue;
    const size_t U = b->chunk_host.size();
    if ((double)(2 * bk.count) < SPEC_MIN_REUSE * (double)U) continue;
    if ((r = dev_grow(b->d_chunks, b->cap_chunks, U)) != XC_OK) return r;
    if ((r = dev_grow(b->d_pairchunk, b->cap_pairchunk, 2 * (size_t)n)) != XC_OK) return r;
    if ((r = dev_grow(b->d_spec, b->cap_spec, U * (spec_bytes_per_chunk() / sizeof(float2)))) != XC_OK) return r;
    if ((r = dev_grow(b->d_chunkflags, b->cap_chunkflags, U)) != XC_OK) return r;
    XC_CHECK(cudaMemcpyAsync(b->d_chunks, b->chunk_host.data(), U * sizeof(ChunkDesc), cudaMemcpyHostToDevice,
                             stream));
    XC_CHECK(cudaMemcpyAsync(b->d_pairchunk, b->pair_chunk_host.data(), 2 * (size_t)n * sizeof(int),
                             cudaMemcpyHostToDevice, stream));
    b->h2d_bytes += U * sizeof(ChunkDesc) + 2 * (size_t)n * sizeof(int);
    b->spec = true;
    b->spec_chunks = (int)U;
  }
  b->graph_valid = false;
  b->graph_timed_valid = false;
  return XC_OK;
}

// z-score threshold of the scan kernel's FP32 screen.  A segment is kept when
// exp(-Phi(z) * targetTotal) >= min_prob, z = (pm*N - hits) / sd
// (AlignProbability.cc:107-125), i.e. when Phi(z) <= -log(min_prob) /
// targetTotal, i.e. z <= z*.  z* comes from bisection on the normal CDF in
// double, with the bound raised by 1% and by 4.5e-16 -- the reference forms
// Phi as 0.5 * (1 + erf(.)), which loses everything below ~1e-16 to
// cancellation, so its exact test accepts up to that much beyond the true CDF.
// The kernel rejects only above z* + 0.02, orders of magnitude beyond the
// FP32 error of its z; survivors take the exact FP64 test.
float screen_z(double min_prob, double target_total) {
  if (!(min_prob > 0) || !(target_total > 0)) return INFINITY;
  const double bound = -log(min_prob);
  if (!(bound >= 0)) return -INFINITY;   // min_prob > 1: nothing passes the exact test either
  const double r = bound / target_total * 1.01 + 4.5e-16;
  if (r >= 1.0) return INFINITY;
  double lo = -60.0, hi = 60.0;          // Phi(lo) < r <= Phi(hi) for every r the doubles reach
  for (int it = 0; it < 200; it++) {
    const double mid = 0.5 * (lo + hi);
    if (0.5 * erfc(-mid / sqrt(2.0)) <= r) lo = mid; else hi = mid;
  }
  return (float)(hi + 0.02);
}

// Floors of the scan kernel's in-word runs.  A run of r passing checks
// (r = 1..32) makes a segment of N = r + 45 bases with h equal bases; equal
// bases agree in G+C, so the two sequences' G+C counts differ by at most
// N - h, and pm = (gT gQ + (N-gT)(N-gQ)) / 2N^2 >= (1 - m^2) / 4 with
// m = 1 - h/N (the minimum over that band).  For pm <= 1/2 and pm N < h,
// z = (pm N - h) / sqrt(pm (1 - pm) N) grows with pm, so z >= z_min(h, N)
// at pm = (1 - m^2) / 4.  Byte r-1 of out is the least h with
// z_min(h, N) <= screen_z (+1e-6); every h below it has z > screen_z for
// every composition, which the screen rejects (and the exact test after it).
// Segments shorter than min_len get 255.  Zeros (no floor) when the screen
// keeps everything or is not negative.  Returns the least floor.
int run_hits_floor(float screen_z, int min_len, uint32_t out[8]) {
  for (int k = 0; k < 8; k++) out[k] = 0u;
  if (!(screen_z < 0.f) || !std::isfinite(screen_z)) return 0;
  int least = 255;
  const double sz = (double)screen_z + 1e-6;
  for (int r = 1; r <= 32; r++) {
    const int n = r + 45;
    int floor_h = n + 1;
    for (int h = 1; h <= n; h++) {
      const double m = 1.0 - (double)h / n;
      const double p = (1.0 - m * m) / 4.0;
      const double z = p * n >= h ? 0.0 : (p * n - h) / sqrt(p * (1.0 - p) * n);
      if (z <= sz) {
        floor_h = h;
        break;
      }
    }
    if (n < min_len) floor_h = 255;
    floor_h = std::min(floor_h, 255);
    least = std::min(least, floor_h);
    out[(r - 1) >> 2] |= (uint32_t)floor_h << (8 * ((r - 1) & 3));
  }
  return least;
}


// Enqueues the kernels of one batch on stream.
static int batch_enqueue(Ctx* c, Batch* b, cudaStream_t s, bool timed) {
  const int nslots = 2 * b->n;
  // stage events: external event nodes inside a graph capture, plain records otherwise
  cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
  if (timed) XC_CHECK(cudaStreamIsCapturing(s, &cst));
  const unsigned evflags = cst == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
  XC_CHECK(cudaMemsetAsync(b->d_misc, 0, 8 * sizeof(int), s));   // counters, error words, work counters
  XC_CHECK(cudaMemsetAsync(b->d_stradcnt, 0, nslots * sizeof(int), s));
  if (timed) XC_CHECK(cudaEventRecordWithFlags(b->ev[0], s, evflags));
  auto corr_bucket = [&](const Bucket& bk, cudaStream_t st) -> int {
    const DevTables& t = c->tab[bk.log2L];
    CorrParams cp{};
    cp.pairs = b->d_desc;
    cp.pool = b->d_pool;
    cp.first = bk.first;
    const int NH = (1 << (bk.log2L - 1)) / 64;
    cp.tab.twN_hi = t.tw;
    cp.tab.twN_lo = t.tw + NH;
    cp.tab.twL_hi = t.tw + NH + 64;
    cp.tab.twL_lo = t.tw + 2 * NH + 64;
    cp.tab.ent = t.ent;
    cp.tab.ent_acgt = t.ent_acgt;
    cp.cutoff = c->prm.cutoff;
    cp.cutoff_fast = c->prm.cutoff_fast;
    cp.off_list = b->d_off;
    cp.off_cnt = b->d_offcnt;
    cp.pair_flags = b->d_flags;
    cp.dbg_sig = b->d_dbg_sig;
    cp.dbg_xc = b->d_dbg_xc;
    cp.acc = b->d_acc;
    cp.work = b->d_misc + 4;   // zeroed above; one FFT-8192 bucket per batch
    if (bk.log2L == PAIR_LOG2L && c->pair_kernel) {
      cp.fb_list = b->d_fb;
      cp.fb_cnt = b->d_misc + 3;   // zeroed above
      cp.pair_form = c->pair_form;
      if (c->pair_form == 2 && b->ragged) {
        if (b->spec) {   // the spectra kernel hands them on by their chunk flags
          cp.fb2_list = b->d_fb2;
          cp.fb2_cnt = b->d_misc + 6;   // zeroed above
        } else if (!b->d_dbg_sig) {   // the bucket's last pairs (signal output: the per-strand kernel)
          cp.rcq_first = bk.first + bk.count - b->ragged;
          cp.rcq_count = b->ragged;
        }
      }
    }
    cp.strand_threads = c->strand_threads[bk.log2L];
    cp.strad_cnt = b->d_stradcnt;
    cp.strad_list = b->d_strad;
    if (bk.log2L == PAIR_LOG2L && b->spec) {
      SpecParams spp{};
      spp.chunks = b->d_chunks;
      spp.count = b->spec_chunks;
      spp.pool = b->d_pool;
      spp.tab = cp.tab;
      spp.spec = b->d_spec;
      spp.chunk_flags = b->d_chunkflags;
      spp.work = b->d_misc + 5;
      cp.pair_chunk = b->d_pairchunk;
      cp.spec = b->d_spec;
      cp.chunk_flags = b->d_chunkflags;
      XC_CHECK(launch_corr_spec(spp, cp, bk.count, st));
      return XC_OK;
    }
    XC_CHECK(launch_corr(bk.log2L, cp, bk.count, st));
    return XC_OK;
  };
  auto scan_bucket = [&](const Bucket& bk, cudaStream_t st) -> int {
    ScanParams sp{};
    sp.pairs = b->d_desc;
    sp.pool = b->d_pool;
    sp.first = bk.first;
    sp.off_list = b->d_off;
    sp.off_cnt = b->d_offcnt;
    sp.pair_flags = b->d_flags;
    sp.score = c->d_score;
    sp.eq = c->d_eq;
    sp.gcw = c->d_gcw;
    sp.ptable = c->prm.use_prob_table ? c->d_ptable : nullptr;
    sp.ptable_cutoff = c->prm.prob_table_cutoff;
    sp.min_prob = c->prm.min_prob;
    sp.target_total = c->prm.target_total;
    sp.screen_z = screen_z(c->prm.min_prob, c->prm.target_total);
    sp.min_len = c->prm.min_len;
    sp.slots = b->slots;
    sp.res = b->d_res;
    sp.res_cnt = b->d_rescnt;
    sp.ovf = b->d_ovf;
    sp.ovf_cnt = b->d_misc + 0;
    sp.ovf_cap = b->ovf_cap;
    sp.err = b->d_misc + 1;
    sp.dbg = b->d_dbg;
    sp.dbg_cnt = b->d_misc + 2;
    sp.dbg_cap = b->dbg_cap;
    if (!sp.dbg && !sp.ptable) sp.word_floor = run_hits_floor(sp.screen_z, sp.min_len, sp.run_floor);
    XC_CHECK(launch_scan(bk.log2L, sp, bk.count, st));
    return XC_OK;
  };
  int r;
  const bool multi = b->buckets.size() > 1 && b->side;
  if (multi && !timed) {
    // Buckets are independent: each runs its correlation and then its scan,
    // the FFT-8192 bucket (or else the largest) on s and the others beside
    // it on the batch's side stream (small launches leave most SMs idle),
    // joined before the finalize kernels.
    const Bucket* main_bk = nullptr;
    for (const Bucket& bk : b->buckets)
      if (bk.log2L == PAIR_LOG2L) main_bk = &bk;
    if (!main_bk)
      for (const Bucket& bk : b->buckets)
        if (!main_bk || bk.count > main_bk->count) main_bk = &bk;
    XC_CHECK(cudaEventRecord(b->fork_ev, s));
    XC_CHECK(cudaStreamWaitEvent(b->side, b->fork_ev, 0));
    for (const Bucket& bk : b->buckets) {
      if (&bk == main_bk) continue;
      if ((r = corr_bucket(bk, b->side)) != XC_OK) return r;
      if ((r = scan_bucket(bk, b->side)) != XC_OK) return r;
    }
    if ((r = corr_bucket(*main_bk, s)) != XC_OK) return r;
    if ((r = scan_bucket(*main_bk, s)) != XC_OK) return r;
    XC_CHECK(cudaEventRecord(b->join_ev, b->side));
    XC_CHECK(cudaStreamWaitEvent(s, b->join_ev, 0));
  } else {
    // timed: the stages one after another, so that the stage events bracket
    // them; the buckets' scans still run beside one another
    for (const Bucket& bk : b->buckets)
      if ((r = corr_bucket(bk, s)) != XC_OK) return r;
    if (timed) XC_CHECK(cudaEventRecordWithFlags(b->ev[1], s, evflags));
    const Bucket* big = nullptr;
    for (const Bucket& bk : b->buckets)
      if (!big || bk.count > big->count) big = &bk;
    if (multi) {
      XC_CHECK(cudaEventRecord(b->fork_ev, s));
      XC_CHECK(cudaStreamWaitEvent(b->side, b->fork_ev, 0));
    }
    for (const Bucket& bk : b->buckets)
      if ((r = scan_bucket(bk, multi && &bk != big ? b->side : s)) != XC_OK) return r;
    if (multi) {
      XC_CHECK(cudaEventRecord(b->join_ev, b->side));
      XC_CHECK(cudaStreamWaitEvent(s, b->join_ev, 0));
    }
  }
  if (timed) XC_CHECK(cudaEventRecordWithFlags(b->ev[2], s, evflags));
  XC_CHECK(launch_finalize(b->d_rescnt, b->d_res, b->slots, nslots, b->d_base, b->d_dense, nullptr, s));
  if (timed) XC_CHECK(cudaEventRecordWithFlags(b->ev[3], s, evflags));
  return XC_OK;
}

int batch_launch_count(const Ctx* c, const Batch* b) {
  int n = 2 * (int)b->buckets.size() + 2;
  for (const Bucket& bk : b->buckets)
    if (bk.log2L == PAIR_LOG2L && c->pair_kernel) {
      n += b->spec ? 2 : 1;   // (spectra,) pair kernel, hand-back
      if (c->pair_form == 2 && b->ragged) {
        n++;   // ragged query windows
        if (!b->spec && b->d_dbg_sig) n--;                         // ragged pairs handed back instead
        else if (!b->spec && b->ragged == bk.count) n--;   // no pair for the both-strands kernel
      }
    }
  return n;
}

// Runs the batch; replays a captured CUDA graph when the batch is unchanged.
int batch_run(Ctx* c, Batch* b, cudaStream_t s, bool use_graph, bool timed) {
  if (timed)
    for (auto& e : b->ev)
      if (!e) XC_CHECK(cudaEventCreate(&e));
  if (!use_graph || b->d_dbg || b->d_dbg_sig || b->d_dbg_xc) return batch_enqueue(c, b, s, timed);
  cudaGraphExec_t& ge = timed ? b->graph_exec_timed : b->graph_exec;
  bool& valid = timed ? b->graph_timed_valid : b->graph_valid;
  cudaStream_t& gs = timed ? b->graph_timed_stream : b->graph_stream;
  if (!valid || gs != s) {
    if (ge) cudaGraphExecDestroy(ge);
    ge = nullptr;
    cudaGraph_t g;
    XC_CHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int r = batch_enqueue(c, b, s, timed);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (r != XC_OK) return r;
    XC_CHECK(e);
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    XC_CHECK(e);
    valid = true;
    gs = s;
  }
  XC_CHECK(cudaGraphLaunch(ge, s));
  return XC_OK;
}

int batch_readback_async(Ctx* c, Batch* b, cudaStream_t s) {
  (void)c;
  const int n = b->n, nslots = 2 * n;
  int r;
  if ((r = host_grow(b->h_base, b->cap_h_base, (size_t)nslots + 1)) != XC_OK) return r;
  if ((r = host_grow(b->h_misc, b->cap_h_misc, 4)) != XC_OK) return r;
  if ((r = host_grow(b->h_flags, b->cap_h_flags, (size_t)n)) != XC_OK) return r;
  size_t est = std::max(b->est_dense, (size_t)4 * n);
  est = std::min(est, b->cap_dense);
  if ((r = host_grow(b->h_dense, b->cap_h_dense, est + 1)) != XC_OK) return r;
  XC_CHECK(cudaMemcpyAsync(b->h_base, b->d_base, (nslots + 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
  XC_CHECK(cudaMemcpyAsync(b->h_misc, b->d_misc, 4 * sizeof(int), cudaMemcpyDeviceToHost, s));
  XC_CHECK(cudaMemcpyAsync(b->h_flags, b->d_flags, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  if (est) XC_CHECK(cudaMemcpyAsync(b->h_dense, b->d_dense, est * sizeof(DevResult), cudaMemcpyDeviceToHost, s));
  b->pre_dense = est;
  b->rb_pending = true;
  return XC_OK;
}

// Reads results back and assembles xc_result records in original pair order.
int batch_collect(Ctx* c, Batch* b, cudaStream_t s, xc_result* out, size_t cap, size_t* n_out,
                  size_t* pair_counts) {
  const int n = b->n, nslots = 2 * n;
  int r;
  if (!b->rb_pending && (r = batch_readback_async(c, b, s)) != XC_OK) return r;
  XC_CHECK(cudaStreamSynchronize(s));
  b->rb_pending = false;
  const int total = b->h_base[nslots];
  const int novf = b->h_misc[0];
  const int err = b->h_misc[1];
  uint64_t d2h = (uint64_t)(nslots + 1) * sizeof(int) + 4 * sizeof(int) + (uint64_t)n * sizeof(uint32_t) +
                 (uint64_t)b->pre_dense * sizeof(DevResult);
  if (err & 1) return XC_INTERNAL_OVERFLOW;   // the caller grows the pool and runs the batch again
  if (err & 4) {
    fprintf(stderr, "satsuma2_gb300: scan kernel: inconsistent segment bounds\n");
    return XC_ERR_CUDA;
  }
  b->est_dense = (size_t)total + (size_t)total / 4;
  const bool again = (size_t)total > b->pre_dense;   // the estimate fell short: read all of them
  if (again) {
    if ((r = host_grow(b->h_dense, b->cap_h_dense, (size_t)total + 1)) != XC_OK) return r;
    XC_CHECK(cudaMemcpyAsync(b->h_dense, b->d_dense, total * sizeof(DevResult), cudaMemcpyDeviceToHost, s));
    d2h += (uint64_t)total * sizeof(DevResult);
  }
  std::vector<DevResultX> ovf;
  if (novf > 0) {
    ovf.resize(novf);
    XC_CHECK(cudaMemcpyAsync(ovf.data(), b->d_ovf, novf * sizeof(DevResultX), cudaMemcpyDeviceToHost, s));
    d2h += (uint64_t)novf * sizeof(DevResultX);
  }
  if (again || novf > 0) XC_CHECK(cudaStreamSynchronize(s));
  b->d2h_bytes = d2h;
  c->last_h2d = b->h2d_bytes;
  c->last_d2h = b->d2h_bytes;
  for (int d = 0; d < n; d++)
    if (b->h_flags[d] & PF_INVALID) return XC_ERR_INPUT;
  // per slot record lists of the overflow pool (device order)
  std::vector<std::vector<DevResult>> extra;
  std::vector<int> extra_of;
  if (novf > 0) {
    extra_of.assign(nslots, -1);
    for (const DevResultX& x : ovf) {
      if (extra_of[x.slot] < 0) {
        extra_of[x.slot] = (int)extra.size();
        extra.emplace_back();
      }
      extra[extra_of[x.slot]].push_back(x.r);
    }
  }
  // counts per original pair
  std::vector<size_t> cnt(n, 0);
  std::vector<int> dev_of(n);
  for (int d = 0; d < n; d++) dev_of[b->order[d]] = d;
  size_t need = 0;
  for (int i = 0; i < n; i++) {
    const int d = dev_of[i];
    for (int s2 = 0; s2 < 2; s2++) {
      const int sl = 2 * d + s2;
      size_t k = (size_t)(b->h_base[sl + 1] - b->h_base[sl]);
      if (novf > 0 && extra_of[sl] >= 0) k += extra[extra_of[sl]].size();
      cnt[i] += k;
    }
    need += cnt[i];
  }
  if (n_out) *n_out = need;
  if (pair_counts)
    for (int i = 0; i < n; i++) pair_counts[i] = cnt[i];
  if (need > cap || (!out && need)) return XC_ERR_CAPACITY;
  // each pair's records from its output offset; pair ranges in parallel when
  // there are many records
  std::vector<size_t> first(n + 1, 0);
  for (int i = 0; i < n; i++) first[i + 1] = first[i] + cnt[i];
  const int qchunk = c->prm.q_chunk;
  auto convert = [&](size_t lo_pair, size_t hi_pair) {
    std::vector<DevResult> merged;
    for (size_t i = lo_pair; i < hi_pair; i++) {
      size_t o = first[i];
      const int d = dev_of[i];
      const xc_pair& p = b->meta[i];
      for (int s2 = 0; s2 < 2; s2++) {
        const int sl = 2 * d + s2;
        const DevResult* rec = b->h_dense + b->h_base[sl];
        size_t nrec = (size_t)(b->h_base[sl + 1] - b->h_base[sl]);
        if (novf > 0 && extra_of[sl] >= 0) {   // slot records plus its overflow records, reordered
          const auto& e = extra[extra_of[sl]];
          merged.assign(rec, rec + nrec);
          merged.insert(merged.end(), e.begin(), e.end());
          std::sort(merged.begin(), merged.end(), [](const DevResult& a, const DevResult& q) {
            return a.key < q.key || (a.key == q.key && a.tstart < q.tstart);
          });
          rec = merged.data();
          nrec = merged.size();
        }
        for (size_t j = 0; j < nrec; j++) {
          const DevResult& rr = rec[j];
          xc_result& x = out[o++];
          memset(&x, 0, sizeof(x));
          // FilterMatches coordinate mapping (HomologyByXCorrSlave.cc:175-181, RCQuery :56-60)
          const int tStart = p.t_chunk_start + rr.tstart;
          const int qStart = s2 == 0 ? p.q_chunk_start + rr.qstart
                                     : rr.qstart + (int)p.query_size - p.q_chunk_start - qchunk;
          x.query_id = p.query_id;
          x.target_id = p.target_id;
          x.query_size = p.query_size;
          x.qstart = (unsigned long)(long)qStart;
          x.tstart = (unsigned long)(long)tStart;
          x.len = (unsigned long)(long)rr.len;
          x.reverse = (unsigned char)s2;
          x.prob = rr.prob;
          x.ident = rr.ident;
        }
      }
    }
  };
  if (need >= 4096)
    parallel_for((size_t)n, 64, convert);
  else
    convert(0, (size_t)n);
  return XC_OK;
}

int batch_rerun_overflow(Ctx* c, Batch* b, cudaStream_t s, xc_result* out, size_t cap, size_t* n_out,
                         size_t* pair_counts) {
  for (int attempt = 0; attempt < 3; attempt++) {
    // the scan kernel counts every record it could not place, so the pool
    // grows to at least what this run asked for; the captured graphs hold the
    // old pool and capacity in their launch parameters
    b->ovf_cap = std::max(b->ovf_cap * 4, b->h_misc[0] + 1024);
    b->graph_valid = false;
    b->graph_timed_valid = false;
    int r = dev_grow(b->d_ovf, b->cap_ovf, (size_t)b->ovf_cap);
    if (r != XC_OK) return r;
    if ((r = batch_run(c, b, s, false)) != XC_OK) return r;
    r = batch_collect(c, b, s, out, cap, n_out, pair_counts);
    if (r != XC_INTERNAL_OVERFLOW) return r;
  }
  fprintf(stderr, "satsuma2_gb300: result overflow pool still full after three runs\n");
  return XC_ERR_NOMEM;
}

// xc_align_pairs: the pairs run as sub-batches alternating between two
// batches and two streams, so the host packing and the host-to-device copy of
// one sub-batch overlap the kernels of the one before; results are collected
// in order.  Sub-batch sizes count in waves of the FFT-8192 correlation kernel
// (one CTA per SM): a first one of 4 waves so the GPU starts early, then
// equal ones of at most 12 waves and max_batch pairs.  On GB300 a 4096-pair
// call took 2.28 ms as 456 + 2 x 1820 pairs, 2.57 ms as 512 + 4 x 896 and
// 2.59 ms in one batch; after the kernels got faster the host's packing of
// the second sub-batch outlasted a 3-wave first one on the GPU, and 608 +
// 2 x 1744 took 1.53 ms against 1.55-1.57 ms as 456 + 2 x 1820.
int ctx_align_pipelined(Ctx* c, const xc_pair* pairs, size_t n, xc_result* out, size_t cap, size_t* n_out,
                        size_t* pair_counts) {
  const size_t maxb = c->prm.max_batch > 0 ? (size_t)c->prm.max_batch : 4096;
  const size_t first = std::min(maxb, (size_t)4 * c->sms), size = std::min(maxb, (size_t)12 * c->sms);
  std::vector<size_t> bound{0};
  if (n <= 2 * first && n <= maxb) {
    bound.push_back(n);
  } else {
    bound.push_back(first);
    const size_t rest = n - first;
    const size_t parts = (rest + size - 1) / size;
    for (size_t i = 1; i <= parts; i++) bound.push_back(first + rest * i / parts);
  }
  const size_t nchunks = bound.size() - 1;
  size_t written = 0, need = 0;
  uint64_t h2d = 0, d2h = 0;
  bool full = false;   // output capacity exceeded: later sub-batches are only counted
  auto start = [&](size_t k) -> int {
    const size_t lo = bound[k], m = bound[k + 1] - lo;
    Batch* b = c->work[k & 1];
    const cudaStream_t s = c->work_stream[k & 1];
    int r = batch_pack(c, b, pairs + lo, m, s);
    if (r == XC_OK) r = batch_run(c, b, s, false);
    if (r == XC_OK) r = batch_readback_async(c, b, s);
    return r;
  };
  auto finish = [&](size_t k) -> int {
    const size_t lo = bound[k];
    Batch* b = c->work[k & 1];
    xc_result* o = (full || !out) ? nullptr : out + written;
    const size_t cp = full ? 0 : (cap >= written ? cap - written : 0);
    size_t got = 0;
    int r = batch_collect(c, b, c->work_stream[k & 1], o, cp, &got, pair_counts ? pair_counts + lo : nullptr);
    if (r == XC_INTERNAL_OVERFLOW)   // device overflow pool too small: grow it, run the sub-batch again
      r = batch_rerun_overflow(c, b, c->work_stream[k & 1], o, cp, &got, pair_counts ? pair_counts + lo : nullptr);
    need += got;
    h2d += c->last_h2d;
    d2h += c->last_d2h;
    if (r == XC_ERR_CAPACITY) {
      full = true;
      return XC_OK;
    }
    if (r != XC_OK) return r;
    written += got;
    return XC_OK;
  };
  int r = XC_OK;
  size_t k = 0, done = 0;
  for (; k < nchunks && r == XC_OK; k++) {
    if (k >= 2) r = finish(done++);
    if (r == XC_OK) r = start(k);
  }
  while (r == XC_OK && done < k) r = finish(done++);
  if (r != XC_OK) {
    for (int i = 0; i < 2; i++) cudaStreamSynchronize(c->work_stream[i]);
    return r;
  }
  c->last_h2d = h2d;
  c->last_d2h = d2h;
  if (n_out) *n_out = need;
  return full ? XC_ERR_CAPACITY : XC_OK;
}

Batch* new_batch(Ctx* c) {
  Batch* b = new Batch();
  b->slots = c->prm.result_slots > 0 ? c->prm.result_slots : 64;
  b->ovf_cap = 1 << 16;
  return b;
}

}  // namespace xc

using namespace xc;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

extern "C" {

const char* xc_version(void) { return "satsuma2_gb300 1.0 (sm_103a)"; }

int xc_create(const xc_params* params, int device, xc_ctx** out) {
  if (!params || !out) return XC_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return XC_ERR_CUDA;
  xc_ctx* c = new xc_ctx();
  c->prm = *params;
  if (c->prm.t_chunk <= 0) c->prm.t_chunk = 4096;
  if (c->prm.q_chunk <= 0) c->prm.q_chunk = 4096;
  c->device = device;
  int r = cuda_err(cudaSetDevice(device), "cudaSetDevice");
  if (r == XC_OK) r = cuda_err(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device), "SM count");
  if (r == XC_OK) r = cuda_err(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
  if (r == XC_OK) r = cuda_err(prepare_kernels(), "kernel attributes");
  if (r == XC_OK) r = build_tables(c);
  if (r == XC_OK && c->prm.use_prob_table) {
    build_probtable(c->prm.target_total, c->h_ptable);
    r = cuda_err(cudaMalloc(&c->d_ptable, c->h_ptable.size() * sizeof(double)), "probtable");
    if (r == XC_OK)
      r = cuda_err(cudaMemcpy(c->d_ptable, c->h_ptable.data(), c->h_ptable.size() * sizeof(double),
                              cudaMemcpyHostToDevice), "probtable copy");
  }
  if (r == XC_OK) {
    // a tuning table written by xc_tune, when SATSUMA2_GB300_TUNING names one
    const char* tf = getenv("SATSUMA2_GB300_TUNING");
    if (tf && tf[0]) {
      FILE* f = fopen(tf, "r");
      if (f) {
        std::string text;
        char buf[4096];
        size_t k;
        while ((k = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, k);
        fclose(f);
        r = apply_tuning_text(c, text.c_str());
      }
    }
  }
  if (r == XC_OK) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) snprintf(c->devname, sizeof(c->devname), "%s", prop.name);
    for (int i = 0; i < 2 && r == XC_OK; i++) {
      c->work[i] = new_batch(c);
      r = cuda_err(cudaStreamCreateWithFlags(&c->work_stream[i], cudaStreamNonBlocking), "stream");
    }
  }
  if (r != XC_OK) {
    xc_destroy(c);
    return r;
  }
  *out = c;
  return XC_OK;
}

int xc_destroy(xc_ctx* c) {
  if (!c) return XC_ERR_ARG;
  server_stop(c);
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (int i = 0; i < 2; i++) {
    if (c->work_stream[i]) cudaStreamSynchronize(c->work_stream[i]);
    delete c->work[i];
    if (c->work_stream[i]) cudaStreamDestroy(c->work_stream[i]);
  }
  for (auto& t : c->tab) {
    cudaFree(t.tw); cudaFree(t.ent); cudaFree(t.ent_acgt);
  }
  cudaFree(c->d_score); cudaFree(c->d_eq); cudaFree(c->d_gcw); cudaFree(c->d_ptable);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return XC_OK;
}

int xc_align_pairs(xc_ctx* c, const xc_pair* pairs, size_t n, xc_result* out, size_t cap, size_t* n_out,
                   size_t* pair_counts) {
  if (!c || (!pairs && n)) return XC_ERR_ARG;
  if (n_out) *n_out = 0;
  if (n == 0) return XC_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  return ctx_align_pipelined(c, pairs, n, out, cap, n_out, pair_counts);
}

int xc_batch_upload(xc_ctx* c, const xc_pair* pairs, size_t n, xc_batch** out) {
  if (!c || !out || (!pairs && n) || n == 0) return XC_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  xc_batch* b = new xc_batch();
  b->slots = c->prm.result_slots > 0 ? c->prm.result_slots : 64;
  b->ovf_cap = 1 << 16;
  int r = batch_pack(c, b, pairs, n, c->stream);
  if (r == XC_OK) r = cuda_err(cudaStreamSynchronize(c->stream), "upload");
  if (r != XC_OK) {
    delete b;
    return r;
  }
  *out = b;
  return XC_OK;
}

int xc_batch_run(xc_ctx* c, xc_batch* b, void* stream) {
  if (!c || !b) return XC_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  return batch_run(c, b, s, true);
}

int xc_batch_results(xc_ctx* c, xc_batch* b, xc_result* out, size_t cap, size_t* n_out, size_t* pair_counts) {
  if (!c || !b) return XC_ERR_ARG;
  cudaSetDevice(c->device);
  XC_CHECK(cudaDeviceSynchronize());
  int r = batch_collect(c, b, c->stream, out, cap, n_out, pair_counts);
  if (r == XC_INTERNAL_OVERFLOW) r = batch_rerun_overflow(c, b, c->stream, out, cap, n_out, pair_counts);
  return r;
}

int xc_batch_offsets(xc_ctx* c, xc_batch* b, int* offs, size_t cap, size_t* n_out, int* counts) {
  if (!c || !b) return XC_ERR_ARG;
  cudaSetDevice(c->device);
  XC_CHECK(cudaDeviceSynchronize());
  const int n = b->n;
  std::vector<int> cnt(2 * (size_t)n);
  XC_CHECK(cudaMemcpy(cnt.data(), b->d_offcnt, cnt.size() * sizeof(int), cudaMemcpyDeviceToHost));
  std::vector<int> dev_of(n);
  for (int d = 0; d < n; d++) dev_of[b->order[d]] = d;
  size_t need = 0;
  for (int i = 0; i < n; i++)
    for (int s2 = 0; s2 < 2; s2++) {
      const int k = cnt[2 * dev_of[i] + s2];
      if (counts) counts[2 * i + s2] = k;
      need += (size_t)k;
    }
  if (n_out) *n_out = need;
  if (!offs) return XC_OK;
  if (need > cap) return XC_ERR_CAPACITY;
  size_t o = 0;
  for (int i = 0; i < n; i++) {
    const int d = dev_of[i];
    const PairDesc& D = b->desc_host[d];
    for (int s2 = 0; s2 < 2; s2++) {
      const int k = cnt[2 * d + s2];
      if (k) XC_CHECK(cudaMemcpy(offs + o, b->d_off + D.off_base + ((size_t)s2 << D.log2L), k * sizeof(int),
                                 cudaMemcpyDeviceToHost));
      o += (size_t)k;
    }
  }
  return XC_OK;
}

int xc_batch_straddles(xc_ctx* c, xc_batch* b, int* counts, int* lags) {
  if (!c || !b) return XC_ERR_ARG;
  cudaSetDevice(c->device);
  XC_CHECK(cudaDeviceSynchronize());
  const int n = b->n;
  std::vector<int> cnt(2 * (size_t)n), lst(2 * (size_t)n * STRAD_CAP);
  XC_CHECK(cudaMemcpy(cnt.data(), b->d_stradcnt, cnt.size() * sizeof(int), cudaMemcpyDeviceToHost));
  if (lags) XC_CHECK(cudaMemcpy(lst.data(), b->d_strad, lst.size() * sizeof(int), cudaMemcpyDeviceToHost));
  for (int d = 0; d < n; d++) {
    const int i = b->order[d];
    for (int s2 = 0; s2 < 2; s2++) {
      const int k = cnt[2 * d + s2];
      if (counts) counts[2 * i + s2] = k;
      if (lags) {
        int* dst = lags + (size_t)(2 * i + s2) * STRAD_CAP;
        const int* src = lst.data() + (size_t)(2 * d + s2) * STRAD_CAP;
        const int m = std::min(k, STRAD_CAP);
        std::copy(src, src + m, dst);
        std::sort(dst, dst + m);
        std::fill(dst + m, dst + STRAD_CAP, -1);
      }
    }
  }
  return XC_OK;
}

int xc_batch_free(xc_ctx* c, xc_batch* b) {
  if (!c || !b) return XC_ERR_ARG;
  cudaSetDevice(c->device);
  cudaDeviceSynchronize();
  delete b;
  return XC_OK;
}

int xc_batch_launches(xc_ctx* c, xc_batch* b) {
  if (!c || !b) return XC_ERR_ARG;
  return batch_launch_count(c, b);
}

int xc_batch_run_timed(xc_ctx* c, xc_batch* b, void* stream, float* stage_ms) {
  if (!c || !b) return XC_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  int r = batch_run(c, b, s, true, true);
  if (r != XC_OK) return r;
  XC_CHECK(cudaEventSynchronize(b->ev[3]));
  if (stage_ms)
    for (int i = 0; i < 3; i++) XC_CHECK(cudaEventElapsedTime(&stage_ms[i], b->ev[i], b->ev[i + 1]));
  return XC_OK;
}

int xc_transfer_stats(xc_ctx* c, uint64_t* h2d, uint64_t* d2h) {
  if (!c) return XC_ERR_ARG;
  if (h2d) *h2d = c->last_h2d;
  if (d2h) *d2h = c->last_d2h;
  return XC_OK;
}

int xc_debug_pair(xc_ctx* c, const xc_pair* pair, float* sig, float* xcv, int* offs, int* n_offs, int* segs,
                  int* n_segs, int seg_cap, int* fft_len_out) {
  if (!c || !pair) return XC_ERR_ARG;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  Batch b;
  b.slots = c->prm.result_slots > 0 ? c->prm.result_slots : 64;
  b.ovf_cap = 1 << 16;
  int r = batch_pack(c, &b, pair, 1, c->stream);
  if (r != XC_OK) return r;
  const int L = 1 << b.log2L[0];
  if (fft_len_out) *fft_len_out = L;
  b.dbg_cap = 1 << 20;
  XC_CHECK(cudaMalloc(&b.d_dbg, (size_t)b.dbg_cap * sizeof(DbgSeg)));
  if (sig) {   // signal output runs the pair on corr_kernel, one CTA per strand
    XC_CHECK(cudaMalloc(&b.d_dbg_sig, (size_t)2 * 8 * L * sizeof(float)));
    XC_CHECK(cudaMemset(b.d_dbg_sig, 0, (size_t)2 * 8 * L * sizeof(float)));
  }
  XC_CHECK(cudaMalloc(&b.d_dbg_xc, (size_t)2 * L * sizeof(float)));
  if ((r = batch_run(c, &b, c->stream, false)) != XC_OK) return r;
  XC_CHECK(cudaStreamSynchronize(c->stream));
  int misc[4];
  XC_CHECK(cudaMemcpy(misc, b.d_misc, sizeof(misc), cudaMemcpyDeviceToHost));
  uint32_t flag;
  XC_CHECK(cudaMemcpy(&flag, b.d_flags, sizeof(flag), cudaMemcpyDeviceToHost));
  if (flag & PF_INVALID) return XC_ERR_INPUT;
  if (sig) XC_CHECK(cudaMemcpy(sig, b.d_dbg_sig, (size_t)2 * 8 * L * sizeof(float), cudaMemcpyDeviceToHost));
  if (xcv) XC_CHECK(cudaMemcpy(xcv, b.d_dbg_xc, (size_t)2 * L * sizeof(float), cudaMemcpyDeviceToHost));
  int oc[2];
  XC_CHECK(cudaMemcpy(oc, b.d_offcnt, sizeof(oc), cudaMemcpyDeviceToHost));
  if (n_offs) { n_offs[0] = oc[0]; n_offs[1] = oc[1]; }
  if (offs) {
    XC_CHECK(cudaMemcpy(offs, b.d_off, (size_t)oc[0] * sizeof(int), cudaMemcpyDeviceToHost));
    XC_CHECK(cudaMemcpy(offs + L, b.d_off + L, (size_t)oc[1] * sizeof(int), cudaMemcpyDeviceToHost));
  }
  const int nd = std::min(misc[2], b.dbg_cap);
  std::vector<DbgSeg> dg(nd);
  if (nd) XC_CHECK(cudaMemcpy(dg.data(), b.d_dbg, nd * sizeof(DbgSeg), cudaMemcpyDeviceToHost));
  std::sort(dg.begin(), dg.end(), [](const DbgSeg& a, const DbgSeg& q) {
    if (a.slot != q.slot) return a.slot < q.slot;
    if (a.key != q.key) return a.key < q.key;
    return a.tstart < q.tstart;
  });
  int ns[2] = {0, 0};
  for (const DbgSeg& g : dg) {
    const int s2 = g.slot & 1;
    if (segs && ns[s2] < seg_cap) {
      int* p = segs + ((size_t)s2 * seg_cap + ns[s2]) * 3;
      p[0] = g.tstart; p[1] = g.qstart; p[2] = g.len;
    }
    ns[s2]++;
  }
  if (n_segs) { n_segs[0] = ns[0]; n_segs[1] = ns[1]; }
  if (misc[1] & 2) return XC_ERR_CAPACITY;
  return XC_OK;
}

int xc_device_name(xc_ctx* c, char* buf, size_t len) {
  if (!c || !buf || !len) return XC_ERR_ARG;
  snprintf(buf, len, "%s", c->devname);
  return XC_OK;
}

}  // extern "C"
