// xc_align_pair_noalloc: one chunk pair through the correlation, scan and
// finalize kernels with every device buffer in a static device array.
//
// Some callers cannot call cudaMalloc: a process whose device memory is owned
// by another allocator (a framework's caching allocator or a fixed arena that
// has reserved the free HBM), where a fresh allocation would fail or
// fragment that pool, and latency-bound callers sharing the GPU with other
// streams, for whom cudaFree's device-wide synchronisation is not acceptable.
// This entry point serves them: the kernels' inputs (the two chunks and the
// pair descriptor) and their scratch (FindTop offset lists, per-strand result
// slots, counters) live in the file-scope array g_noalloc_scratch below, of
// fixed size, which every GPU that loads the library holds until exit.
//
// Set-up: the first call through a context, with the context's device
// current, looks up the array's device address with cudaGetSymbolAddress and
// keeps it in the context; later calls through that context reuse it.  That
// first call should come before any stream capture.  A device reset ends every
// context of the library on that device (their tables are gone with it); a
// context created afterwards looks the address up again.
// Every call shares the array and leaves its contents behind: each call
// zeroes the counters that must start at zero (offset counts, result counts,
// the overflow and error words) before its first kernel.  Calls that overlap
// on the GPU would race on the array; the calls in one process serialise on a
// mutex and return only after their results are back on the host.
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "satsuma2_xcorr.h"
#include "xc_runtime.h"

namespace xc {

namespace {

constexpr int NA_MAX_LOG2L = 14;          // largest FFT length: 16384
constexpr int NA_MAX_L = 1 << NA_MAX_LOG2L;
constexpr int NA_SLOTS = 1024;              // kept matches per strand

// Byte layout of the scratch array (256-byte aligned pieces).
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t NA_DESC = 0;                                            // PairDesc
constexpr size_t NA_CNT = 256;                                           // 16 ints, zeroed per call
constexpr size_t NA_POOL = 512;                                          // target, query chunk bytes
constexpr size_t NA_OFF = NA_POOL + align256((size_t)NA_MAX_L + 32);     // 2 x L FindTop offsets
constexpr size_t NA_RES = NA_OFF + align256((size_t)2 * NA_MAX_L * sizeof(int));
constexpr size_t NA_DENSE = NA_RES + align256((size_t)2 * NA_SLOTS * sizeof(DevResult));
constexpr size_t NA_BYTES = NA_DENSE + align256((size_t)2 * NA_SLOTS * sizeof(DevResult));
// counter words inside NA_CNT
constexpr int C_OFFCNT = 0;   // [2] FindTop offsets per strand
constexpr int C_FLAGS = 2;    // [1] pair flags
constexpr int C_FB2 = 3;      // [1] the pair index it may hand on to the ragged-query kernel
constexpr int C_WORK = 6;     // [1] the both-strands kernel's work counter
constexpr int C_FB2CNT = 7;   // [1] pairs handed on to the ragged-query kernel
constexpr int C_RESCNT = 4;   // [2] kept matches per strand
constexpr int C_MISC = 8;     // [4] overflow count, error bits, debug count, pairs handed back
constexpr int C_BASE = 12;    // [3] dense result bases
constexpr int C_FB = 15;      // [1] the pair index the both-strands kernel may hand back

static_assert(NA_BYTES <= 320 * 1024, "scratch layout exceeds the stated 320 KiB maximum");
// Every length accepted here keeps the correlation kernel's channel sums in
// shared memory; longer ones would need the global scratch (CorrParams::acc)
// that this entry point does not provide.
static_assert(NA_MAX_LOG2L <= MAX_SMEM_LOG2L, "FFT lengths beyond one SM need a channel-sum scratch");

}  // namespace

// 320 KiB: one pair of FFT length <= 16384, <= 1024 kept matches per strand.
static __device__ __align__(256) unsigned char g_noalloc_scratch[320 * 1024];

namespace {

std::mutex g_noalloc_mu;                          // one call at a time per process

// Device address of the scratch array for this context's device, looked up
// at the context's first call with that device current.
int noalloc_scratch(Ctx* c, unsigned char** out) {
  if (!c->noalloc_base) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      fprintf(stderr, "satsuma2_gb300: cudaGetSymbolAddress(g_noalloc_scratch): %s\n", cudaGetErrorString(e));
      return XC_ERR_CUDA;
    }
    c->noalloc_base = static_cast<unsigned char*>(p);
  }
  *out = c->noalloc_base;
  return XC_OK;
}

int cuda_fail(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return XC_OK;
  fprintf(stderr, "satsuma2_gb300: xc_align_pair_noalloc: %s: %s\n", what, cudaGetErrorString(e));
  return XC_ERR_CUDA;
}

#define NA_CHECK(call)                         \
  do {                                         \
    const int _r = cuda_fail((call), #call);   \
    if (_r != XC_OK) return _r;                \
  } while (0)

int align_pair_noalloc(Ctx* c, const xc_pair& p, xc_result* out, size_t cap, size_t* n_out) {
  if (p.tlen < 0 || p.qlen < 0 || (p.tlen && !p.tseq) || (p.qlen && !p.qseq)) return XC_ERR_ARG;
  const int lg = pair_log2L(c->prm, p);
  if (lg < MIN_LOG2L || lg > NA_MAX_LOG2L) {
    fprintf(stderr, "satsuma2_gb300: xc_align_pair_noalloc: FFT length 2^%d outside 2^%d..2^%d\n", lg,
            MIN_LOG2L, NA_MAX_LOG2L);
    return XC_ERR_UNSUPPORTED;
  }
  if (p.tlen > (1 << lg) / 2 || p.qlen > (1 << lg) / 2) return XC_ERR_INPUT;

  unsigned char* base = nullptr;
  int r = noalloc_scratch(c, &base);
  if (r != XC_OK) return r;
  PairDesc* d_desc = reinterpret_cast<PairDesc*>(base + NA_DESC);
  int* cnt = reinterpret_cast<int*>(base + NA_CNT);
  uint8_t* pool = base + NA_POOL;
  int* offl = reinterpret_cast<int*>(base + NA_OFF);
  DevResult* res = reinterpret_cast<DevResult*>(base + NA_RES);
  DevResult* dense = reinterpret_cast<DevResult*>(base + NA_DENSE);
  const cudaStream_t s = c->stream;

  // inputs into the array: both chunks (16-byte aligned), then the descriptor
  const uint32_t qoff = (uint32_t)((p.tlen + 15) & ~15);
  PairDesc D;
  D.t_off = 0;
  D.q_off = qoff;
  D.tlen = p.tlen;
  D.qlen = p.qlen;
  D.log2L = lg;
  D.flags = p.fast ? PF_FAST : 0u;
  D.off_base = 0;
  D.pad = 0;
  NA_CHECK(cudaMemsetAsync(cnt, 0, 16 * sizeof(int), s));
  if (p.tlen) NA_CHECK(cudaMemcpyAsync(pool, p.tseq, (size_t)p.tlen, cudaMemcpyHostToDevice, s));
  if (p.qlen) NA_CHECK(cudaMemcpyAsync(pool + qoff, p.qseq, (size_t)p.qlen, cudaMemcpyHostToDevice, s));
  NA_CHECK(cudaMemcpyAsync(d_desc, &D, sizeof(D), cudaMemcpyHostToDevice, s));

  const DevTables& t = c->tab[lg];
  CorrParams cp{};
  cp.pairs = d_desc;
  cp.pool = pool;
  cp.first = 0;
  const int NH = (1 << (lg - 1)) / 64;
  cp.tab.twN_hi = t.tw;
  cp.tab.twN_lo = t.tw + NH;
  cp.tab.twL_hi = t.tw + NH + 64;
  cp.tab.twL_lo = t.tw + 2 * NH + 64;
  cp.tab.ent = t.ent;
  cp.tab.ent_acgt = t.ent_acgt;
  cp.cutoff = c->prm.cutoff;
  cp.cutoff_fast = c->prm.cutoff_fast;
  cp.off_list = offl;
  cp.off_cnt = cnt + C_OFFCNT;
  cp.pair_flags = reinterpret_cast<uint32_t*>(cnt + C_FLAGS);
  if (lg == PAIR_LOG2L && c->pair_kernel) {
    // the same correlation kernels as xc_align_pairs: both strands in one
    // CTA, the ragged-query kernel for an A/C/G/T query of >= 1024 bases
    // that is not a multiple of 16, or the per-strand kernel for a pair
    // handed back
    cp.fb_list = cnt + C_FB;
    cp.fb_cnt = cnt + C_MISC + 3;
    cp.pair_form = c->pair_form;
    if (c->pair_form == 2 && p.qlen >= 1024 && p.qlen % 16 != 0) {
      cp.fb2_list = cnt + C_FB2;
      cp.fb2_cnt = cnt + C_FB2CNT;
    }
  }
  cp.work = cnt + C_WORK;
  cp.strand_threads = c->strand_threads[lg];
  NA_CHECK(launch_corr(lg, cp, 1, s));

  ScanParams sp{};
  sp.pairs = d_desc;
  sp.pool = pool;
  sp.first = 0;
  sp.off_list = offl;
  sp.off_cnt = cnt + C_OFFCNT;
  sp.pair_flags = reinterpret_cast<uint32_t*>(cnt + C_FLAGS);
  sp.score = c->d_score;
  sp.eq = c->d_eq;
  sp.gcw = c->d_gcw;
  sp.ptable = c->prm.use_prob_table ? c->d_ptable : nullptr;
  sp.ptable_cutoff = c->prm.prob_table_cutoff;
  sp.min_prob = c->prm.min_prob;
  sp.target_total = c->prm.target_total;
  sp.screen_z = screen_z(c->prm.min_prob, c->prm.target_total);
  sp.min_len = c->prm.min_len;
  sp.slots = NA_SLOTS;
  sp.res = res;
  sp.res_cnt = cnt + C_RESCNT;
  sp.ovf = nullptr;           // no overflow pool: matches beyond NA_SLOTS are counted, not kept
  sp.ovf_cnt = cnt + C_MISC + 0;
  sp.ovf_cap = 0;
  sp.err = cnt + C_MISC + 1;
  sp.dbg = nullptr;
  sp.dbg_cnt = cnt + C_MISC + 2;
  sp.dbg_cap = 0;
  if (!sp.ptable) sp.word_floor = run_hits_floor(sp.screen_z, sp.min_len, sp.run_floor);
  NA_CHECK(launch_scan(lg, sp, 1, s));
  NA_CHECK(launch_finalize(cnt + C_RESCNT, res, NA_SLOTS, 2, cnt + C_BASE, dense, nullptr, s));

  int h[16];
  NA_CHECK(cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s));
  NA_CHECK(cudaStreamSynchronize(s));
  if (h[C_FLAGS] & PF_INVALID) return XC_ERR_INPUT;
  // error bits of the scan: bit 0 (records beyond the slots, no overflow pool
  // here) is reported below as XC_ERR_CAPACITY; any other bit is a failure
  if (h[C_MISC + 1] & ~1) {
    fprintf(stderr, "satsuma2_gb300: xc_align_pair_noalloc: scan kernel error bits 0x%x\n", h[C_MISC + 1]);
    return XC_ERR_CUDA;
  }
  const int total = h[C_BASE + 2];
  const size_t need = (size_t)total + (size_t)h[C_MISC + 0];   // kept + beyond the slots
  if (n_out) *n_out = need;
  if (h[C_MISC + 0] > 0) {
    fprintf(stderr,
            "satsuma2_gb300: xc_align_pair_noalloc: %zu matches found; a strand exceeds its %d kept slots\n",
            need, NA_SLOTS);
    return XC_ERR_CAPACITY;
  }
  if (need > cap || (!out && need)) return XC_ERR_CAPACITY;

  // dense records (strand 0 then strand 1, each in the reference's order) to
  // t_result, through a small stack buffer
  const int qchunk = c->prm.q_chunk;
  DevResult buf[64];
  for (int k0 = 0; k0 < total; k0 += 64) {
    const int m = total - k0 < 64 ? total - k0 : 64;
    NA_CHECK(cudaMemcpyAsync(buf, dense + k0, (size_t)m * sizeof(DevResult), cudaMemcpyDeviceToHost, s));
    NA_CHECK(cudaStreamSynchronize(s));
    for (int j = 0; j < m; j++) {
      const int k = k0 + j;
      const int strand = k >= h[C_BASE + 1] ? 1 : 0;
      const DevResult& rr = buf[j];
      xc_result& x = out[k];
      memset(&x, 0, sizeof(x));
      // FilterMatches coordinate mapping (HomologyByXCorrSlave.cc:175-181, RCQuery :56-60)
      const int tStart = p.t_chunk_start + rr.tstart;
      const int qStart = strand == 0 ? p.q_chunk_start + rr.qstart
                                     : rr.qstart + (int)p.query_size - p.q_chunk_start - qchunk;
      x.query_id = p.query_id;
      x.target_id = p.target_id;
      x.query_size = p.query_size;
      x.qstart = (unsigned long)(long)qStart;
      x.tstart = (unsigned long)(long)tStart;
      x.len = (unsigned long)(long)rr.len;
      x.reverse = (unsigned char)strand;
      x.prob = rr.prob;
      x.ident = rr.ident;
    }
  }
  return XC_OK;
}

}  // namespace

}  // namespace xc

extern "C" int xc_align_pair_noalloc(xc_ctx* c, const xc_pair* pair, xc_result* out, size_t cap, size_t* n_out) {
  if (n_out) *n_out = 0;
  if (!c || !pair) return XC_ERR_ARG;
  std::lock_guard<std::mutex> lk(xc::g_noalloc_mu);
  std::lock_guard<std::mutex> lc(c->mu);
  const cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return xc::cuda_fail(e, "cudaSetDevice");
  return xc::align_pair_noalloc(c, *pair, out, cap, n_out);
}
