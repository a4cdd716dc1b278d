// Host-side runtime structures shared by xc_runtime.cu and xc_server.cu.
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <mutex>
#include <vector>

#include "satsuma2_xcorr.h"
#include "xc_internal.h"

namespace xc {

struct Bucket {
  int log2L;
  int first;
  int count;
};

// Slot of the table that finds a chunk passed again by the same pointer and length.
struct HashSlot {
  const char* p;
  int len;
  uint32_t uid;
};

// Device and pinned host buffers of one packed batch of chunk pairs.  Pairs
// are stored in "device order" (grouped by FFT length); order[d] maps a device
// index to the caller's index.
struct Batch {
  int n = 0;
  int slots = 64;                 // result slots per pair strand
  int ovf_cap = 1 << 16;          // overflow records
  int dbg_cap = 0;
  std::vector<xc_pair> meta;      // caller's pairs (ids, chunk starts), caller order
  std::vector<int> order;
  std::vector<int> log2L;         // per caller index
  std::vector<Bucket> buckets;
  std::vector<PairDesc> desc_host;
  uint64_t pool_bytes = 0, h2d_bytes = 0;

  uint8_t* d_pool = nullptr;      size_t cap_pool = 0;
  PairDesc* d_desc = nullptr;     size_t cap_desc = 0;
  int* d_off = nullptr;           size_t cap_off = 0;
  int* d_offcnt = nullptr;        size_t cap_offcnt = 0;
  uint32_t* d_flags = nullptr;    size_t cap_flags = 0;
  DevResult* d_res = nullptr;     size_t cap_res = 0;
  int* d_rescnt = nullptr;        size_t cap_rescnt = 0;
  DevResultX* d_ovf = nullptr;    size_t cap_ovf = 0;
  int* d_misc = nullptr;          size_t cap_misc = 0;   // [0] ovf count [1] err [2] dbg count
                                                         // [3] pairs the both-strands kernel handed back
                                                         // [4] [5] work counters [6] ragged query windows
  int* d_fb = nullptr;            size_t cap_fb = 0;     // those pairs' indices
  int* d_fb2 = nullptr;           size_t cap_fb2 = 0;    // A/C/G/T pairs with a ragged query window it handed on
  int ragged = 0;                 // FFT-8192 pairs whose query is >= 1024 bases and not a multiple of 16
  int* d_stradcnt = nullptr;      size_t cap_stradcnt = 0;   // near-threshold lags per pair strand
  int* d_strad = nullptr;         size_t cap_strad = 0;      // the first STRAD_CAP of them
  // spectra path of the FFT-8192 bucket (its pairs share chunks): distinct
  // chunks, each pair's two chunk indices, the chunks' spectra and flags
  bool spec = false;
  int spec_chunks = 0;
  std::vector<ChunkDesc> chunk_host;
  std::vector<int> pair_chunk_host;
  ChunkDesc* d_chunks = nullptr;  size_t cap_chunks = 0;
  int* d_pairchunk = nullptr;     size_t cap_pairchunk = 0;
  float2* d_spec = nullptr;       size_t cap_spec = 0;
  uint32_t* d_chunkflags = nullptr; size_t cap_chunkflags = 0;
  uint64_t unique_bytes = 0;      // sequence bytes after de-duplication
  std::vector<HashSlot> ht;       // (pointer, length) -> distinct chunk, reused across packs
  int* d_base = nullptr;          size_t cap_base = 0;
  DevResult* d_dense = nullptr;   size_t cap_dense = 0;
  float2* d_acc = nullptr;        size_t cap_acc = 0;     // channel sums of FFT lengths beyond one SM
  DbgSeg* d_dbg = nullptr;
  float* d_dbg_sig = nullptr;
  float* d_dbg_xc = nullptr;

  uint8_t* h_pool = nullptr;      size_t cap_h_pool = 0;
  PairDesc* h_desc = nullptr;     size_t cap_h_desc = 0;
  int* h_base = nullptr;          size_t cap_h_base = 0;
  DevResult* h_dense = nullptr;   size_t cap_h_dense = 0;
  uint32_t* h_flags = nullptr;    size_t cap_h_flags = 0;
  size_t pre_dense = 0;           // dense records the queued read-back copies
  size_t est_dense = 0;           // estimate for the next read-back (last total + 25%)
  bool rb_pending = false;        // batch_readback_async queued, not yet collected
  int* h_misc = nullptr;          size_t cap_h_misc = 0;
  DevResultX* h_ovf = nullptr;

  cudaGraphExec_t graph_exec = nullptr;
  bool graph_valid = false;
  cudaStream_t graph_stream = nullptr;
  // stage-timing variant: events between the correlation, scan and finalize launches
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaStream_t side = nullptr;     // several FFT buckets: their scans beside the largest one's
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  cudaGraphExec_t graph_exec_timed = nullptr;
  bool graph_timed_valid = false;
  cudaStream_t graph_timed_stream = nullptr;
  uint64_t d2h_bytes = 0;

  ~Batch();
};

struct Server;

struct DevTables {
  float2* tw = nullptr;    // W_N hi (N/64), W_N lo (64), W_L hi (N/64), W_L lo (64)
  double* ent = nullptr;
  float* ent_acgt = nullptr;   // entropy weight of full A/C/G/T windows by base counts
};

struct Ctx {
  xc_params prm{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;               // serialises the synchronous entry points
  DevTables tab[MAX_LOG2L + 1];
  int8_t* d_score = nullptr;
  double* d_eq = nullptr;
  double* d_gcw = nullptr;
  double* d_ptable = nullptr;
  std::vector<double> h_ptable;
  Batch* work[2] = {nullptr, nullptr};       // xc_align_pairs: two sub-batches in flight
  cudaStream_t work_stream[2] = {nullptr, nullptr};
  Server* server = nullptr;
  char devname[256] = {0};
  uint64_t last_h2d = 0, last_d2h = 0;
  int sms = 152;               // multiprocessors of the device (sub-batch sizing)
  bool pair_kernel = false;    // both-strands correlation kernel usable (entropy table complement-symmetric)
  int pair_form = 2;           // its form: 2 persistent 512-thread kernel, 1 the 1024-thread one
  bool spec_reuse = true;      // FFT-8192 batches whose pairs share chunks transform each chunk once
  int strand_threads[MAX_LOG2L + 1] = {};   // per-strand kernel's threads per FFT length (0 = 512; xc_tune)
  unsigned char* noalloc_base = nullptr;   // xc_align_pair_noalloc's static array on this device (set at first use)
};



// Pairs per distinct chunk (2 x pairs / chunks) from which an FFT-8192 bucket
// takes the spectra path: each chunk transformed once, 128 KB of spectra per
// chunk written and read back from L2 per pair, where the both-strands kernel
// transforms both chunks of every pair in shared memory.
constexpr double SPEC_MIN_REUSE = 3.0;

// batch_collect's status when the batch's device overflow pool filled during
// the run (records were dropped on the device).  Internal only: every caller
// grows the pool and runs the batch again (batch_rerun_overflow), so it never
// reaches the C ABI, and it is never confused with XC_ERR_CAPACITY (the
// caller's output buffer is too small).
constexpr int XC_INTERNAL_OVERFLOW = -100;

int pair_log2L(const xc_params& p, const xc_pair& q);
Batch* new_batch(Ctx* c);
int batch_pack(Ctx* c, Batch* b, const xc_pair* pairs, size_t n, cudaStream_t stream);
int batch_run(Ctx* c, Batch* b, cudaStream_t s, bool use_graph, bool timed = false);
// Queues the result read-back (counts, flags, an estimate of the dense
// records) on s behind the batch's kernels; batch_collect then waits once.
int batch_readback_async(Ctx* c, Batch* b, cudaStream_t s);
int batch_collect(Ctx* c, Batch* b, cudaStream_t s, xc_result* out, size_t cap, size_t* n_out,
                  size_t* pair_counts);
// After batch_collect returned XC_INTERNAL_OVERFLOW: grows the overflow pool to
// what the run asked for and runs the batch again on s (the pairs are still on
// the device), then collects; XC_ERR_NOMEM if three runs still overflow.
int batch_rerun_overflow(Ctx* c, Batch* b, cudaStream_t s, xc_result* out, size_t cap, size_t* n_out,
                         size_t* pair_counts);
int batch_launch_count(const Ctx* c, const Batch* b);
// z-score threshold of the scan kernel's FP32 probability screen.
float screen_z(double min_prob, double target_total);
int run_hits_floor(float screen_z, int min_len, uint32_t out[8]);
int ctx_align_pipelined(Ctx* c, const xc_pair* pairs, size_t n, xc_result* out, size_t cap, size_t* n_out,
                        size_t* pair_counts);
void server_stop(Ctx* c);
// Applies a tuning table (xc_tune's text: "fft_len=L strand_threads=T" and
// "pair_form=F" lines; other text ignored); XC_ERR_ARG on a bad value.
int apply_tuning_text(Ctx* c, const char* text);

}  // namespace xc

// The opaque handles of the C ABI.
struct xc_ctx : public xc::Ctx {};
struct xc_batch : public xc::Batch {};
