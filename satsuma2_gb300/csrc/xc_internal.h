// Internal definitions shared by the kernels (xc_corr.cu, xc_scan.cu) and the host
// runtime (xc_runtime.cu).  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace xc {

constexpr int MIN_LOG2L = 10;    // FFT length 1024
constexpr int MAX_LOG2L = 15;    // FFT length 32768
constexpr int MAX_SMEM_LOG2L = 14;  // longest FFT whose two transforms and channel sums fit one SM
constexpr int NT_CORR = 512;     // threads of the correlation kernel (one pair strand)
constexpr int NT_PAIR = 1024;    // threads of the both-strands correlation kernel (first form)
constexpr int NT_PAIR2 = 512;    // threads of the persistent both-strands correlation kernel
constexpr int PAIR_LOG2L = 13;   // FFT length of the both-strands kernel (its buffers fill one SM)
constexpr int NT_SCAN = 128;     // threads of the scan kernel
constexpr int OFF_CHUNK = 256;   // offsets staged per scan chunk
constexpr int SCAN_CTAS_PER_SM = 8;   // scan register budget: 64 per thread (8 measured 3% faster than 7)
constexpr int WINDOW = 46;       // DoOne window: m_minLen + 1 positions (CrossCorr.cc:701-705)
constexpr int MIN_HITS = 19;     // ACGT windows pass when 100*hits > 1889 (CrossCorr.cc:675)

// Near-threshold band of FindTop: lags whose FP32 correlation lies within
// straddle_rel(L) * max(1, max|xc|) of the FP32 threshold.  The reference's
// FP32 FFT (FFTReal) and this one each differ from the exact correlation by
// ~2e-7 of the peak (measured), so only there can their keep/drop decisions
// part; the band is about 60x that.  At L = 32768 FFTReal rotates its
// twiddles with a float oscillator beyond its 12th pass and its own error
// grows to ~1.5e-4 of the peak, hence the wider band.  The parity tests use
// the same band around the FP64 threshold.
constexpr int STRAD_CAP = 16;    // near-threshold lags listed per pair strand (all are counted)
__host__ __device__ constexpr float straddle_rel(int log2L) { return log2L > 14 ? 3e-4f : 2e-5f; }

// Pair flags written by the correlation kernel, read by the scan kernel.
enum : uint32_t {
  PF_FAST = 1u,        // use cutoff_fast
  PF_GENERIC = 2u,     // some byte outside A/C/G/T: byte-table scan path
  PF_INVALID = 4u,     // some byte >= 128: pair rejected
};

struct __align__(16) PairDesc {
  uint32_t t_off, q_off;   // byte offsets of the chunks in the sequence pool
  int32_t tlen, qlen;
  int32_t log2L;           // FFT length
  uint32_t flags;          // PF_FAST from the host
  uint32_t off_base;       // FindTop offsets: strand s at off_base + s*L
  uint32_t pad;
};

// Per-FFT-length device tables (host-built in double, rounded once).
// Twiddles W_M^m = hi[m >> 6] * lo[m & 63] for M = N (transform) and M = L.
struct LTables {
  const float2* twN_hi;    // exp(-2*pi*i*64a/N), a < N/64, N = L/2
  const float2* twN_lo;    // exp(-2*pi*i*b/N), b < 64
  const float2* twL_hi;    // exp(-2*pi*i*64a/L), a < N/64
  const float2* twL_lo;    // exp(-2*pi*i*b/L), b < 64
  const double* ent;       // Ent(p) for p = (a4/4)/k: [k][a4], k <= win, a4 <= 4*win
  const float* ent_acgt;   // weight of a full window of a A, c C, g G, t T: [(a*(win+1)+c)*(win+1)+g]
};

// One kept match, strand-local coordinates.  key = FindTop offset index.
struct __align__(16) DevResult {
  int32_t key;
  int32_t tstart;
  int32_t qstart;
  int32_t len;
  double prob;
  double ident;
};

struct __align__(16) DevResultX {   // overflow record
  int32_t slot;                     // pair*2 + strand
  int32_t pad[3];
  DevResult r;
};

struct __align__(16) DbgSeg {
  int32_t slot, key, tstart, qstart, len, pad[3];
};

struct CorrParams {
  const PairDesc* pairs;
  const uint8_t* pool;
  int first;                // first pair index of this launch (bucket)
  LTables tab;
  double cutoff, cutoff_fast;
  int* off_list;            // offsets output
  int* off_cnt;             // [pair*2 + strand]
  uint32_t* pair_flags;     // [pair]
  float* dbg_sig;           // optional: [pair*2+strand][2][4][L]
  float* dbg_xc;            // optional: [pair*2+strand][L]
  float2* acc;              // L > 2^MAX_SMEM_LOG2L: channel sums, [pair*2+strand][acc_stride(log2L)]
  int* fb_list;             // log2L == PAIR_LOG2L: both-strands kernel first; the pairs it
  int* fb_cnt;              //   hands back ([*fb_cnt], zeroed before) go to corr_kernel
  int* fb2_list;            // optional: the A/C/G/T pairs with a ragged query window the
  int* fb2_cnt;             //   persistent kernel hands to corr_rcq_kernel ([*fb2_cnt], zeroed before)
  int rcq_first, rcq_count; // without fb2_list: corr_rcq_kernel takes pairs rcq_first.. (+rcq_count),
                            //   the bucket's ragged query windows, placed after the pair kernel's
  int* strad_cnt;           // optional: near-threshold lags per [pair*2 + strand] (zeroed before)
  int* strad_list;          //   and the first STRAD_CAP of them, [pair*2 + strand][STRAD_CAP]
  int count;                // pairs of this launch (set by launch_corr)
  int* work;                // persistent kernels: counter of pairs taken after each CTA's first (zeroed before the launch)
  int pair_form;            // with fb_list: 2 = persistent 512-thread kernel, 1 = 1024-thread form
  // spectra path (FFT 8192 batches whose pairs share chunks): the pair kernel
  // reads both chunks' spectra instead of transforming them
  int strand_threads;       // threads per strand of the per-strand kernel (0 = NT_CORR; see strand_threads_ok)
  const int* pair_chunk;    // [pair][2]: target and query chunk indices
  const float2* spec;       // [chunk][4][N] spectra, bin order (see SpecParams)
  const uint32_t* chunk_flags;
};

// Chunk flags of the spectra path.
enum : uint32_t {
  CF_HIGH = 1u,      // a byte >= 128: the pairs with this chunk are rejected
  CF_GENERIC = 2u,   // a byte other than A/C/G/T: its pairs go to the per-strand kernel
};

struct ChunkDesc {
  uint32_t off;             // byte offset of the chunk in the sequence pool
  int32_t len;
};

// spec_kernel: the transforms of each distinct chunk of a batch, once.
struct SpecParams {
  const ChunkDesc* chunks;
  int count;
  const uint8_t* pool;
  LTables tab;
  float2* spec;             // [chunk][4][N]: channels (A,T) even-bin, odd-bin transform, then (C,G); bin order
  uint32_t* chunk_flags;    // [chunk]: CF_* (0 = spectra written)
  int* work;                // counter of chunks taken after each CTA's first (zeroed before the launch)
};

// Global channel-sum scratch of one pair strand for FFT lengths beyond one
// SM's shared memory: even bins 0..N/2, then odd bins 0..N/2-1 (8 apart).
__host__ __device__ constexpr size_t acc_stride(int log2L) {
  return log2L > MAX_SMEM_LOG2L ? ((size_t)1 << (log2L - 1)) + 16 : 0;
}

struct ScanParams {
  const PairDesc* pairs;
  const uint8_t* pool;
  int first;
  const int* off_list;
  const int* off_cnt;
  const uint32_t* pair_flags;
  const int8_t* score;      // [128*128] (int)(DNA_EqualAmb*100+0.5)
  const double* eq;         // [128*128] DNA_Equal
  const double* gcw;        // [128] DNA_C + DNA_G
  const double* ptable;     // ProbTable [512*2048] or nullptr
  double ptable_cutoff;
  double min_prob;
  double target_total;
  float screen_z;           // FP32 screen: reject when pm*N - hits > screen_z * sd (+inf keeps all)
  uint32_t run_floor[8];    // bytes [r-1]: least equal-base count with which a run of r passing
                            // checks can pass the screen (run_hits_floor; zeros: no floor)
  int word_floor;           // the least of them (0: every screened word is marked)
  int min_len;
  int slots;                // result slots per pair strand
  DevResult* res;           // [pair*2+strand][slots]
  int* res_cnt;             // [pair*2+strand]
  DevResultX* ovf;
  int* ovf_cnt;
  int ovf_cap;
  int* err;                 // bit 0: overflow pool full; bit 1: debug buffer full
  DbgSeg* dbg;              // optional raw segments
  int* dbg_cnt;
  int dbg_cap;
};

// Launchers (xc_corr.cu, xc_scan.cu).
cudaError_t launch_corr(int log2L, const CorrParams& p, int npairs, cudaStream_t s);
// FFT 8192 with shared chunks: spec_kernel over the distinct chunks, then the
// pair kernel from their spectra, corr_rcq_kernel over the ragged query
// windows (fb2_list), then corr_kernel over the pairs handed back.
cudaError_t launch_corr_spec(const SpecParams& sp, const CorrParams& p, int npairs, cudaStream_t s);
size_t spec_bytes_per_chunk();
// Thread counts per strand the per-strand correlation kernel is built for.
bool strand_threads_ok(int log2L, int nt);
cudaError_t launch_scan(int log2L, const ScanParams& p, int npairs, cudaStream_t s);
cudaError_t launch_finalize(const int* res_cnt, const DevResult* res, int slots, int nslots,
                            int* dense_base, DevResult* dense, int* scan_tmp, cudaStream_t s);
cudaError_t upload_constants(const unsigned char* rc256, const uchar4* w4q128,
                             const double* w4d /*4*128*/);
size_t corr_smem_bytes(int log2L);
size_t corr_pair_smem_bytes(int log2L);
size_t scan_smem_bytes(int log2L);
cudaError_t prepare_kernels();

}  // namespace xc
