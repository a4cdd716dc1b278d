/*
 * satsuma2_xcorr.h -- C ABI of the GB300 cross-correlation library
 * (satsuma2_gb300/libsatsuma2_gb300.so).
 *
 * The library replaces the per-chunk-pair compute of satsuma2's slave,
 * HomologyByXCorr::align_target / Align / FilterMatches
 * (analysis/HomologyByXCorrSlave.cc:168-300): a target chunk and a query
 * chunk go in, scored t_result records come out, with the slave's -cutoff,
 * -cutoff_fast, -l, -t_chunk, -q_chunk and -prob_table semantics.  Everything
 * runs on one GPU; there is no CPU fallback: without a usable device every
 * compute call returns XC_ERR_CUDA.
 *
 * Plain C types only.  All calls return 0 on success or a negative XC_ERR_*.
 * A context is safe to use from several host threads for xc_submit/xc_wait;
 * the synchronous calls serialise on the context.
 */
#ifndef SATSUMA2_XCORR_H
#define SATSUMA2_XCORR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XC_OK 0
#define XC_ERR_ARG (-1)          /* bad argument (null pointer, bad size) */
#define XC_ERR_CUDA (-2)         /* CUDA runtime error or no device */
#define XC_ERR_NOMEM (-3)        /* device or pinned host allocation failed */
#define XC_ERR_CAPACITY (-4)     /* output buffer too small; *n_out holds the size needed */
#define XC_ERR_INPUT (-5)        /* a byte >= 128, or a chunk longer than half the FFT length */
#define XC_ERR_TIMEOUT (-6)      /* xc_wait timed out; the ticket stays valid */
#define XC_ERR_UNSUPPORTED (-7)  /* FFT length outside 1024..32768 */
#define XC_ERR_BUSY (-8)         /* admission refused: request queue or memory budget full */

/* Result record.  Same fields, order and 72-byte LP64 layout as t_result
 * (analysis/WorkQueue.h:23-33), so records go on the slave's wire unchanged. */
typedef struct {
  unsigned long query_id;    /* query sequence index (SeqChunk::GetID) */
  unsigned long target_id;   /* target sequence index */
  unsigned long query_size;  /* full length of the query sequence */
  unsigned long qstart;      /* query start; reverse strand mapped as RCQuery does */
  unsigned long tstart;      /* target start in sequence coordinates */
  unsigned long len;         /* match length */
  unsigned char reverse;     /* 1 = reverse-complemented query strand (C++ bool) */
  double prob;               /* GetMatchProbability, or the table cutoff in table mode */
  double ident;              /* identity, as PrintMatch computes it */
} xc_result;

/* Work request of the slave protocol; same layout as t_pair
 * (analysis/WorkQueue.h:17-22, 28 bytes): an inclusive block of target chunk
 * indices x query chunk indices. */
typedef struct {
  int targetFrom, targetTo, queryFrom, queryTo;
  unsigned char fast;        /* C++ bool: use the fast cutoff */
  int slave_id;
  unsigned char status;
} xc_block;

/* Slave parameters (HomologyByXCorrSlave.cc:28-53, 334-384). */
typedef struct {
  double cutoff;             /* -cutoff, FindTop cutoff (default 1.8) */
  double cutoff_fast;        /* -cutoff_fast (2.9), used for pairs with fast set */
  double min_prob;           /* probability a match must reach.  The reference
                                slave keeps m_minProb = 0.99 whatever -min_prob
                                says (HomologyByXCorrSlave.cc:76); pass 0.99 for
                                slave-faithful output. */
  double target_total;       /* sum of all target sequence lengths (:405-408) */
  int min_len;               /* -l, minimum match length (0) */
  int t_chunk;               /* -t_chunk (4096); FFT length is 2*t_chunk */
  int q_chunk;               /* -q_chunk (4096); reverse-strand qstart uses it */
  int fft_len;               /* 0: 2*t_chunk as the slave does; >0: that length;
                                -1: per pair nextpow2(2*max(tlen,qlen)), min 1024 */
  int use_prob_table;        /* -prob_table: ProbTable lookup instead of erf/exp */
  double prob_table_cutoff;  /* ProbTable's cutoff, i.e. the slave's -min_prob */
  int max_batch;             /* pairs per device batch (0 = 4096) */
  int result_slots;          /* result slots per pair strand before overflow (0 = 64) */
} xc_params;

/* One chunk pair.  Sequences are uppercase ASCII (the slave uppercases at
 * FASTA read, DNAVector.cc:1235,1274); lengths at most fft_len/2. */
typedef struct {
  const char* tseq;          /* target chunk bytes */
  int tlen;
  int t_chunk_start;         /* chunk start within its target sequence */
  unsigned long target_id;   /* target sequence index */
  const char* qseq;          /* query chunk bytes (forward strand) */
  int qlen;
  int q_chunk_start;         /* chunk start within its query sequence */
  unsigned long query_id;    /* query sequence index */
  unsigned long query_size;  /* full query sequence length */
  int fast;                  /* nonzero: use cutoff_fast */
} xc_pair;

typedef struct xc_ctx xc_ctx;
typedef struct xc_batch xc_batch;

/* Creates a context on a CUDA device.  Replaces the slave's per-thread
 * HomologyByXCorr objects and, with use_prob_table, the ProbTable built at
 * start-up (HomologyByXCorrSlave.cc:413-421). */
int xc_create(const xc_params* params, int device, xc_ctx** ctx);
int xc_destroy(xc_ctx* ctx);

/* Runs n chunk pairs, both strands each, and writes their results to out in
 * pair order; within a pair the forward strand first, each strand in FindTop
 * offset order then position order -- the order Align appends them
 * (HomologyByXCorrSlave.cc:221-253).  pair_counts, if not NULL, gets the
 * number of results of each pair.  Returns XC_ERR_CAPACITY with *n_out set if
 * cap is too small.  Replaces HomologyByXCorr::Align + FilterMatches. */
int xc_align_pairs(xc_ctx* ctx, const xc_pair* pairs, size_t n, xc_result* out, size_t cap,
                   size_t* n_out, size_t* pair_counts);

/* Device-resident batches: upload once, run many times, read back.  The run
 * is asynchronous on `stream` (a cudaStream_t, NULL = the context stream);
 * xc_batch_results synchronises.  Used to time the kernels alone. */
int xc_batch_upload(xc_ctx* ctx, const xc_pair* pairs, size_t n, xc_batch** batch);
int xc_batch_run(xc_ctx* ctx, xc_batch* batch, void* stream);
int xc_batch_results(xc_ctx* ctx, xc_batch* batch, xc_result* out, size_t cap, size_t* n_out,
                     size_t* pair_counts);
int xc_batch_free(xc_ctx* ctx, xc_batch* batch);
/* Kernel launches one xc_batch_run makes (for launch accounting). */
int xc_batch_launches(xc_ctx* ctx, xc_batch* batch);
/* xc_batch_run with CUDA events between its stages, then a synchronise:
 * stage_ms[0] = correlation + FindTop kernels, [1] = scan kernels,
 * [2] = result ordering/packing kernels (all buckets of each stage). */
int xc_batch_run_timed(xc_ctx* ctx, xc_batch* batch, void* stream, float* stage_ms);
/* FindTop offsets the last run of a device batch kept: counts[2*i + s] for
 * caller pair i and strand s (0 forward, 1 reverse-complemented query) if
 * counts is not NULL, and the offsets (lag index j into the FFT-length
 * correlation: query index - target index = j - L/2), packed in that order
 * into offs.  *n_out gets the total; XC_ERR_CAPACITY when it exceeds cap.
 * SeqAnalyzer::FindTop's output (CrossCorr.cc:878-944), for inspection. */
int xc_batch_offsets(xc_ctx* ctx, xc_batch* batch, int* offs, size_t cap, size_t* n_out, int* counts);
/* Near-threshold lags of the last run of a device batch: lags whose FP32
 * correlation lies within XC_STRADDLE_REL (XC_STRADDLE_REL_L32768 at FFT
 * 32768) times max(1, max|xc|) of FindTop's FP32 threshold, where the
 * reference's FP32 FFT and this one can decide differently (the compare of
 * CrossCorr.cc:932).  counts[2*i + s] gets their number for caller pair i,
 * strand s; lags (if not NULL, XC_STRAD_CAP ints per pair strand) the first
 * XC_STRAD_CAP of them in increasing order, -1 after the last.  Every lag
 * outside this list is kept or dropped as an exact computation would. */
#define XC_STRAD_CAP 16
#define XC_STRADDLE_REL 2e-5
#define XC_STRADDLE_REL_L32768 3e-4
int xc_batch_straddles(xc_ctx* ctx, xc_batch* batch, int* counts, int* lags);
/* Bytes the last xc_align_pairs call (or batch upload / readback) moved:
 * host-to-device and device-to-host. */
int xc_transfer_stats(xc_ctx* ctx, uint64_t* h2d_bytes, uint64_t* d2h_bytes);

/* Serving: thread-safe submission of chunk pairs from any host thread (the
 * slave's -p workers), continuous batching on the device, and a bounded wait.
 * xc_submit returns XC_ERR_BUSY when admission is refused.  xc_wait returns
 * XC_ERR_TIMEOUT after timeout_ms without results, and XC_ERR_CAPACITY with
 * *n_out > cap when out is too small; in both cases the ticket stays valid.
 * Any other status (XC_OK included) releases the ticket. */
int xc_submit(xc_ctx* ctx, const xc_pair* pairs, size_t n, uint64_t* ticket);
int xc_wait(xc_ctx* ctx, uint64_t ticket, int timeout_ms, xc_result* out, size_t cap,
            size_t* n_out);
/* Latency statistics of completed tickets (submit -> results ready), ms. */
int xc_serving_stats(xc_ctx* ctx, double* p50_ms, double* p99_ms, uint64_t* completed,
                     uint64_t* pairs_done);

/* Stage outputs for tests, one pair: signals (strand s, sequence k in
 * {target, query or reverse-complemented query}, channel c at
 * sig[((s*2+k)*4+c)*L + i], i < L/2), the correlation xc[s*L + i], FindTop
 * offsets offs[s*L + j] with n_offs[s], and raw DoOne segments (tStart,
 * qStart, len) at segs[(s*seg_cap + j)*3] with n_segs[s].  Any output may be
 * NULL.  *fft_len_out gets the FFT length L used; size sig for 16*L floats,
 * xc for 2*L and offs for 2*L ints (L <= 32768). */
int xc_debug_pair(xc_ctx* ctx, const xc_pair* pair, float* sig, float* xc, int* offs,
                  int* n_offs, int* segs, int* n_segs, int seg_cap, int* fft_len_out);

/* One chunk pair, both strands, through the same kernels as
 * xc_align_pairs(ctx, pair, 1, ...) and with the same records, but without
 * allocating any device or pinned host memory.  No counterpart in the
 * reference: it is for callers that cannot call cudaMalloc -- a process whose
 * device memory belongs to another allocator (a framework's caching allocator
 * or a fixed arena holding the free HBM), and latency-bound callers sharing
 * the GPU, for whom cudaFree's device-wide synchronisation is not acceptable.
 * The chunks, the kernels' scratch and the results before read-back live in
 * one static device array of 320 KiB that every GPU loading the library holds
 * until exit.  Limits: FFT length at most 16384 (else XC_ERR_UNSUPPORTED) and
 * at most 1024 kept matches per strand (else XC_ERR_CAPACITY, with *n_out the
 * number of matches found).  The first call through a context looks the array
 * up (cudaGetSymbolAddress) with the context's device current; make that
 * first call before any stream capture.  Calls share the array: each clears
 * what must start at zero, and calls in one process serialise and return only
 * when their results are on the host; calls that overlapped on the GPU would
 * race on the array. */
int xc_align_pair_noalloc(xc_ctx* ctx, const xc_pair* pair, xc_result* out, size_t cap,
                          size_t* n_out);

/* Autotuner of the correlation stage.  For each FFT length 1024..8192 it
 * times, on a synthetic batch of that length, the kernel forms the library
 * is built with -- threads per transform and pairs per CTA: the per-strand
 * kernel with 512, 256 or 128 threads per strand at 1024..4096; at 8192 the
 * persistent both-strands kernel, the one-CTA-per-pair form or the
 * per-strand kernel -- and keeps the fastest in the context.  All forms give
 * the same results bit for bit.  It replaces FFTReal's one fixed pass plan
 * (extern/RealFFT/FFTReal.hpp:429-458).  table (if not NULL, cap bytes) gets
 * the choices as text, one line per length, with every candidate's time;
 * *table_len its length.  Takes about a second; serialises on the context. */
int xc_tune(xc_ctx* ctx, char* table, size_t cap, size_t* table_len);
/* Applies a table xc_tune wrote (lines "fft_len=L strand_threads=T" and, at
 * 8192, "pair_form=F": 2 persistent, 1 one CTA per pair, 0 per-strand only).
 * xc_create applies the file SATSUMA2_GB300_TUNING names, if set. */
int xc_apply_tuning(xc_ctx* ctx, const char* table);

/* Library version and the device it runs on. */
const char* xc_version(void);
int xc_device_name(xc_ctx* ctx, char* buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif
