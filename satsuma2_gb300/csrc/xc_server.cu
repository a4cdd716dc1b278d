// Serving: thread-safe submission of chunk-pair requests with continuous
// batching on one GPU.
//
// The slave's -p worker threads (HomologyByXCorrSlave.cc:302-319) each popped
// a t_pair block and ran it alone.  Here any number of host threads call
// xc_submit; a scheduler thread packs waiting pairs -- across request
// boundaries -- into the next free in-flight slot (its own stream and buffers)
// and launches it while earlier slots are still running, so work that arrives
// while the GPU is busy joins the next launch.  Requests are admitted against
// a budget of queued pairs and of the device memory their batches need
// (measured with cudaMemGetInfo when the server starts); xc_submit answers
// XC_ERR_BUSY beyond it.  xc_wait is bounded: it returns XC_ERR_TIMEOUT and
// keeps the ticket.  No device code waits on the host or on other kernels.
//
// What overlaps on the device: a slot's host packing and host-to-device copy
// run while the previous slot's kernels run, and its read-back while the next
// slot's kernels run; the kernels of successive slots themselves run one batch
// after another (see the scheduler).  A batch whose result overflow pool fills
// is grown and run again by the scheduler, so one request's yield never fails
// the requests batched with it.
#include "satsuma2_xcorr.h"
#include "xc_runtime.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>

namespace xc {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  std::vector<char> bytes;
  std::vector<xc_pair> pairs;
  size_t next = 0;          // next pair to schedule
  size_t done = 0;          // pairs with results
  // Results in pair order: a request's pairs are scheduled in order and
  // batches retire oldest first, so each batch appends the next ones.
  std::vector<xc_result> results;
  int status = XC_OK;
  bool complete = false;
  size_t footprint = 0;     // device bytes accounted at admission
  Clock::time_point t_submit, t_done;
};

struct Server;

struct Slot {
  Server* S = nullptr;
  Batch* b = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;
  cudaEvent_t kend = nullptr;   // this slot's kernels done
  std::vector<std::pair<Request*, size_t>> items;
  std::vector<xc_pair> pairs;
  bool busy = false;
  uint64_t seq = 0;
};

constexpr int NSLOTS = 3;
constexpr size_t LAT_RING = 1 << 16;   // latencies kept for the percentiles: the last 65536 requests

struct Server {
  Ctx* ctx = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, Request*> reqs;
  uint64_t next_ticket = 1;
  size_t queued_pairs = 0, queued_bytes = 0;
  size_t max_pairs = 0, budget_bytes = 0;
  bool stop = false;
  std::thread sched;
  Slot slots[NSLOTS];
  uint64_t launch_seq = 0;
  cudaEvent_t last_kend = nullptr;   // kernels of the last launched batch done
  std::vector<double> lat_ms;        // ring of the last LAT_RING request latencies
  size_t lat_next = 0;
  uint64_t slots_done = 0;           // bumped by the stream callback of each finished slot
  uint64_t completed = 0, pairs_done = 0;
  int device = 0;
  size_t max_batch = 4096;
  size_t min_batch = 1024;   // while the GPU is busy, wait for this many pairs ...
  double max_wait_ms = 1.0;  // ... or for the oldest request to wait this long
  size_t res_per_pair = 8;   // read-back buffer estimate (records per pair)
};

// Device bytes one pair needs inside a batch (sequences, offsets, results).
static size_t pair_footprint(const Ctx* c, const xc_pair& p, int slots) {
  const int lg = pair_log2L(c->prm, p);
  const size_t L = lg > 0 ? (size_t)1 << lg : 8192;
  return (size_t)p.tlen + p.qlen + 32 + 2 * L * sizeof(int) + 2 * (size_t)slots * 2 * sizeof(DevResult) + 64 +
         2 * acc_stride(lg > 0 ? lg : 13) * sizeof(float2);
}

// Stream callback queued behind each slot's read-back: wakes the scheduler
// (no CUDA call here, as host functions on a stream require).
static void CUDART_CB slot_finished(void* arg) {
  Slot* sl = static_cast<Slot*>(arg);
  {
    std::lock_guard<std::mutex> lk(sl->S->mu);
    sl->S->slots_done++;
  }
  sl->S->cv_work.notify_all();
}

static void record_latency(Server* S, double ms) {
  if (S->lat_ms.size() < LAT_RING) S->lat_ms.push_back(ms);
  else S->lat_ms[S->lat_next] = ms;
  S->lat_next = (S->lat_next + 1) % LAT_RING;
}

static void complete_slot(Server* S, Slot& sl) {
  const size_t n = sl.items.size();
  std::vector<size_t> counts(n);
  size_t need = 0;
  // one read-back into a buffer sized from the last batch's yield; a second
  // only when it was too small
  std::vector<xc_result> res(std::max<size_t>(S->res_per_pair * n + 1024, 4096));
  int r = batch_collect(S->ctx, sl.b, sl.s, res.data(), res.size(), &need, counts.data());
  // the batch's device overflow pool filled: grow it and run the batch again,
  // so every request in it gets its full results
  if (r == XC_INTERNAL_OVERFLOW) r = batch_rerun_overflow(S->ctx, sl.b, sl.s, res.data(), res.size(), &need, counts.data());
  if (r == XC_ERR_CAPACITY && need > res.size()) {
    res.resize(need);
    r = batch_collect(S->ctx, sl.b, sl.s, res.data(), res.size(), &need, counts.data());
  }
  if (r == XC_OK && n) S->res_per_pair = std::max<size_t>(4, 2 * need / n);
  const auto now = Clock::now();
  std::lock_guard<std::mutex> lk(S->mu);
  size_t o = 0;
  for (size_t i = 0; i < n; i++) {
    Request* q = sl.items[i].first;
    if (r == XC_OK) {
      // one append per run of this request's consecutive pairs
      size_t j = i, cnt = 0;
      while (j < n && sl.items[j].first == q) cnt += counts[j++];
      q->results.insert(q->results.end(), res.begin() + o, res.begin() + o + cnt);
      o += cnt;
      for (; i + 1 < j; i++) q->done++;   // all but the last of the run; the last below
    } else {
      q->status = r;
    }
    q->done++;
    if (q->done == q->pairs.size() && !q->complete) {
      q->complete = true;
      q->t_done = now;
      record_latency(S, std::chrono::duration<double, std::milli>(now - q->t_submit).count());
      S->completed++;
      S->pairs_done += q->pairs.size();
      S->queued_bytes -= std::min(S->queued_bytes, q->footprint);
    }
  }
  sl.items.clear();
  sl.busy = false;
  S->cv_done.notify_all();
}

static void scheduler(Server* S) {
  cudaSetDevice(S->device);
  for (;;) {
    // 1. retire finished slots, oldest first
    for (;;) {
      Slot* oldest = nullptr;
      for (auto& sl : S->slots)
        if (sl.busy && (!oldest || sl.seq < oldest->seq)) oldest = &sl;
      if (!oldest) break;
      if (cudaEventQuery(oldest->ev) != cudaSuccess) break;
      complete_slot(S, *oldest);
    }
    // 2. fill a free slot from the queue: at once while at most one batch
    //    is in flight, otherwise once a batch worth launching has gathered
    //    (or the oldest request has waited long enough)
    Slot* free_slot = nullptr;
    int busy = 0;
    for (auto& sl : S->slots) {
      busy += sl.busy;
      if (!sl.busy && !free_slot) free_slot = &sl;
    }
    bool launched = false, holding = false;
    if (free_slot) {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->stop && S->queue.empty() && busy == 0) return;
      if (busy >= 2 && !S->queue.empty() && S->queued_pairs < S->min_batch &&
          std::chrono::duration<double, std::milli>(Clock::now() - S->queue.front()->t_submit).count() <
              S->max_wait_ms) {
        holding = true;
        lk.unlock();
      }
    }
    if (free_slot && !holding) {
      std::unique_lock<std::mutex> lk(S->mu);
      free_slot->items.clear();
      free_slot->pairs.clear();
      while (!S->queue.empty() && free_slot->pairs.size() < S->max_batch) {
        Request* q = S->queue.front();
        while (q->next < q->pairs.size() && free_slot->pairs.size() < S->max_batch) {
          free_slot->items.emplace_back(q, q->next);
          free_slot->pairs.push_back(q->pairs[q->next]);
          q->next++;
        }
        if (q->next == q->pairs.size()) S->queue.pop_front();
      }
      S->queued_pairs -= std::min(S->queued_pairs, free_slot->pairs.size());
      lk.unlock();
      if (!free_slot->pairs.empty()) {
        int r = batch_pack(S->ctx, free_slot->b, free_slot->pairs.data(), free_slot->pairs.size(), free_slot->s);
        // The slots' kernels run one batch after another: the host-to-device
        // copy above still overlaps the batch before, but two batches' kernels
        // sharing the SMs ran 27% slower (a correlation CTA needs a whole SM's
        // shared memory, so it waits for every scan CTA there to finish).
        if (r == XC_OK && S->last_kend && cudaStreamWaitEvent(free_slot->s, S->last_kend, 0) != cudaSuccess)
          r = XC_ERR_CUDA;
        if (r == XC_OK) r = batch_run(S->ctx, free_slot->b, free_slot->s, false);
        if (r == XC_OK && cudaEventRecord(free_slot->kend, free_slot->s) != cudaSuccess) r = XC_ERR_CUDA;
        if (r == XC_OK) S->last_kend = free_slot->kend;
        if (r == XC_OK) r = batch_readback_async(S->ctx, free_slot->b, free_slot->s);
        if (r == XC_OK && cudaEventRecord(free_slot->ev, free_slot->s) != cudaSuccess) r = XC_ERR_CUDA;
        if (r == XC_OK && cudaLaunchHostFunc(free_slot->s, slot_finished, free_slot) != cudaSuccess) r = XC_ERR_CUDA;
        free_slot->busy = true;
        free_slot->seq = ++S->launch_seq;
        if (r != XC_OK) {
          std::lock_guard<std::mutex> lk2(S->mu);
          for (auto& it : free_slot->items) {
            it.first->status = r;
            it.first->done++;
            if (it.first->done == it.first->pairs.size()) {
              it.first->complete = true;
              it.first->t_done = Clock::now();
            }
          }
          free_slot->items.clear();
          free_slot->busy = false;
          S->cv_done.notify_all();
        }
        launched = true;
      }
    }
    if (launched) continue;
    // 3. idle: sleep until a slot's stream callback reports it finished, new
    //    work arrives for a free slot, or a held batch's wait runs out
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->stop && S->queue.empty() && busy == 0) return;
      const uint64_t seen = S->slots_done;
      auto limit = std::chrono::milliseconds(5);   // a bound only: every wake-up has a cause above
      if (holding && !S->queue.empty()) {
        const double left = S->max_wait_ms -
            std::chrono::duration<double, std::milli>(Clock::now() - S->queue.front()->t_submit).count();
        limit = std::min(limit, std::chrono::milliseconds((long)std::max(0.0, std::ceil(left))));
      }
      const bool can_take = free_slot != nullptr && !holding;
      S->cv_work.wait_for(lk, limit, [&] {
        return S->stop || S->slots_done != seen || (can_take && !S->queue.empty());
      });
    }
  }
}

static int server_start(Ctx* c) {
  if (c->server) return XC_OK;
  Server* S = new Server();
  S->ctx = c;
  S->device = c->device;
  S->max_batch = c->prm.max_batch > 0 ? (size_t)c->prm.max_batch : 4096;
  size_t free_b = 0, total_b = 0;
  cudaSetDevice(c->device);
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    delete S;
    return XC_ERR_CUDA;
  }
  S->budget_bytes = free_b / 2;
  S->max_pairs = 64 * S->max_batch;
  S->min_batch = std::min<size_t>(S->max_batch, 1024);
  for (auto& sl : S->slots) {
    sl.S = S;
    sl.b = new_batch(c);
    if (cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.kend, cudaEventDisableTiming) != cudaSuccess) {
      delete S;
      return XC_ERR_CUDA;
    }
  }
  S->sched = std::thread(scheduler, S);
  c->server = S;
  return XC_OK;
}

void server_stop(Ctx* c) {
  Server* S = c->server;
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->queue.clear();
  }
  S->cv_work.notify_all();
  if (S->sched.joinable()) S->sched.join();
  for (auto& sl : S->slots) {
    if (sl.s) cudaStreamSynchronize(sl.s);
    delete sl.b;
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.kend) cudaEventDestroy(sl.kend);
    if (sl.s) cudaStreamDestroy(sl.s);
  }
  for (auto& kv : S->reqs) delete kv.second;
  delete S;
  c->server = nullptr;
}

}  // namespace xc

using namespace xc;

extern "C" {

int xc_submit(xc_ctx* c, const xc_pair* pairs, size_t n, uint64_t* ticket) {
  if (!c || !ticket || (!pairs && n) || n == 0) return XC_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(c->mu);
    int r = server_start(c);
    if (r != XC_OK) return r;
  }
  Server* S = c->server;
  // copy the caller's sequences (valid only during this call); a chunk the
  // request passes several times by the same pointer and length (a block's
  // chunks) is copied once, so its pairs share it downstream
  Request* q = new Request();
  size_t bytes = 0;
  size_t hsize = 16;
  while (hsize < 4 * n) hsize *= 2;
  std::vector<HashSlot> ht(hsize, HashSlot{nullptr, 0, 0});   // open addressing: (pointer, length) -> copy
  std::vector<std::pair<const char*, int>> srcs;               // distinct chunks, in copy order
  std::vector<size_t> offs;
  std::vector<std::pair<size_t, size_t>> where(n);   // byte offsets of each pair's target and query copy
  for (size_t i = 0; i < n; i++) {
    if (pairs[i].tlen < 0 || pairs[i].qlen < 0) {
      delete q;
      return XC_ERR_ARG;
    }
    const int lg = pair_log2L(c->prm, pairs[i]);
    if (lg < MIN_LOG2L || lg > MAX_LOG2L) {
      delete q;
      return XC_ERR_UNSUPPORTED;
    }
    if (pairs[i].tlen > (1 << lg) / 2 || pairs[i].qlen > (1 << lg) / 2) {
      delete q;
      return XC_ERR_INPUT;
    }
    auto at = [&](const char* ptr, int len) -> size_t {
      if (len == 0) return bytes;
      for (size_t h = (((uint64_t)(uintptr_t)ptr * 0x9E3779B97F4A7C15ull) ^ (uint64_t)len * 0xC2B2AE3D27D4EB4Full) >> 20;;
           h++) {
        HashSlot& sl = ht[h & (hsize - 1)];
        if (!sl.p) {
          sl.p = ptr;
          sl.len = len;
          sl.uid = (uint32_t)srcs.size();
          srcs.emplace_back(ptr, len);
          offs.push_back(bytes);
          bytes += (size_t)len;
          return bytes - (size_t)len;
        }
        if (sl.p == ptr && sl.len == len) return offs[sl.uid];
      }
    };
    where[i].first = at(pairs[i].tseq, pairs[i].tlen);
    where[i].second = at(pairs[i].qseq, pairs[i].qlen);
    q->footprint += pair_footprint(c, pairs[i], S->slots[0].b->slots);
  }
  q->bytes.resize(bytes);
  for (size_t k = 0; k < srcs.size(); k++) memcpy(&q->bytes[offs[k]], srcs[k].first, (size_t)srcs[k].second);
  q->pairs.assign(pairs, pairs + n);
  for (size_t i = 0; i < n; i++) {
    xc_pair& p = q->pairs[i];
    p.tseq = q->bytes.data() + where[i].first;
    p.qseq = q->bytes.data() + where[i].second;
  }
  q->results.reserve(n * 4);
  std::unique_lock<std::mutex> lk(S->mu);
  if (S->stop) {
    delete q;
    return XC_ERR_ARG;
  }
  if (S->queued_pairs + n > S->max_pairs || S->queued_bytes + q->footprint > S->budget_bytes) {
    delete q;
    return XC_ERR_BUSY;
  }
  q->ticket = S->next_ticket++;
  q->t_submit = Clock::now();
  S->queued_pairs += n;
  S->queued_bytes += q->footprint;
  S->reqs[q->ticket] = q;
  S->queue.push_back(q);
  *ticket = q->ticket;
  lk.unlock();
  S->cv_work.notify_one();
  return XC_OK;
}

int xc_wait(xc_ctx* c, uint64_t ticket, int timeout_ms, xc_result* out, size_t cap, size_t* n_out) {
  if (!c || !c->server) return XC_ERR_ARG;
  Server* S = c->server;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return XC_ERR_ARG;
  Request* q = it->second;
  const auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
  while (!q->complete) {
    if (S->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !q->complete) return XC_ERR_TIMEOUT;
  }
  if (q->status != XC_OK) {
    const int st = q->status;
    S->reqs.erase(it);
    delete q;
    return st;
  }
  const size_t need = q->results.size();
  if (n_out) *n_out = need;
  if (need > cap || (!out && need)) return XC_ERR_CAPACITY;
  if (need) memcpy(out, q->results.data(), need * sizeof(xc_result));
  S->reqs.erase(it);
  delete q;
  return XC_OK;
}

int xc_serving_stats(xc_ctx* c, double* p50, double* p99, uint64_t* completed, uint64_t* pairs_done) {
  if (!c) return XC_ERR_ARG;
  if (!c->server) {
    if (p50) *p50 = 0;
    if (p99) *p99 = 0;
    if (completed) *completed = 0;
    if (pairs_done) *pairs_done = 0;
    return XC_OK;
  }
  Server* S = c->server;
  std::vector<double> v;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    v = S->lat_ms;
    if (completed) *completed = S->completed;
    if (pairs_done) *pairs_done = S->pairs_done;
  }
  auto pct = [&](double p) {
    if (v.empty()) return 0.0;
    const size_t i = (size_t)std::min<double>((double)v.size() - 1, std::floor(p * (double)(v.size() - 1) + 0.5));
    std::nth_element(v.begin(), v.begin() + i, v.end());
    return v[i];
  };
  if (p50) *p50 = pct(0.50);
  if (p99) *p99 = pct(0.99);
  return XC_OK;
}

}  // extern "C"
