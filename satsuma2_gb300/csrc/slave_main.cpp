// satsuma2_slave: a drop-in for satsuma2's HomologyByXCorrSlave whose
// per-block compute runs on the GPU library (include/satsuma2_xcorr.h).
//
// What stays as the reference slave does it (analysis/HomologyByXCorrSlave.cc):
//  * flags and defaults (:334-384): -master -port -sid -p -q -t -l -q_chunk
//    -t_chunk -min_prob -cutoff -cutoff_fast -prob_table -debug_targets, each
//    given as "-name value" (booleans "0"/"false" are false);
//  * FASTA loading (vecDNAVector::Read, DNAVector.cc:1176-1282): '>' starts a
//    record, the first whitespace-separated token of every other line is
//    sequence, letters are uppercased;
//  * chunking (ChunkManager::ChunkItSelect, SeqChunk.cc:72-165): query chunks
//    of q_chunk with no overlap, target chunks of t_chunk with t_chunk/4
//    overlap, sequences shorter than 6 skipped, all-N/X chunks emptied;
//  * targetTotal = sum of the target sequence lengths (:405-408);
//  * the slave keeps p >= 0.99 whatever -min_prob says; -min_prob is the
//    ProbTable cutoff in -prob_table mode (:76,379,415);
//  * the master protocol (:447-526): connect, send the slave id (int), the
//    result count (unsigned) and the t_result records, read a count (int;
//    -1 = finish) and that many t_pair blocks; pull while fewer than 2 x
//    threads blocks are queued;
//  * blocks are aligned query-major, target-minor (align_target, :270-300),
//    and their records appended in that order.
//
// What differs: the -p workers hand whole blocks to the library
// (xc_submit/xc_wait), which batches them on the GPU; socket reads and writes
// loop until complete; an idle slave waits on a condition instead of
// sleeping 10 s.  -device picks the GPU (default 0).  FASTQ input is not
// read (the reference detects '@' and reads FASTQ; this slave exits with a
// message).
#include <arpa/inet.h>
#include <netdb.h>
#include <netinet/in.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/socket.h>
#include <unistd.h>

#include <atomic>
#include <cctype>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "satsuma2_xcorr.h"

namespace {

// Work request and result records on the wire (WorkQueue.h:17-33).
struct Block {
  int targetFrom, targetTo, queryFrom, queryTo;
  bool fast;
  int slave_id;
  unsigned char status;
};
static_assert(sizeof(Block) == 28, "t_pair is 28 bytes");
static_assert(sizeof(xc_result) == 72, "t_result is 72 bytes");

struct Chunk {
  std::string bases;   // chunk bytes (empty when all N/X)
  int start;           // start within its sequence
  int seq;             // sequence index
};

struct Genome {
  std::vector<std::string> seqs;
  std::vector<Chunk> chunks;
};

bool read_fasta(const std::string& path, std::vector<std::string>& seqs) {
  std::ifstream in(path);
  if (!in) return false;
  std::string line;
  bool first = true;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string tok;
    if (!(ls >> tok)) continue;   // no item on the line
    if (first && tok[0] == '@') {
      fprintf(stderr, "satsuma2_slave: %s looks like FASTQ, which this slave does not read\n", path.c_str());
      return false;
    }
    first = false;
    if (tok[0] == '>') {
      seqs.emplace_back();
      continue;
    }
    if (seqs.empty()) continue;   // sequence before any header: the reference keeps no record for it
    for (char& ch : tok) ch = (char)toupper((unsigned char)ch);
    seqs.back() += tok;
  }
  return true;
}

void chunk_genome(Genome& g, int size, int overlap) {
  const int step = size - overlap;
  for (int i = 0; i < (int)g.seqs.size(); i++) {
    const int l = (int)g.seqs[i].size();
    if (l < 6) continue;
    const int n = 1 + l / step;
    for (int j = 0; j < n; j++) {
      const int start = j * step;
      const int end = std::min((j + 1) * step + overlap, l);
      Chunk c;
      c.start = start;
      c.seq = i;
      if (end > start) c.bases = g.seqs[i].substr(start, end - start);
      int ns = 0;
      for (char ch : c.bases) ns += ch == 'N' || ch == 'X';
      if (ns >= (int)c.bases.size()) c.bases.clear();
      g.chunks.push_back(std::move(c));
    }
  }
}

bool send_all(int fd, const void* p, size_t n) {
  const char* b = static_cast<const char*>(p);
  while (n) {
    const ssize_t k = write(fd, b, n);
    if (k <= 0) return false;
    b += k;
    n -= (size_t)k;
  }
  return true;
}

bool recv_all(int fd, void* p, size_t n) {
  char* b = static_cast<char*>(p);
  while (n) {
    const ssize_t k = read(fd, b, n);
    if (k <= 0) return false;
    b += k;
    n -= (size_t)k;
  }
  return true;
}

struct Slave {
  Genome target, query;
  xc_ctx* ctx = nullptr;
  std::mutex qmu;
  std::condition_variable qcv;    // a block was queued or taken
  std::deque<Block> blocks;
  std::mutex rmu;
  std::vector<xc_result> results;
  std::atomic<bool> finished{false};
  std::atomic<int> errors{0};

  void align_block(const Block& b) {
    std::vector<xc_pair> pairs;
    for (int qi = b.queryFrom; qi <= b.queryTo; qi++)
      for (int ti = b.targetFrom; ti <= b.targetTo; ti++) {
        if (qi < 0 || ti < 0 || qi >= (int)query.chunks.size() || ti >= (int)target.chunks.size()) continue;
        const Chunk& t = target.chunks[ti];
        const Chunk& q = query.chunks[qi];
        xc_pair p;
        p.tseq = t.bases.data();
        p.tlen = (int)t.bases.size();
        p.t_chunk_start = t.start;
        p.target_id = (unsigned long)t.seq;
        p.qseq = q.bases.data();
        p.qlen = (int)q.bases.size();
        p.q_chunk_start = q.start;
        p.query_id = (unsigned long)q.seq;
        p.query_size = (unsigned long)query.seqs[q.seq].size();
        p.fast = b.fast ? 1 : 0;
        pairs.push_back(p);
      }
    if (pairs.empty()) return;
    uint64_t ticket = 0;
    int r;
    while ((r = xc_submit(ctx, pairs.data(), pairs.size(), &ticket)) == XC_ERR_BUSY)
      std::this_thread::sleep_for(std::chrono::microseconds(500));
    if (r != XC_OK) {
      fprintf(stderr, "satsuma2_slave: xc_submit failed (%d)\n", r);
      errors++;
      return;
    }
    std::vector<xc_result> out(64 * pairs.size());
    size_t n = 0;
    for (;;) {
      r = xc_wait(ctx, ticket, 1000, out.data(), out.size(), &n);
      if (r == XC_ERR_TIMEOUT) continue;             // the ticket stays valid
      if (r == XC_ERR_CAPACITY && n > out.size()) {   // buffer too small: the ticket stays valid
        out.resize(n);
        continue;
      }
      break;   // done, or failed: a failed ticket is released and never waited on again
    }
    if (r != XC_OK) {
      fprintf(stderr, "satsuma2_slave: block failed (%d)\n", r);
      errors++;
      return;
    }
    std::lock_guard<std::mutex> lk(rmu);
    results.insert(results.end(), out.begin(), out.begin() + n);
  }

  void worker() {
    while (!finished) {
      Block b;
      {
        std::unique_lock<std::mutex> lk(qmu);
        if (blocks.empty()) {
          qcv.wait_for(lk, std::chrono::seconds(1));
          continue;
        }
        b = blocks.front();
        blocks.pop_front();
      }
      qcv.notify_all();
      align_block(b);
    }
  }
};

int connect_master(const std::string& host, int port) {
  addrinfo hints;
  memset(&hints, 0, sizeof(hints));
  hints.ai_family = AF_INET;
  hints.ai_socktype = SOCK_STREAM;
  addrinfo* res = nullptr;
  if (getaddrinfo(host.c_str(), std::to_string(port).c_str(), &hints, &res) != 0 || !res) return -1;
  const int fd = socket(res->ai_family, res->ai_socktype, res->ai_protocol);
  if (fd >= 0 && connect(fd, res->ai_addr, res->ai_addrlen) != 0) {
    close(fd);
    freeaddrinfo(res);
    return -1;
  }
  freeaddrinfo(res);
  return fd;
}

}  // namespace

int main(int argc, char** argv) {
  std::map<std::string, std::string> a;
  for (int i = 1; i + 1 < argc; i += 2) a[argv[i]] = argv[i + 1];
  auto str = [&](const char* k, const char* d) -> std::string {
    auto it = a.find(k);
    if (it != a.end()) return it->second;
    if (!d) {
      fprintf(stderr, "need to specify %s\n", k);
      exit(255);
    }
    return d;
  };
  auto num = [&](const char* k, const char* d) { return atof(str(k, d).c_str()); };
  const std::string master = str("-master", nullptr);
  const int port = (int)num("-port", "3491");   // MYPORT (WorkQueue.h:40)
  const int slave_id = (int)num("-sid", nullptr);
  const int threads = std::max(1, (int)num("-p", "1"));
  const std::string qfile = str("-q", nullptr), tfile = str("-t", nullptr);
  const int min_len = (int)num("-l", "0");
  const int q_chunk = (int)num("-q_chunk", "4096");
  const int t_chunk = (int)num("-t_chunk", "4096");
  const double min_prob = num("-min_prob", "0.9999");
  const double cutoff = num("-cutoff", "1.8");
  const double cutoff_fast = num("-cutoff_fast", "2.9");
  const std::string pt = str("-prob_table", "false");
  const bool prob_table = !(pt == "0" || pt == "false");
  const unsigned debug_targets = (unsigned)num("-debug_targets", "0");
  const int device = (int)num("-device", "0");
  if (q_chunk > t_chunk) {
    // the reference sizes every signal 2*t_chunk, so longer query chunks overrun it
    fprintf(stderr, "satsuma2_slave: -q_chunk %d larger than -t_chunk %d is not supported\n", q_chunk, t_chunk);
    return 255;
  }

  Slave S;
  if (!read_fasta(qfile, S.query.seqs) || !read_fasta(tfile, S.target.seqs)) {
    fprintf(stderr, "satsuma2_slave: cannot read %s or %s\n", qfile.c_str(), tfile.c_str());
    return 255;
  }
  chunk_genome(S.query, q_chunk, 0);
  chunk_genome(S.target, t_chunk, t_chunk / 4);
  double target_total = 0;
  for (const std::string& s : S.target.seqs) target_total += (double)s.size();
  printf("satsuma2_slave: %zu target chunks, %zu query chunks, targetTotal %.0f\n", S.target.chunks.size(),
         S.query.chunks.size(), target_total);

  xc_params prm;
  memset(&prm, 0, sizeof(prm));
  prm.cutoff = cutoff;
  prm.cutoff_fast = cutoff_fast;
  prm.min_prob = 0.99;            // the slave's fixed m_minProb
  prm.target_total = target_total;
  prm.min_len = min_len;
  prm.t_chunk = t_chunk;
  prm.q_chunk = q_chunk;
  prm.fft_len = 0;                // 2 * t_chunk, as create_signals sizes them
  prm.use_prob_table = prob_table ? 1 : 0;
  prm.prob_table_cutoff = min_prob;
  prm.max_batch = 4096;
  prm.result_slots = 64;
  int r = xc_create(&prm, device, &S.ctx);
  if (r != XC_OK) {
    fprintf(stderr, "satsuma2_slave: no GPU context (%d)\n", r);
    return 255;
  }

  std::vector<std::thread> workers;
  for (int w = 0; w < threads; w++) workers.emplace_back([&S] { S.worker(); });

  unsigned total_targets = 0;
  while (!S.finished) {
    {
      std::unique_lock<std::mutex> lk(S.qmu);
      if (S.blocks.size() >= (size_t)(2 * threads)) {
        S.qcv.wait_for(lk, std::chrono::seconds(10));
        continue;
      }
    }
    int fd = -1;
    while (fd < 0) {
      fd = connect_master(master, port);
      if (fd < 0 || !send_all(fd, &slave_id, sizeof(slave_id))) {
        if (fd >= 0) close(fd);
        fd = -1;
        fprintf(stderr, "satsuma2_slave: cannot reach the master, retrying\n");
        sleep(1);
      }
    }
    std::vector<xc_result> out;
    {
      std::lock_guard<std::mutex> lk(S.rmu);
      out.swap(S.results);
    }
    const unsigned cnt = (unsigned)out.size();
    int target_count = 0;
    const bool sent = send_all(fd, &cnt, sizeof(cnt)) && (!cnt || send_all(fd, out.data(), cnt * sizeof(xc_result)));
    bool ok = sent && recv_all(fd, &target_count, sizeof(target_count));
    if (ok && target_count == -1) S.finished = true;
    if (ok && target_count > 0) {
      std::vector<Block> got((size_t)target_count);
      ok = recv_all(fd, got.data(), got.size() * sizeof(Block));
      if (ok) {
        std::lock_guard<std::mutex> lk(S.qmu);
        for (const Block& b : got) S.blocks.push_back(b);
      }
      S.qcv.notify_all();
    }
    close(fd);
    if (!ok) {
      // a broken exchange: results that did not go out wait for the next one
      if (!sent) {
        std::lock_guard<std::mutex> lk(S.rmu);
        S.results.insert(S.results.begin(), out.begin(), out.end());
      }
      sleep(1);
      continue;
    }
    if (target_count > 0) total_targets += (unsigned)target_count;
    if (debug_targets && total_targets >= debug_targets) S.finished = true;
  }
  for (auto& t : workers) t.join();
  xc_destroy(S.ctx);
  return S.errors ? 1 : 0;
}
