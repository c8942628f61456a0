// resident.h -- the device-resident request loop of the served form.
//
// A persistent kernel stays on the GPU and takes work from a task queue in
// device memory.  The host stages a request -- residues, pair table,
// scoring matrix, letter table, descriptor and one task per pair -- in one
// page-locked block, copies it into a device arena, the descriptor table
// and the queue asynchronously, and publishes the new queue tail in stream
// order (no host wait).  Each warp of the kernel claims tasks (one pair per
// warp, 32 lanes), writes the pair's letter codes and runs the int32 fill on
// it, writing the pair's result into the request's result array in the
// arena; after each pair it adds one to the request's done counter in
// mapped host memory, which the host reads without any device call.
// Results stay in the arena until the request is polled.
//
// Every wait is bounded: a warp that finds the queue empty for idle_polls
// polls in a row (about a microsecond apart at most) leaves the loop, and
// the kernel ends when its last warp leaves, reporting why in mapped
// memory; the host relaunches it when work arrives.  A stop flag in mapped
// memory ends it at once.
//
// Each pair runs in packed int16x2 (the fill of fill_i16.cuh on 32 lanes,
// class codes written by the kernel beside the letter codes) when the
// batch planner's range rules allow it -- checked pairs that come near
// 32767 re-run in int32 in the same warp -- and in int32 otherwise; the
// lane type travels in the task.
//
// Scope: score and identity requests (global or local, any matrix) whose
// pairs are at most kMaxLen residues long; alignment requests and longer
// pairs are served by ticks.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "engine.h"

namespace tsq {
namespace resident {

constexpr int32_t kMaxLen = 2048;     // longest sequence of a resident request
constexpr int32_t kMaxReqs = 4096;    // request slots (descriptors, done counters)
constexpr int64_t kRingCap = 1 << 20; // task queue entries
constexpr int32_t kMaxPairs = 65536;  // pairs of one resident request

// Why the kernel last ended (mapped host memory).
enum : int32_t { kRunning = 0, kIdleExit = 1, kStopped = 2 };

struct ReqDesc {  // one request, in device memory
  const uint8_t *seqs;  // ASCII residues
  uint8_t *codes;       // letter codes, written by the kernel
  const uint8_t *lut;   // byte -> letter code
  const PairDev *pairs;
  ResultDev *res;
  const int8_t *matrix;  // 26 x 26
  int32_t gap_open, gap_extend;
  int32_t local, out;
  // int16x2 lanes: class codes (written by the kernel), byte -> class,
  // the nclasses x nclasses class scores, per-pair overflow flags.
  uint8_t *ccodes;
  const uint8_t *clut;
  const int8_t *cmatrix;
  int32_t *overflow;
  int64_t seqs_len;
  int32_t nclasses, max_score;
  // Publication number: a warp keeps the matrices it copied for as long as
  // its tasks come from the same publication (a later request can sit at
  // the same arena addresses with other scores).
  uint64_t uid;
};

// Lane types of a task (bits 24.. of Task::pair).
enum : int32_t { kLaneI32 = 0, kLaneI16 = 1, kLaneI16Checked = 2 };

struct Task {  // one pair of a request
  int32_t req, pair;  // pair: index | lane type << 24
};

struct Ctl {  // device memory
  unsigned long long head, tail;
  int32_t live;  // warps still in the loop
  int32_t pad;
};

struct HostBlock {  // mapped host memory
  volatile int32_t stop;
  volatile int32_t exit_status;
  volatile uint32_t done[kMaxReqs];
};

// Arena range of one request.
struct Range {
  int64_t off = 0, bytes = 0;
};
// Arena bytes a request of seqs_len residues and n pairs takes.
int64_t arena_need(int64_t seqs_len, int64_t n);

class Loop {
 public:
  ~Loop();
  int init(int device, int64_t arena_bytes, int32_t idle_polls);
  static bool eligible(const tsq_params &p, const std::vector<tsq_pair_desc> &pairs);
  // Reserves arena space and a slot; TSQ_E_PENDING when there is no room now.
  int admit(int64_t seqs_len, int64_t n, int32_t *slot, Range *range);
  // Uploads, encodes and publishes the request's tasks; relaunches the kernel
  // if it has ended.
  int publish(int32_t slot, const Range &range, const std::vector<uint8_t> &seqs,
              const std::vector<tsq_pair_desc> &pairs, const tsq_params &p, const int8_t *custom_score,
              const uint8_t *custom_valid);
  bool done(int32_t slot, int64_t n) const { return int64_t(host_->done[slot]) >= n; }
  // Copies a finished request's results out of the arena (any host thread;
  // the range stays reserved until release).
  int fetch(const Range &range, int64_t seqs_len, int64_t n, tsq_result *out);
  void release(int32_t slot, const Range &range);
  // The host saw a request's n tasks done.
  void retired(int64_t n) { outstanding_ -= n; }
  // Notices that the kernel has ended; relaunches it while tasks remain.
  int tend();
  void shutdown();
  int64_t launches() const { return launches_; }
  int64_t idle_exits() const { return idle_exits_; }
  bool running() const { return running_; }

 private:
  int launch();
  int device_ = 0, blocks_ = 0, warps_ = 0;
  int32_t idle_polls_ = 0;
  uint8_t *arena_ = nullptr;
  int64_t arena_bytes_ = 0;
  std::vector<Range> free_;  // free ranges, by offset
  std::vector<int32_t> free_slots_;
  ReqDesc *reqs_ = nullptr;
  Task *ring_ = nullptr;
  Ctl *ctl_ = nullptr;
  int32_t *bnd_ = nullptr;
  HostBlock *host_ = nullptr;      // host address of the mapped block
  HostBlock *host_dev_ = nullptr;  // its device address
  cudaStream_t kstream_ = nullptr, ustream_ = nullptr;
  cudaEvent_t kdone_ = nullptr;
  std::unique_ptr<PinBuf[]> stages_;  // per slot: the page-locked block the request is staged in
  bool running_ = false;
  unsigned long long tail_ = 0;  // tasks published so far
  uint64_t published_ = 0;       // requests published so far
  int64_t launches_ = 0, idle_exits_ = 0;
  int64_t outstanding_ = 0;  // tasks published and not yet seen done
};

}  // namespace resident
}  // namespace tsq
