// engine.h -- host-side batch engine behind the C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <functional>
#include <vector>

#include "tsq_internal.h"

namespace tsq {

// Device buffer that only grows; reused across plans of the same object.
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaStream_t owner = nullptr;  // stream of a stream-ordered allocation
  // Grows the buffer (contents are not kept).  With a stream, a buffer below
  // async_max bytes is freed and allocated in stream order, so growing one
  // batch's buffers does not wait for other streams' work; larger ones come
  // from cudaMalloc (stream-ordered allocation maps memory far more slowly).
  cudaError_t ensure(size_t bytes, cudaStream_t stream = nullptr, size_t async_max = size_t(256) << 20);
  // Frees in the owner stream's order when there is one; the owner stream
  // must still exist.
  void release();
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
  ~DevBuf() { release(); }
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
};

// Page-locked host buffer (for results coming back asynchronously).
struct PinBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes);
  void release();
  template <class T>
  T *as() const {
    return static_cast<T *>(p);
  }
  ~PinBuf() { release(); }
  PinBuf() = default;
  PinBuf(const PinBuf &) = delete;
  PinBuf &operator=(const PinBuf &) = delete;
};

// One persistent fill launch: every warp task of one row height R and lane
// type, all lane widths G mixed, longest first.
struct Launch {
  int R = 8, i16 = 0;  // i16: 0 int32, 1 int16x2, 2 int16x2 with overflow check
  bool rerun = false;  // int32 re-run of flagged pairs (warp tasks built on the device)
  bool cta = false;    // one long pair per CTA (fill_cta.cuh); pairs tasks[task_begin, +n_wtasks)
  int32_t task_begin = 0;
  int32_t wt_begin = 0, n_wtasks = 0;  // slice of the warp-task list
  int32_t blocks = 0;
  int32_t bnd_cols = 0;
  int64_t bnd_offset = 0;  // bytes into the boundary scratch
};

// What the autotuner forces while it times one candidate: a lane width for
// every pair, and (cta) the CTA fill for every int32 pair.  Carried by the
// batch object into its plan, so the planner's worker threads see it.
struct TuneForce {
  bool shape = false;
  Shape sh{};
  bool cta = false;
};

// A tuned table's choice for a length bucket: lane width, lane type (i16: 1
// int16x2 where its range is proven or checked, 0 int32) and whether int32
// pairs take the CTA fill.
struct TunedChoice {
  Shape sh{};
  int cta = 0;
};

// Kernel-shape choice.  A tuned table (lengths -> shape) overrides the
// occupancy heuristic when loaded and enabled.
struct ShapeChooser {
  int out_mode = kOutScore;
  bool local = false;
  int sms = 152;
  int64_t npairs = 0;
  // Balanced steps per resident lane over the whole batch: no pair may need
  // more than about half of it, or it becomes the batch's tail.
  double avg_lane_steps = 0.0;
  bool use_table = false;
  TuneForce force;
  // Set by prepare() from the fields above: the occupancy lane width and
  // the reciprocal of half the balanced lane steps (the per-pair choice
  // then takes no division).
  int g_occ = 32;
  double inv_half_lane_steps = 0.0;
  void prepare();
  // rows_per_lane: 8 or 16 (a power of two).
  Shape pick(int m, int n, int rows_per_lane) const;
};

// Record of the planner's radix sorts.
struct SortRec {
  uint64_t key;
  int32_t idx;
};

// Host scratch of the planner, kept by the batch object so that repeated
// plans of similar batches neither allocate nor clear it.
struct PlanScratch {
  std::vector<int8_t> lsel;
  std::vector<int32_t> gsel, rsel, order;
  std::vector<int64_t> cost;  // bands x steps per pair
  std::vector<SortRec> recs, tmp;
  // The same per pair, gathered into sorted order.
  std::vector<int8_t> s_lt;
  std::vector<int32_t> s_g, s_cols;
  std::vector<int64_t> s_cost;
};

bool tune_table_loaded();
bool tune_table_pick(int out_mode, int m, int n, TunedChoice *c);

}  // namespace tsq

struct tsq_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  // ev[0..3]: run start, fill start, fill end, run end (inside the graph
  // when captured); ev[4..5]: around a graph launch.
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  bool capturing = false;
  cudaEvent_t ev_fetch = nullptr;  // results copied to the pinned host buffers
  cudaStream_t side = nullptr;     // the CTA launch runs here, forked from and joined to `stream`
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  tsq::Scheme scheme{};
  tsq_params params{};
  int out_mode = tsq::kOutScore;
  bool local = false;
  bool use_graph = false;
  bool autotune = false;
  int32_t wait_polls = 0;  // CTA fill: polls per bounded wait (0 = default)
  tsq::TuneForce tune_force;  // set by the autotuner for the next plan
  int64_t n = 0;
  int64_t seqs_len = 0;
  int64_t cells = 0;
  std::vector<tsq::PairDev> pairs_h;
  tsq::PlanScratch scratch;
  std::vector<tsq::Launch> launches;
  std::vector<int64_t> aln_off_h;
  int64_t aln_bytes = 0;
  bool has_run = false;
  // Chunk of a larger call: the residues and their codes live in another
  // batch object (the call's first chunk), which uploads and encodes them;
  // this object's fills wait on that object's ev_encoded.
  const tsq_batch *input_owner = nullptr;
  cudaEvent_t ev_encoded = nullptr;  // recorded after this object's encode
  // Segmented input (chunks of one call): the residues arrive in segments
  // uploaded and encoded on the caller's input stream (input_segment); the
  // fills wait on input_ready, the event after this chunk's segment.
  bool input_segmented = false;
  cudaEvent_t input_ready = nullptr;
  // Set by input_prepare: the next plan keeps the residue buffers and code
  // tables it set up.
  bool input_prepared = false;

  tsq::DevBuf seqs, codes, pairs, tasks, wtasks, res, bnd, planes, plane_off, aln, aln_off, shape_g, shape_r, counters,
      lut, matrix, overflow, rerun_tasks, rerun_wtasks;
  // Score classes for the int16x2 fill (score output only).
  tsq::DevBuf ccodes, clut, cmatrix;
  bool classes = false;
  tsq::PinBuf res_h, aln_h, rerun_h;
  // Device buffers below this size grow in stream order.  A serving slot,
  // whose growth must not wait for the other slots' kernels, takes every
  // size in stream order; a one-off large batch prefers cudaMalloc's faster
  // mapping of its traceback planes.
  size_t async_max = size_t(256) << 20;
  // Frees every device buffer (in stream order) before the streams go.
  void release_device_buffers();
  int64_t n_checked = 0;
  int32_t checked_begin = 0;

  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  tsq_batch_stats stats{};

  ~tsq_batch();
};

namespace tsq {
int batch_plan(tsq_batch *b, const uint8_t *seqs, int64_t seqs_len, const tsq_pair_desc *pairs, int64_t n,
               const tsq_params *p, const tsq_batch_opts *opts, bool plain);
// Plans one chunk of a larger call.  The first chunk (owner == nullptr)
// uploads and encodes the residues; later chunks use the owner's, and
// their pair offsets refer to them.  call_pairs / call_cells are the whole
// call's totals, so that every pair gets the lane width a single plan of the
// call would give it.
int batch_plan_chunk(tsq_batch *b, const tsq_batch *owner, const uint8_t *seqs, int64_t seqs_len,
                     const tsq_pair_desc *pairs, int64_t n, const tsq_params *p, const tsq_batch_opts *opts,
                     int64_t call_pairs, int64_t call_cells, bool segmented);
// Uploads residues [begin, end) of `seqs` into the owner's device buffers and
// encodes them, on `stream`; begin is a multiple of 16.  The owner must be
// planned (its code tables are on the device).
int input_segment(const tsq_batch *owner, const uint8_t *seqs, int64_t begin, int64_t end, cudaStream_t stream);
// Readies the first chunk's object of a call to receive seqs_len residues
// before it is planned: its device buffers, and the code tables for the
// parameters, usable from any stream on return.  Its next plan (with
// segmented input) keeps them, so input_segment can upload and encode the
// whole input while the host plans.
int input_prepare(tsq_batch *owner, int64_t seqs_len, const tsq_params *p, const tsq_batch_opts *opts);
// Encodes the owner's whole input (owner->seqs_len residues) on `stream`
// straight from memory the device reads in place (a page-locked host buffer
// through its device address, 16-byte aligned); the owner keeps no copy of
// the residues, which score and identity fills do not read.
int input_encode_mapped(const tsq_batch *owner, const uint8_t *src_dev, cudaStream_t stream);
int batch_run_async(tsq_batch *b);
int batch_sync(tsq_batch *b);
int batch_results(tsq_batch *b, tsq_result *out);
// The same, pair q's result going to out[dst[q]].
int batch_results(tsq_batch *b, tsq_result *out, const int32_t *dst);
// Asynchronous read-back: enqueue the copies, poll, then convert a range.
int batch_fetch_async(tsq_batch *b);
int batch_fetch_query(tsq_batch *b);  // TSQ_OK when the copies landed, TSQ_E_PENDING before
int batch_collect(tsq_batch *b, int64_t begin, int64_t count, tsq_result *out, const int32_t *dst = nullptr);
// Orders a call's pairs by cost, costliest first: cells binned at four steps
// per octave, bins descending, input order within a bin.  Writes the pairs
// in that order and each one's input index; returns the total cells.
// Parallel on the worker pool; `bin` is scratch.
int64_t cost_order(const tsq_pair_desc *pairs, int64_t n, std::vector<uint8_t> &bin, tsq_pair_desc *out_pairs,
                   int32_t *out_index);

// ---- per-pair rules shared by the planner and the one-pair path ----------
// Rows per lane of every fill.
constexpr int kFillRows = 8;
// Longest sequence the int32 kernels take: coordinates travel in 20 bits.
constexpr int64_t kMaxPairLen = (1 << 20) - 1;
int out_mode_of(const tsq_params *p);
bool lanes16_possible(int out_mode, bool local, int lane);
// TSQ_E_INVALID_ARG for gap costs, mode, output or lane out of range.
int check_params(const tsq_params *p);
// TSQ_E_TOO_LARGE for a pair beyond the kernels' value and length ranges.
int pair_limits(const tsq_params *p, const Scheme &sc, int out_mode, int32_t a_len, int32_t b_len);
// Whether a pair's int16x2 values provably stay in range: lower (its most
// negative values above the kernels' minus infinity) and upper (its best
// score below 32767, so the fill needs no overflow check).
struct Range16 {
  bool lower = false, upper = false;
};
Range16 range16(const tsq_params *p, const Scheme &sc, int32_t a_len, int32_t b_len);
// Copies a result record into o and, when rows is set (an alignment whose
// status is OK), its two rows from the walker's output of 2 * cap bytes.
// Returns TSQ_OK, or TSQ_E_CUDA / TSQ_E_NOMEM when the rows cannot be taken.
int collect_one(const ResultDev &d, const char *rows, int64_t cap, tsq_result &o);

// The plain form's one-pair path (pair.cpp).  One object per host thread.
struct PairPath {
  int device = -1;
  int sms = 0;
  cudaStream_t stream = nullptr;
  DevBuf dev;       // upload block | codes | class codes | result | rows | boundary | planes
  PinBuf up, down;  // the upload block; the result record and rows coming back
  void reset();     // frees the buffers and the stream (device change)
  ~PairPath() { reset(); }
};
// A tsq_align_pair call the one-pair path does not take returns this; the
// caller then runs the batch engine, which owns those cases' checks.
constexpr int kPairNotTaken = -1000;
int pair_align(PairPath *pp, const uint8_t *a, int32_t la, const uint8_t *b, int32_t lb, const tsq_params *p,
               tsq_result *out);
int64_t batch_device_bytes(const tsq_batch *b);
// Returns the memory the engine's stream-ordered pool keeps mapped on a
// device but does not use (before a call sizes itself by the free memory).
void trim_engine_pool(int device);
// Runs task(i) for i in [0, tasks) on the planner's host worker pool (in
// turn on the calling thread when the pool is busy).
void run_tasks(int tasks, const std::function<void(int)> &task);
int cuda_status(cudaError_t e);
}  // namespace tsq
