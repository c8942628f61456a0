// engine.cpp -- planning and running batches of pairs on one GPU.
//
// A plan buckets the pairs by kernel shape (lanes per pair G, rows per lane
// R), sorts every bucket by (bands, columns) descending so the groups of a
// warp get pairs of nearly the same shape and the longest pairs start first,
// and turns each bucket into one persistent launch whose warps pull pairs
// from an atomic counter.  A run is: reset the counters, encode the residues,
// one fill launch per bucket, and (alignment output) the traceback walk.
// The run can be captured once as a CUDA graph and replayed.
#include "engine.h"
#include "trace.h"

#include <algorithm>
#include <array>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <map>
#include <mutex>
#include <numeric>
#include <thread>

namespace tsq {

namespace {
void run_slices(int tasks, const std::function<void(int)> &task);

// The engine's stream-ordered allocations come from a memory pool of its
// own per device, which keeps freed memory mapped up to a release
// threshold of 40 % of the device's memory (the default pool returns it at
// every synchronisation).  Mapping is the slow part of a stream-ordered
// allocation -- about 1 ms per GB on GB300 -- so a server whose traceback
// ticks need gigabytes of planes pays it once, not per tick.
cudaMemPool_t engine_pool(int dev) {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> g(mu);
  const auto it = pools.find(dev);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  size_t free_b = 0, total_b = 0;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess || cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    if (pool) cudaMemPoolDestroy(pool);
    pool = nullptr;
  } else {
    uint64_t keep = uint64_t(double(total_b) * 0.4);
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  pools[dev] = pool;  // (nullptr: the default pool is used)
  return pool;
}

cudaMemPool_t engine_pool(cudaStream_t stream) {
  int dev = 0;
  if (cudaStreamGetDevice(stream, &dev) != cudaSuccess) {
    cudaGetLastError();
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  }
  return engine_pool(dev);
}
}  // namespace

void run_tasks(int tasks, const std::function<void(int)> &task) { run_slices(tasks, task); }

void trim_engine_pool(int device) {
  cudaMemPool_t pool = engine_pool(device);
  if (pool) cudaMemPoolTrimTo(pool, 0);
}

cudaError_t DevBuf::ensure(size_t bytes, cudaStream_t stream, size_t async_max) {
  if (bytes == 0) bytes = 16;
  if (bytes <= cap) return cudaSuccess;
  const size_t want = (bytes + 255) & ~size_t(255);
  release();
  // Stream-ordered allocation takes no device-wide synchronisation, so a
  // batch object that grows does not wait for kernels other streams run.
  // Mapping new memory that way is slow, though (measured on GB300: 16 ms
  // for 16 GB against 0.5 ms by cudaMalloc, 267 ms against 4.7 ms for
  // 200 GB), so buffers from async_max up come from cudaMalloc, whose free
  // waits for the device, and stream-ordered ones come from the engine's
  // pool, which keeps freed memory mapped for the next allocation.
  const bool async = stream && want < async_max;
  cudaError_t e = cudaSuccess;
  if (async) {
    cudaMemPool_t pool = engine_pool(stream);
    e = pool ? cudaMallocFromPoolAsync(&p, want, pool, stream) : cudaMallocAsync(&p, want, stream);
  } else {
    e = cudaMalloc(&p, want);
  }
  if (e != cudaSuccess) {
    p = nullptr;
    return e;
  }
  cap = want;
  owner = async ? stream : nullptr;
  return cudaSuccess;
}

void DevBuf::release() {
  if (p) {
    if (owner)
      cudaFreeAsync(p, owner);
    else
      cudaFree(p);
  }
  p = nullptr;
  cap = 0;
  owner = nullptr;
}

// Page-locked host blocks are pooled for the life of the process and not
// freed: allocating and freeing page-locked memory takes milliseconds per
// hundred megabytes and can wait for the device, which would stall batches
// that other threads or server slots have in flight.  Blocks come in
// power-of-two sizes from 64 KiB; a request takes the smallest idle block of
// its size class up to four times larger.  The pool keeps at most
// kPinPoolBytes of idle blocks and frees beyond that (rare: only after a
// burst of very large batches).
namespace {
constexpr size_t kPinMin = size_t(1) << 16;
constexpr size_t kPinPoolBytes = size_t(8) << 30;
// The lock and the list are never destroyed, so buffers released during
// process exit (thread-local caches) still find them.
std::mutex &g_pin_mu = *new std::mutex();
std::vector<std::pair<size_t, void *>> &g_pin_idle = *new std::vector<std::pair<size_t, void *>>();  // (size, block)
size_t g_pin_idle_bytes = 0;

size_t pin_class(size_t bytes) {
  size_t c = kPinMin;
  while (c < bytes) c <<= 1;
  return c;
}
}  // namespace

cudaError_t PinBuf::ensure(size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes <= cap) return cudaSuccess;
  release();
  const size_t want = pin_class(bytes);
  {
    std::lock_guard<std::mutex> g(g_pin_mu);
    size_t best = g_pin_idle.size();
    for (size_t k = 0; k < g_pin_idle.size(); ++k) {
      const size_t c = g_pin_idle[k].first;
      if (c >= want && c <= 4 * want && (best == g_pin_idle.size() || c < g_pin_idle[best].first)) best = k;
    }
    if (best < g_pin_idle.size()) {
      p = g_pin_idle[best].second;
      cap = g_pin_idle[best].first;
      g_pin_idle[best] = g_pin_idle.back();
      g_pin_idle.pop_back();
      g_pin_idle_bytes -= cap;
      return cudaSuccess;
    }
  }
  cudaError_t e = cudaMallocHost(&p, want);
  if (e != cudaSuccess) {
    p = nullptr;
    return e;
  }
  cap = want;
  return cudaSuccess;
}

void PinBuf::release() {
  if (p) {
    bool keep = false;
    {
      std::lock_guard<std::mutex> g(g_pin_mu);
      if (g_pin_idle_bytes + cap <= kPinPoolBytes) {
        g_pin_idle.emplace_back(cap, p);
        g_pin_idle_bytes += cap;
        keep = true;
      }
    }
    if (!keep) cudaFreeHost(p);
  }
  p = nullptr;
  cap = 0;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return TSQ_OK;
  if (e == cudaErrorMemoryAllocation) return TSQ_E_NOMEM;
  return TSQ_E_CUDA;
}

#define TSQ_TRY(expr)                          \
  do {                                         \
    const cudaError_t e_ = (expr);             \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

namespace {

int pow2ceil(int64_t x) {
  if (x <= 1) return 1;
  if (x >= (int64_t(1) << 30)) return 1 << 30;
  return 1 << (64 - __builtin_clzll(uint64_t(x - 1)));
}

constexpr int kR = kFillRows;
constexpr int64_t kMaxLen = kMaxPairLen;

// A small pool of host worker threads for the planner's per-pair passes,
// started on first use and kept for the life of the process (spawning
// threads per plan costs as much as the work).  One job at a time: a caller
// that finds the pool busy runs its job alone.
class WorkerPool {
 public:
  static WorkerPool &get() {
    static WorkerPool pool;
    return pool;
  }
  int workers() const { return int(threads_.size()); }
  // Runs task(i) for i in [0, tasks) on the workers and the calling thread.
  // False (nothing run) when another job holds the pool.
  bool run(int tasks, const std::function<void(int)> &task) {
    std::unique_lock<std::mutex> busy(busy_, std::try_to_lock);
    if (!busy.owns_lock()) return false;
    {
      std::lock_guard<std::mutex> g(mu_);
      task_ = &task;
      tasks_ = tasks;
      next_.store(0);
      left_ = tasks;
      gen_.fetch_add(1);
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> g(mu_);
    done_.wait(g, [&] { return left_ == 0; });
    task_ = nullptr;
    return true;
  }

 private:
  WorkerPool() {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int n = int(std::min(7u, hw > 1 ? hw - 1 : 0u));
    for (int i = 0; i < n; ++i) threads_.emplace_back([this] { loop(); });
  }
  ~WorkerPool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
      stop_flag_.store(true);
    }
    cv_.notify_all();
    for (std::thread &t : threads_) t.join();
  }
  void work() {
    for (;;) {
      const int i = next_.fetch_add(1);
      if (i >= tasks_) return;
      (*task_)(i);
      std::lock_guard<std::mutex> g(mu_);
      if (--left_ == 0) done_.notify_all();
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      // A plan runs several passes in a row: after a job, poll for the next
      // one for about 50 microseconds before sleeping (waking a sleeping
      // worker costs tens of microseconds per pass).
      const auto t0 = std::chrono::steady_clock::now();
      while (gen_.load(std::memory_order_acquire) == seen && !stop_flag_.load(std::memory_order_relaxed) &&
             std::chrono::steady_clock::now() - t0 < std::chrono::microseconds(50)) {
      }
      {
        std::unique_lock<std::mutex> g(mu_);
        cv_.wait(g, [&] { return stop_ || gen_.load() != seen; });
        if (stop_) return;
        seen = gen_.load();
      }
      work();
    }
  }
  std::vector<std::thread> threads_;
  std::mutex busy_, mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)> *task_ = nullptr;
  int tasks_ = 0, left_ = 0;
  std::atomic<int> next_{0};
  std::atomic<uint64_t> gen_{0};
  bool stop_ = false;
  std::atomic<bool> stop_flag_{false};
};

// Runs f(begin, end, slot) over [0, n) in up to 8 slices (slot = slice
// number) on the worker pool; one slice when n is small or the pool is busy.
template <class F>
int parallel_for(int64_t n, F &&f) {
  WorkerPool &pool = WorkerPool::get();
  const int slices = int(std::min<int64_t>({8, int64_t(pool.workers()) + 1, std::max<int64_t>(1, n / 1024)}));
  if (slices > 1) {
    const int64_t chunk = (n + slices - 1) / slices;
    const std::function<void(int)> task = [&](int i) {
      f(std::min(n, i * chunk), std::min(n, (i + 1) * chunk), i);
    };
    if (pool.run(slices, task)) return slices;
  }
  f(int64_t(0), n, 0);
  return 1;
}

// Runs task(i) for i in [0, tasks) on the worker pool, or in turn on the
// calling thread when the pool is busy.
void run_slices(int tasks, const std::function<void(int)> &task) {
  if (tasks > 1 && WorkerPool::get().run(tasks, task)) return;
  for (int i = 0; i < tasks; ++i) task(i);
}

// Stable LSD radix sort by key (ascending) in 11-bit digits over the low
// `bits` bits; a digit that is the same for every record costs only its
// count.  tmp is scratch (grown to the size of a when smaller).
void radix_sort(std::vector<SortRec> &a, std::vector<SortRec> &tmp, int bits) {
  const size_t n = a.size();
  if (tmp.size() < n) tmp.resize(n);
  SortRec *src = a.data(), *dst = tmp.data();
  uint32_t cnt[1u << 11];
  for (int shift = 0; shift < bits; shift += 11) {
    std::fill(cnt, cnt + (1u << 11), 0u);
    for (size_t q = 0; q < n; ++q) ++cnt[(src[q].key >> shift) & 2047u];
    if (std::find(cnt, cnt + (1u << 11), uint32_t(n)) != cnt + (1u << 11)) continue;
    uint32_t sum = 0;
    for (uint32_t &c : cnt) {
      const uint32_t v = c;
      c = sum;
      sum += v;
    }
    for (size_t q = 0; q < n; ++q) dst[cnt[(src[q].key >> shift) & 2047u]++] = src[q];
    std::swap(src, dst);
  }
  if (src != a.data()) std::copy(src, src + n, a.data());
}

int bit_width(uint64_t v) { return v == 0 ? 0 : 64 - __builtin_clzll(v); }

}  // namespace

void ShapeChooser::prepare() {
  const int64_t target_warps = int64_t(sms) * 24;
  g_occ = npairs > 0 ? pow2ceil((target_warps * 32 + npairs - 1) / npairs) : 32;
  inv_half_lane_steps = avg_lane_steps > 0 ? 1.0 / (0.5 * avg_lane_steps) : 0.0;
}

Shape ShapeChooser::pick(int m, int n, int rows_per_lane) const {
  // Lanes per pair G: (1) enough groups to fill every SM about 24 warps
  // deep; (2) enough lanes that this pair's sweep -- about m*n / (G*R)
  // dependent steps -- stays under half the balanced per-lane work of the
  // batch, so a long pair does not become the tail; (3) no more lanes than
  // its rows can use.
  const int rshift = rows_per_lane == 16 ? 4 : 3;
  int g_lat = 1;
  if (inv_half_lane_steps > 0) {
    const double steps_at_g1 = double(m) * double(n) * (1.0 / double(rows_per_lane));
    g_lat = pow2ceil(int64_t(steps_at_g1 * inv_half_lane_steps) + 1);
  }
  const int rows_cap = pow2ceil((m + rows_per_lane - 1) >> rshift);
  int G = std::max(g_occ, g_lat);
  if (force.shape) return force.sh;
  Shape sh{};
  TunedChoice tc;
  if (use_table && tune_table_pick(out_mode, m, n, &tc) && shape_supported(Shape{tc.sh.G, tc.sh.R, 0}, out_mode, local)) {
    sh = tc.sh;
    G = std::max(G, sh.G);
  } else {
    sh.R = kR;
    sh.i16 = 0;
  }
  sh.G = std::max(4, std::min(32, std::min(G, std::max(4, rows_cap))));
  return sh;
}

}  // namespace tsq

void tsq_batch::release_device_buffers() {
  for (tsq::DevBuf *d : {&seqs, &codes, &pairs, &tasks, &wtasks, &res, &bnd, &planes, &plane_off, &aln, &aln_off,
                         &shape_g, &shape_r, &counters, &lut, &matrix, &overflow, &rerun_tasks, &rerun_wtasks, &ccodes,
                         &clut, &cmatrix})
    d->release();
}

tsq_batch::~tsq_batch() {
  release_device_buffers();
  if (ev_fetch) cudaEventDestroy(ev_fetch);
  if (ev_fork) cudaEventDestroy(ev_fork);
  if (ev_join) cudaEventDestroy(ev_join);
  if (ev_encoded) cudaEventDestroy(ev_encoded);
  if (side) cudaStreamDestroy(side);
  if (gexec) cudaGraphExecDestroy(gexec);
  if (graph) cudaGraphDestroy(graph);
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
  if (stream) cudaStreamDestroy(stream);
}

namespace tsq {

namespace {
int plan_impl(tsq_batch *b, const tsq_batch *owner, const uint8_t *seqs, int64_t seqs_len,
              const tsq_pair_desc *pairs, int64_t n, const tsq_params *p, const tsq_batch_opts *opts, bool plain,
              int64_t call_pairs, int64_t call_cells, bool segmented);
int prepare_object(tsq_batch *b, const tsq_params *p, const tsq_batch_opts *opts, Scheme *sc, int *sms);
}  // namespace

// int16x2 fills exist for every output but local identity.
bool lanes16_possible(int out_mode, bool local, int lane) {
  return lane != TSQ_LANE_I32 && !(out_mode == kOutIdent && local);
}

int out_mode_of(const tsq_params *p) {
  return p->output == TSQ_OUT_ALIGNMENT ? kOutTrace : (p->output == TSQ_OUT_IDENTITY ? kOutIdent : kOutScore);
}

int check_params(const tsq_params *p) {
  if (p->gap_open < 0 || p->gap_extend < 0 || p->gap_open > 1000000 || p->gap_extend > 1000000)
    return TSQ_E_INVALID_ARG;
  if (p->mode != TSQ_GLOBAL && p->mode != TSQ_LOCAL) return TSQ_E_INVALID_ARG;
  if (p->output < TSQ_OUT_SCORE || p->output > TSQ_OUT_ALIGNMENT) return TSQ_E_INVALID_ARG;
  if (p->lane < TSQ_LANE_AUTO || p->lane > TSQ_LANE_I32) return TSQ_E_INVALID_ARG;
  return TSQ_OK;
}

// The value range the int32 kernels assume: every H, E, F stays above
// -(3*open + (m+n+1)*ext + 128), which must be far from their "minus
// infinity" (-2^29).  Identity counts travel in 16 bits, local maxima in 24
// bits of the reduction key.
int pair_limits(const tsq_params *p, const Scheme &sc, int out_mode, int32_t a_len, int32_t b_len) {
  if (a_len > kMaxLen || b_len > kMaxLen) return TSQ_E_TOO_LARGE;
  if (3 * int64_t(p->gap_open) + (int64_t(a_len) + b_len + 1) * p->gap_extend + 128 >= (int64_t(1) << 28))
    return TSQ_E_TOO_LARGE;
  if (out_mode == kOutIdent && int64_t(a_len) + b_len > 65535) return TSQ_E_TOO_LARGE;
  if (p->mode == TSQ_LOCAL && int64_t(std::max(sc.max_score, 0)) * std::min(a_len, b_len) >= (1 << 23))
    return TSQ_E_TOO_LARGE;
  return TSQ_OK;
}

// int16x2 range of a pair: the upper bound max_score * min(m, n) (no
// overflow check needed) and the lower bound -(3*open + (m + 512 + n +
// 1)*ext + open + ext + 128 + |min|), 512 being the most padding rows a pass
// can add, against the int16 kernels' minus infinity (-32000); the int16x2
// kernel also subtracts open + ext from values at this bound (T and XO),
// which must stay above -32768.
Range16 range16(const tsq_params *p, const Scheme &sc, int32_t a_len, int32_t b_len) {
  const int64_t go = p->gap_open, ge = p->gap_extend;
  const int64_t smax = std::max(sc.max_score, 0), sneg = std::max<int64_t>(0, -int64_t(sc.min_score));
  const int64_t lowest = 3 * go + (int64_t(a_len) + 512 + b_len + 1) * ge + go + ge + 128 + sneg;
  Range16 r;
  r.lower = lowest + go + ge < 31000 && ge <= 700 && b_len <= 65535;
  r.upper = smax * std::min(a_len, b_len) + smax < 32767;
  return r;
}

int collect_one(const ResultDev &d, const char *rows, int64_t cap, tsq_result &o) {
  o.score = d.score;
  o.a_begin = d.a_begin;
  o.a_end = d.a_end;
  o.b_begin = d.b_begin;
  o.b_end = d.b_end;
  o.n_ident = d.n_ident;
  o.n_cols = d.n_cols;
  o.status = d.status;
  o.aln_a = o.aln_b = nullptr;
  if (!rows) return TSQ_OK;
  const int64_t L = d.n_cols;
  if (L < 0 || L > cap) return TSQ_E_CUDA;
  o.aln_a = static_cast<char *>(std::malloc(size_t(L) + 1));
  o.aln_b = static_cast<char *>(std::malloc(size_t(L) + 1));
  if (!o.aln_a || !o.aln_b) {
    std::free(o.aln_a);
    std::free(o.aln_b);
    o.aln_a = o.aln_b = nullptr;
    return TSQ_E_NOMEM;
  }
  // The walker writes each row right-aligned in cap bytes.
  std::memcpy(o.aln_a, rows + cap - L, size_t(L));
  std::memcpy(o.aln_b, rows + 2 * cap - L, size_t(L));
  o.aln_a[L] = 0;
  o.aln_b[L] = 0;
  return TSQ_OK;
}

int batch_plan(tsq_batch *b, const uint8_t *seqs, int64_t seqs_len, const tsq_pair_desc *pairs, int64_t n,
               const tsq_params *p, const tsq_batch_opts *opts, bool plain) {
  TraceRange tr(plain ? "plan (one pair)" : "plan");
  return plan_impl(b, nullptr, seqs, seqs_len, pairs, n, p, opts, plain, 0, 0, false);
}

int batch_plan_chunk(tsq_batch *b, const tsq_batch *owner, const uint8_t *seqs, int64_t seqs_len,
                     const tsq_pair_desc *pairs, int64_t n, const tsq_params *p, const tsq_batch_opts *opts,
                     int64_t call_pairs, int64_t call_cells, bool segmented) {
  if (!b || owner == b || call_pairs < n || call_cells < 0) return TSQ_E_INVALID_ARG;
  TraceRange tr("plan chunk");
  if (!owner)
    return plan_impl(b, nullptr, seqs, seqs_len, pairs, n, p, opts, false, call_pairs, call_cells, segmented);
  const tsq_batch_opts o{owner->device, 0, opts ? opts->autotune : 0, opts ? opts->wait_polls : 0};
  return plan_impl(b, owner, nullptr, owner->seqs_len, pairs, n, p, &o, false, call_pairs, call_cells, segmented);
}

int input_segment(const tsq_batch *owner, const uint8_t *seqs, int64_t begin, int64_t end, cudaStream_t stream) {
  if (!owner || begin < 0 || end > owner->seqs_len || begin % 16 != 0 || (end > begin && !seqs))
    return TSQ_E_INVALID_ARG;
  if (end <= begin) return TSQ_OK;
  TSQ_TRY(cudaMemcpyAsync(owner->seqs.as<uint8_t>() + begin, seqs + begin, size_t(end - begin),
                          cudaMemcpyHostToDevice, stream));
  TSQ_TRY(launch_encode(owner->seqs.as<uint8_t>() + begin, end - begin, owner->lut.as<uint8_t>(),
                        owner->codes.as<uint8_t>() + begin, owner->classes ? owner->clut.as<uint8_t>() : nullptr,
                        owner->classes ? owner->ccodes.as<uint8_t>() + begin : nullptr, stream));
  return TSQ_OK;
}

int input_encode_mapped(const tsq_batch *owner, const uint8_t *src_dev, cudaStream_t stream) {
  if (!owner || !src_dev || reinterpret_cast<uintptr_t>(src_dev) % 16 != 0) return TSQ_E_INVALID_ARG;
  TSQ_TRY(launch_encode(src_dev, owner->seqs_len, owner->lut.as<uint8_t>(), owner->codes.as<uint8_t>(),
                        owner->classes ? owner->clut.as<uint8_t>() : nullptr,
                        owner->classes ? owner->ccodes.as<uint8_t>() : nullptr, stream));
  return TSQ_OK;
}

int input_prepare(tsq_batch *owner, int64_t seqs_len, const tsq_params *p, const tsq_batch_opts *opts) {
  if (!owner || !p || seqs_len < 0) return TSQ_E_INVALID_ARG;
  Scheme sc;
  int sms = 0;
  int rc = prepare_object(owner, p, opts, &sc, &sms);
  if (rc) return rc;
  cudaStream_t st = owner->stream;
  owner->classes = lanes16_possible(out_mode_of(p), p->mode == TSQ_LOCAL, p->lane);
  owner->seqs_len = seqs_len;
  TSQ_TRY(owner->seqs.ensure(size_t(seqs_len) + 128, st, owner->async_max));
  TSQ_TRY(owner->codes.ensure(size_t(seqs_len) + 128, st, owner->async_max));
  if (owner->classes) {
    TSQ_TRY(owner->ccodes.ensure(size_t(seqs_len) + 128, st, owner->async_max));
    // The fills' staging reads up to 64 bytes past a sequence: class 0 there.
    TSQ_TRY(cudaMemsetAsync(owner->ccodes.as<uint8_t>() + seqs_len, 0, 128, st));
  }
  TSQ_TRY(owner->lut.ensure(256, st, owner->async_max));
  uint8_t lut[256], clut[256];
  build_lut(sc, lut);
  TSQ_TRY(cudaMemcpyAsync(owner->lut.p, lut, 256, cudaMemcpyHostToDevice, st));
  if (owner->classes) {
    TSQ_TRY(owner->clut.ensure(256, st, owner->async_max));
    build_class_lut(sc, clut);
    TSQ_TRY(cudaMemcpyAsync(owner->clut.p, clut, 256, cudaMemcpyHostToDevice, st));
  }
  // The buffers and tables are then usable from the input stream.
  TSQ_TRY(cudaStreamSynchronize(st));
  owner->input_prepared = true;
  return TSQ_OK;
}

namespace {
// Checks the parameters, builds the scheme and readies the object for a new
// plan on its device: drops an old graph, (re)creates its streams and events.
int prepare_object(tsq_batch *b, const tsq_params *p, const tsq_batch_opts *opts, Scheme *sc, int *sms) {
  int rc = check_params(p);
  if (rc) return rc;
  rc = build_scheme(p, sc);
  if (rc) return rc;

  int dev = opts && opts->device >= 0 ? opts->device : -1;
  if (dev < 0) TSQ_TRY(cudaGetDevice(&dev));
  TSQ_TRY(cudaSetDevice(dev));
  TSQ_TRY(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev));

  // A replanned object drops its old graph.
  if (b->gexec) {
    cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  if (b->stream && b->device != dev) {
    b->release_device_buffers();
    cudaStreamDestroy(b->stream);
    b->stream = nullptr;
    if (b->side) cudaStreamDestroy(b->side);
    b->side = nullptr;
  }
  b->device = dev;
  if (!b->stream) TSQ_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  if (!b->side) TSQ_TRY(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
  if (!b->ev_fork) TSQ_TRY(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
  if (!b->ev_join) TSQ_TRY(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming));
  for (auto &e : b->ev)
    if (!e) TSQ_TRY(cudaEventCreate(&e));
  if (!b->ev_encoded) TSQ_TRY(cudaEventCreateWithFlags(&b->ev_encoded, cudaEventDisableTiming));
  return TSQ_OK;
}

int plan_impl(tsq_batch *b, const tsq_batch *owner, const uint8_t *seqs, int64_t seqs_len,
              const tsq_pair_desc *pairs, int64_t n, const tsq_params *p, const tsq_batch_opts *opts, bool plain,
              int64_t call_pairs, int64_t call_cells, bool segmented) {
  if (!b) return TSQ_E_INVALID_ARG;
  // The flag holds for this plan only, whatever it returns.
  const bool prepared = b->input_prepared;
  b->input_prepared = false;
  if (!p || n < 0 || seqs_len < 0) return TSQ_E_INVALID_ARG;
  b->input_owner = owner;
  b->input_segmented = segmented;
  if (n > 0 && !pairs) return TSQ_E_INVALID_ARG;
  if (seqs_len > 0 && !seqs && !owner) return TSQ_E_INVALID_ARG;
  if (n > INT32_MAX / 2) return TSQ_E_TOO_LARGE;
  Scheme sc;
  int sms = 0;
  int rc = prepare_object(b, p, opts, &sc, &sms);
  if (rc) return rc;

  b->scheme = sc;
  b->params = *p;
  b->out_mode = out_mode_of(p);
  b->local = p->mode == TSQ_LOCAL;
  b->use_graph = opts ? opts->use_graph != 0 : false;
  b->autotune = opts ? opts->autotune != 0 : false;
  b->wait_polls = opts && opts->wait_polls > 0 ? opts->wait_polls : 0;
  b->n = n;
  b->seqs_len = seqs_len;
  b->has_run = false;
  b->stats = tsq_batch_stats{};

  // Validate the pair table and the value range the int32 kernels assume:
  // every H, E, F stays above -(3*open + (m+n+1)*ext + 128), which must be
  // far from the kernels' "minus infinity" (-2^29).  Parallel over the
  // pairs; the error reported is that of the first bad pair.
  b->pairs_h.resize(size_t(n));
  struct ValPart {
    int64_t cells = 0, bad_at = INT64_MAX;
    int32_t max_n = 0;
    int rc = TSQ_OK;
  };
  std::vector<ValPart> vparts(8);
  parallel_for(n, [&](int64_t lo, int64_t hi, int slot) {
    ValPart v;
    for (int64_t k = lo; k < hi; ++k) {
      const tsq_pair_desc &d = pairs[k];
      int rc = TSQ_OK;
      if (d.a_len < 0 || d.b_len < 0 || d.a_off < 0 || d.b_off < 0)
        rc = TSQ_E_INVALID_ARG;
      else if (d.a_off > seqs_len - d.a_len || d.b_off > seqs_len - d.b_len)
        rc = TSQ_E_INVALID_ARG;
      else
        rc = pair_limits(p, sc, b->out_mode, d.a_len, d.b_len);
      if (rc != TSQ_OK) {
        v.bad_at = k;
        v.rc = rc;
        break;
      }
      b->pairs_h[size_t(k)] = PairDev{d.a_off, d.b_off, d.a_len, d.b_len};
      v.cells += int64_t(d.a_len) * d.b_len;
      v.max_n = std::max(v.max_n, d.b_len);
    }
    vparts[size_t(slot)] = v;
  });
  int64_t cells = 0;
  int32_t max_n = 0;
  {
    int64_t bad_at = INT64_MAX;
    int bad_rc = TSQ_OK;
    for (const ValPart &v : vparts) {
      cells += v.cells;
      max_n = std::max(max_n, v.max_n);
      if (v.bad_at < bad_at) {
        bad_at = v.bad_at;
        bad_rc = v.rc;
      }
    }
    if (bad_rc != TSQ_OK) return bad_rc;
  }
  b->cells = cells;

  // The residues go up first, so the copy overlaps the planning below.  Any
  // return from here on waits for it: the caller's buffer must outlive it.
  // (A chunk of a larger call uses its first chunk's residues instead.)
  struct SyncOnExit {
    cudaStream_t st;
    ~SyncOnExit() { cudaStreamSynchronize(st); }
  } sync_on_exit{b->stream};
  // Batches that may run int16x2 fills also get class codes.
  b->classes = lanes16_possible(b->out_mode, b->local, p->lane);
  if (!b->input_owner) {
    TSQ_TRY(b->seqs.ensure(size_t(seqs_len) + 128, b->stream, b->async_max));
    TSQ_TRY(b->codes.ensure(size_t(seqs_len) + 128, b->stream, b->async_max));
    if (b->classes) {
      TSQ_TRY(b->ccodes.ensure(size_t(seqs_len) + 128, b->stream, b->async_max));
      // The fills' staging reads up to 64 bytes past a sequence: class 0 there.
      TSQ_TRY(cudaMemsetAsync(b->ccodes.as<uint8_t>() + seqs_len, 0, 128, b->stream));
    }
    if (seqs_len > 0 && !segmented)
      TSQ_TRY(cudaMemcpyAsync(b->seqs.p, seqs, size_t(seqs_len), cudaMemcpyHostToDevice, b->stream));
  }

  // ---- lane types, shapes and order (one parallel pass over the pairs) ----
  // Fills run in int16x2 when the pair's values provably fit (range16: both
  // bounds).  Pairs with the lower bound but not the upper one run the
  // overflow-checked int16x2 kernel and are re-run in int32 if flagged;
  // everything else runs in int32.
  //
  // Long int32 pairs go to the CTA fill (their bands striped over the 16
  // or 8 warps of a CTA):
  // those whose sweep on one 32-lane group -- ceil(m/256) bands of n+31
  // steps -- would outlast the batch's balanced per-lane work (or, alone,
  // 20,000 steps).  Under the automatic lane type, score and traceback
  // pairs take the CTA fill in int16x2 lanes with rebased values
  // (fill_cta16.cuh) when open + ext + max_score <= 40: the long int32
  // pairs, and the int16x2 pairs whose sweep on one 32-lane group --
  // ceil(m/512) passes of n+63 steps -- exceeds the same budget.
  //
  // Order: lane type (CTA int16x2, CTA int32, checked int16x2, int16x2,
  // int32), then lane
  // width, then bands and columns descending, then input order -- one
  // 44-bit key, sorted by a stable LSD radix sort (O(n): the plan of an
  // 8M-pair batch must not cost seconds).
  ShapeChooser ch;
  ch.out_mode = b->out_mode;
  ch.local = b->local;
  ch.sms = sms;
  // Shapes follow the whole call's size (a chunk's pairs get the lane widths
  // a single plan would give them).
  const int64_t shape_pairs = call_pairs > 0 ? call_pairs : n;
  const int64_t shape_cells = call_pairs > 0 ? call_cells : cells;
  ch.npairs = plain ? 1 : shape_pairs;
  if (!plain) {
    const double lanes = double(sms) * 24.0 * 32.0;
    ch.avg_lane_steps = double(shape_cells) / (lanes * kR);
  }
  ch.use_table = b->autotune && tune_table_loaded();
  ch.force = b->tune_force;
  ch.prepare();
  PlanScratch &ps = b->scratch;
  ps.lsel.resize(size_t(n));
  ps.gsel.resize(size_t(n));
  ps.rsel.resize(size_t(n));
  ps.recs.resize(size_t(n));
  ps.cost.resize(size_t(n));
  std::vector<int8_t> &lsel = ps.lsel;
  std::vector<int32_t> &gsel = ps.gsel;
  std::vector<int32_t> &rsel = ps.rsel;
  std::vector<SortRec> &recs = ps.recs;
  auto two_bands = [&](int64_t k) { return lsel[size_t(k)] == 1 || lsel[size_t(k)] == 2; };
  auto bands = [&](int64_t k) {  // P = G * R (* 2): a power of two
    const int P = gsel[size_t(k)] * rsel[size_t(k)] * (two_bands(k) ? 2 : 1);
    return (b->pairs_h[size_t(k)].a_len + P - 1) >> __builtin_ctz(unsigned(P));
  };
  auto steps = [&](int64_t k) {
    return b->pairs_h[size_t(k)].b_len + gsel[size_t(k)] * (two_bands(k) ? 2 : 1) - 1;
  };
  struct ShapePart {
    int64_t n_checked = 0;
    uint64_t buckets[3] = {0, 0, 0};  // bit (G*4 + lane type) seen
    bool bad_shape = false;
    int32_t max_bands = 0, max_cols = 0;
  };
  std::vector<ShapePart> sparts(8);
  {
    const double lanes = double(sms) * 24.0 * 32.0;
    const double cta_budget = std::max(20000.0, plain ? 0.0 : double(shape_cells) / (lanes * kR));
    const bool try16 = lanes16_possible(b->out_mode, b->local, p->lane);
    // Long pairs take the CTA fill in int16x2 lanes (rebased values) where
    // the scheme allows it and the lane type is automatic.
    const bool cta16 = p->lane == TSQ_LANE_AUTO && cta16_supported(b->out_mode, b->local, sc, p->gap_open,
                                                                     p->gap_extend);
    parallel_for(n, [&](int64_t lo, int64_t hi, int slot) {
      ShapePart sp;
      for (int64_t k = lo; k < hi; ++k) {
        const PairDev &pd = b->pairs_h[size_t(k)];
        int8_t lt = 0;
        // A tuned table may prefer int32 over int16x2 for this length bucket,
        // or the CTA fill for its int32 pairs.
        TunedChoice tc;
        const bool tuned = ch.use_table && !ch.force.shape && tune_table_pick(b->out_mode, pd.a_len, pd.b_len, &tc);
        if (try16 && !(tuned && tc.sh.i16 == 0)) {
          const Range16 r16 = range16(p, sc, pd.a_len, pd.b_len);
          if (r16.lower) lt = (r16.upper && p->lane == TSQ_LANE_AUTO) ? 1 : 2;
        }
        if (lt == 0 && pd.a_len > 0 && pd.b_len > 0) {
          const double steps32 = double((pd.a_len + 255) / 256) * double(pd.b_len + 31);
          if (steps32 > cta_budget || ch.force.cta || (tuned && tc.cta)) lt = cta16 ? 4 : 3;
        } else if (lt != 0 && cta16 && !ch.force.shape) {
          // An int16x2 pair whose sweep on one 32-lane group -- ceil(m/512)
          // passes of n+63 steps -- would be the batch's tail (and, when
          // checked, might need an int32 re-run on one warp as well).
          const double steps16 = double((pd.a_len + 511) / 512) * double(pd.b_len + 63);
          if (steps16 > cta_budget) lt = 4;
        }
        lsel[size_t(k)] = lt;
        sp.n_checked += lt == 2;
        const int rows_per_lane = (lt == 1 || lt == 2) ? 2 * kR : kR;
        Shape shp = ch.pick(pd.a_len, pd.b_len, rows_per_lane);
        if (lt >= 3) shp = Shape{32, kR, 0};  // one 32-lane group per warp of the CTA
        shp.i16 = 0;
        if (!shape_supported(shp, b->out_mode, b->local)) sp.bad_shape = true;
        gsel[size_t(k)] = shp.G;
        rsel[size_t(k)] = shp.R;
        const int bit = shp.G * 4 + lt;
        sp.buckets[bit >> 6] |= uint64_t(1) << (bit & 63);
        const int gi = shp.G == 4 ? 0 : shp.G == 8 ? 1 : shp.G == 16 ? 2 : 3;
        const int32_t bandk = std::min(bands(k), (1 << 19) - 1);
        const int32_t colk = std::min(pd.b_len, (1 << 20) - 1);
        ps.cost[size_t(k)] = int64_t(bands(k)) * steps(k);
        sp.max_bands = std::max(sp.max_bands, bandk);
        sp.max_cols = std::max(sp.max_cols, colk);
        // Ranks of the lane types 0..4, in launch order: CTA int16x2, CTA
        // int32, checked int16x2, int16x2, int32.
        static const uint64_t kLaneRank[5] = {4, 3, 2, 1, 0};
        // Provisional key; packed to the bits the batch needs below.
        recs[size_t(k)] = SortRec{(kLaneRank[lt] << 42) | (uint64_t(gi) << 40) | (uint64_t(bandk) << 20) |
                                      uint64_t(colk),
                                  int32_t(k)};
      }
      sparts[size_t(slot)] = sp;
    });
  }
  int64_t n_checked = 0;
  uint64_t bucket_bits[3] = {0, 0, 0};
  int32_t max_bands = 0, max_cols = 0;
  for (const ShapePart &sp : sparts) {
    if (sp.bad_shape) return TSQ_E_INVALID_ARG;
    n_checked += sp.n_checked;
    for (int w = 0; w < 3; ++w) bucket_bits[w] |= sp.buckets[w];
    max_bands = std::max(max_bands, sp.max_bands);
    max_cols = std::max(max_cols, sp.max_cols);
  }
  {
    // Pack (lane rank, lane width, bands descending, columns descending)
    // into as few bits as this batch needs: fewer radix passes.
    const int wb = bit_width(uint64_t(max_bands)), wc = bit_width(uint64_t(max_cols));
    for (SortRec &r : recs) {
      const uint64_t top = r.key >> 40, bandk = (r.key >> 20) & ((1u << 20) - 1), colk = r.key & ((1u << 20) - 1);
      r.key = (top << (wb + wc)) | ((uint64_t(max_bands) - bandk) << wc) | (uint64_t(max_cols) - colk);
    }
    radix_sort(recs, ps.tmp, 5 + wb + wc);  // 3 bits of lane rank, 2 of lane width
  }
  ps.order.resize(size_t(n));
  ps.s_lt.resize(size_t(n));
  ps.s_g.resize(size_t(n));
  ps.s_cols.resize(size_t(n));
  ps.s_cost.resize(size_t(n));
  std::vector<int32_t> &order = ps.order;
  parallel_for(n, [&](int64_t lo, int64_t hi, int) {
    for (int64_t q = lo; q < hi; ++q) {
      const int32_t k = recs[size_t(q)].idx;
      order[size_t(q)] = k;
      ps.s_lt[size_t(q)] = lsel[size_t(k)];
      ps.s_g[size_t(q)] = gsel[size_t(k)];
      ps.s_cols[size_t(q)] = b->pairs_h[size_t(k)].b_len;
      ps.s_cost[size_t(q)] = ps.cost[size_t(k)];
    }
  });

  // One launch per lane type (int16x2 checked, int16x2, int32), each a list
  // of warp tasks -- consecutive pairs of one lane width, 32/G per warp --
  // ordered by cost (bands x steps of the longest pair), longest first.
  b->launches.clear();
  std::vector<int2> wt_all;
  int64_t bnd_total = 0;
  int32_t checked_begin = 0;
  for (int64_t s = 0; s < n;) {
    const int8_t lt = ps.s_lt[size_t(s)];
    int64_t e = s;
    int32_t cols = 1;
    while (e < n && ps.s_lt[size_t(e)] == lt) {
      cols = std::max(cols, ps.s_cols[size_t(e)]);
      ++e;
    }
    if (lt == 2) checked_begin = int32_t(s);
    if (lt >= 3) {
      // One long pair per CTA; the CTAs pull pairs longest first.
      Launch L;
      L.R = kR;
      L.i16 = lt == 4 ? 1 : 0;  // int16x2 lanes with rebased values
      L.cta = true;
      L.task_begin = int32_t(s);
      L.n_wtasks = int32_t(e - s);
      const int max_blocks = lt == 4 ? cta16_blocks(b->out_mode, b->local, sc.nclasses) : cta_blocks(b->out_mode, b->local);
      if (max_blocks <= 0) return TSQ_E_CUDA;
      L.blocks = int32_t(std::max<int64_t>(1, std::min<int64_t>(max_blocks, e - s)));
      L.bnd_cols = ((cols + 31) / 32 + 1) * 32;
      L.bnd_offset = bnd_total;
      bnd_total += int64_t(L.blocks) * L.bnd_cols * int64_t(cta_bnd_entry_bytes(b->out_mode));
      bnd_total = (bnd_total + 255) & ~int64_t(255);
      b->launches.push_back(L);
      s = e;
      continue;
    }
    std::vector<int2> wt;
    std::vector<int64_t> wcost;
    wt.reserve(size_t(e - s));
    wcost.reserve(size_t(e - s));
    for (int64_t q = s; q < e;) {
      const int G = ps.s_g[size_t(q)];
      const int per = 32 / G;
      int64_t r = q;
      int64_t cost = 0;
      while (r < e && r - q < per && ps.s_g[size_t(r)] == G) {
        cost = std::max<int64_t>(cost, ps.s_cost[size_t(r)]);
        ++r;
      }
      wt.push_back(make_int2(int32_t(q), (G << 16) | int32_t(r - q)));
      wcost.push_back(cost);
      q = r;
    }
    // Longest first: ascending order of (max cost - cost), stable.
    int64_t max_cost = 0;
    for (int64_t c : wcost) max_cost = std::max(max_cost, c);
    std::vector<SortRec> wrec(wt.size());
    for (size_t w = 0; w < wt.size(); ++w) wrec[w] = SortRec{uint64_t(max_cost - wcost[w]), int32_t(w)};
    radix_sort(wrec, ps.tmp, bit_width(uint64_t(max_cost)));
    std::vector<int32_t> worder(wt.size());
    for (size_t w = 0; w < wt.size(); ++w) worder[w] = wrec[w].idx;
    Launch L;
    L.R = kR;
    L.i16 = lt;
    L.wt_begin = int32_t(wt_all.size());
    L.n_wtasks = int32_t(wt.size());
    for (int32_t w : worder) wt_all.push_back(wt[size_t(w)]);
    const int max_blocks = fill_blocks(L.R, L.i16, b->out_mode, b->local, sc.nclasses);
    if (max_blocks <= 0) return TSQ_E_CUDA;
    const int warps_per_block = fill_threads_for(L.i16) / 32;
    const int64_t needed = (int64_t(L.n_wtasks) + warps_per_block - 1) / warps_per_block;
    L.blocks = int32_t(std::max<int64_t>(1, std::min<int64_t>(max_blocks, needed)));
    // Whole staged chunks are copied, so rows are padded to a chunk past n.
    L.bnd_cols = ((cols + 31) / 32 + 1) * 32;
    L.bnd_offset = bnd_total;
    bnd_total += int64_t(L.blocks) * warps_per_block * 8 * L.bnd_cols *
                 int64_t(fill_bnd_entry_bytes(L.i16, b->out_mode));
    bnd_total = (bnd_total + 255) & ~int64_t(255);
    b->launches.push_back(L);
    s = e;
  }
  // The int32 re-run of pairs the checked int16x2 launch flags: its warp
  // tasks are built on the device, its size bounded by the checked pairs.
  b->n_checked = n_checked;
  b->checked_begin = checked_begin;
  if (n_checked > 0) {
    int32_t cols = 1;
    for (int64_t q = checked_begin; q < checked_begin + n_checked; ++q)
      cols = std::max(cols, b->pairs_h[size_t(order[size_t(q)])].b_len);
    Launch L;
    L.R = kR;
    L.i16 = 0;
    L.rerun = true;
    const int max_blocks = fill_blocks(L.R, 0, b->out_mode, b->local);
    if (max_blocks <= 0) return TSQ_E_CUDA;
    const int warps_per_block = fill_threads_for(0) / 32;
    L.blocks = int32_t(std::max<int64_t>(1, std::min<int64_t>(max_blocks, (n_checked + warps_per_block - 1) /
                                                                             warps_per_block)));
    L.bnd_cols = ((cols + 31) / 32 + 1) * 32;
    L.bnd_offset = bnd_total;
    bnd_total += int64_t(L.blocks) * warps_per_block * 8 * L.bnd_cols * int64_t(fill_bnd_entry_bytes(0, b->out_mode));
    b->launches.push_back(L);
  }
  b->stats.pairs = n;
  b->stats.cells = cells;
  b->stats.launches = int32_t(b->launches.size()) + 1 + (b->out_mode == kOutTrace ? 1 : 0) + (n_checked > 0 ? 1 : 0);
  b->stats.buckets = __builtin_popcountll(bucket_bits[0]) + __builtin_popcountll(bucket_bits[1]) +
                      __builtin_popcountll(bucket_bits[2]);
  const std::vector<int2> &wt_sorted = wt_all;

  // ---- traceback layout ----------------------------------------------------
  std::vector<int64_t> ploff;
  b->aln_off_h.clear();
  b->aln_bytes = 0;
  int64_t plane_total = 0;
  if (b->out_mode == kOutTrace) {
    ploff.resize(size_t(n));
    b->aln_off_h.resize(size_t(n));
    for (int64_t k = 0; k < n; ++k) {
      const PairDev &pd = b->pairs_h[size_t(k)];
      ploff[size_t(k)] = plane_total;
      plane_total += plane_bytes(pd.a_len, pd.b_len, Shape{gsel[size_t(k)], rsel[size_t(k)], 0});
      b->aln_off_h[size_t(k)] = b->aln_bytes;
      b->aln_bytes += 2 * (int64_t(pd.a_len) + pd.b_len);
    }
  }

  // ---- device buffers and uploads -------------------------------------------
  uint8_t lut[256];
  build_lut(sc, lut);
  // (seqs and codes were sized above: staged code chunks read up to 64
  // bytes past a sequence, hence the padding.)
  TSQ_TRY(b->pairs.ensure(sizeof(PairDev) * size_t(n), b->stream, b->async_max));
  TSQ_TRY(b->tasks.ensure(sizeof(int32_t) * size_t(n), b->stream, b->async_max));
  TSQ_TRY(b->res.ensure(sizeof(ResultDev) * size_t(n), b->stream, b->async_max));
  TSQ_TRY(b->bnd.ensure(size_t(bnd_total), b->stream, b->async_max));
  TSQ_TRY(b->wtasks.ensure(sizeof(int2) * std::max<size_t>(1, wt_sorted.size()), b->stream, b->async_max));
  TSQ_TRY(b->counters.ensure(sizeof(int32_t) * (b->launches.size() + 2), b->stream, b->async_max));
  TSQ_TRY(b->shape_g.ensure(sizeof(int32_t) * size_t(n), b->stream, b->async_max));
  TSQ_TRY(b->shape_r.ensure(sizeof(int32_t) * size_t(n), b->stream, b->async_max));
  if (n_checked > 0) {
    TSQ_TRY(b->overflow.ensure(sizeof(int32_t) * size_t(n), b->stream, b->async_max));
    TSQ_TRY(b->rerun_tasks.ensure(sizeof(int32_t) * size_t(n_checked), b->stream, b->async_max));
    TSQ_TRY(b->rerun_wtasks.ensure(sizeof(int2) * size_t(n_checked), b->stream, b->async_max));
  }
  TSQ_TRY(b->rerun_h.ensure(sizeof(int32_t)));
  TSQ_TRY(b->lut.ensure(256, b->stream, b->async_max));
  TSQ_TRY(b->matrix.ensure(kLetters * kLetters, b->stream, b->async_max));
  if (b->classes) {
    TSQ_TRY(b->clut.ensure(256, b->stream, b->async_max));
    TSQ_TRY(b->cmatrix.ensure(kLetters * kLetters, b->stream, b->async_max));
  }
  TSQ_TRY(b->res_h.ensure(sizeof(ResultDev) * size_t(n)));
  if (b->out_mode == kOutTrace) {
    TSQ_TRY(b->planes.ensure(size_t(plane_total), b->stream, b->async_max));
    TSQ_TRY(b->plane_off.ensure(sizeof(int64_t) * size_t(n), b->stream, b->async_max));
    TSQ_TRY(b->aln.ensure(size_t(b->aln_bytes), b->stream, b->async_max));
    TSQ_TRY(b->aln_off.ensure(sizeof(int64_t) * size_t(n), b->stream, b->async_max));
    TSQ_TRY(b->aln_h.ensure(size_t(b->aln_bytes)));
  }
  cudaStream_t st = b->stream;
  if (n > 0) {
    TSQ_TRY(cudaMemcpyAsync(b->pairs.p, b->pairs_h.data(), sizeof(PairDev) * size_t(n), cudaMemcpyHostToDevice, st));
    TSQ_TRY(cudaMemcpyAsync(b->tasks.p, order.data(), sizeof(int32_t) * size_t(n), cudaMemcpyHostToDevice, st));
    TSQ_TRY(cudaMemcpyAsync(b->wtasks.p, wt_sorted.data(), sizeof(int2) * wt_sorted.size(), cudaMemcpyHostToDevice,
                            st));
  }
  // (An input set up by input_prepare has its code tables on the device
  // already, read by encode kernels that may be running now.)
  if (!prepared) TSQ_TRY(cudaMemcpyAsync(b->lut.p, lut, 256, cudaMemcpyHostToDevice, st));
  TSQ_TRY(cudaMemcpyAsync(b->matrix.p, sc.score, kLetters * kLetters, cudaMemcpyHostToDevice, st));
  uint8_t clut[256];
  if (b->classes) {
    build_class_lut(sc, clut);
    if (!prepared) TSQ_TRY(cudaMemcpyAsync(b->clut.p, clut, 256, cudaMemcpyHostToDevice, st));
    TSQ_TRY(cudaMemcpyAsync(b->cmatrix.p, sc.cscore, size_t(sc.nclasses) * sc.nclasses, cudaMemcpyHostToDevice,
                            st));
  }
  if (b->out_mode == kOutTrace && n > 0) {
    TSQ_TRY(cudaMemcpyAsync(b->plane_off.p, ploff.data(), sizeof(int64_t) * size_t(n), cudaMemcpyHostToDevice, st));
    TSQ_TRY(cudaMemcpyAsync(b->aln_off.p, b->aln_off_h.data(), sizeof(int64_t) * size_t(n), cudaMemcpyHostToDevice,
                            st));
  }
  if (n > 0) {
    TSQ_TRY(cudaMemcpyAsync(b->shape_g.p, gsel.data(), sizeof(int32_t) * size_t(n), cudaMemcpyHostToDevice, st));
    TSQ_TRY(cudaMemcpyAsync(b->shape_r.p, rsel.data(), sizeof(int32_t) * size_t(n), cudaMemcpyHostToDevice, st));
  }
  // The host vectors above go out of scope: wait for the copies.
  TSQ_TRY(cudaStreamSynchronize(st));
  return TSQ_OK;
}
}  // namespace

namespace {

const uint8_t *seqs_dev(const tsq_batch *b) {
  return b->input_owner ? b->input_owner->seqs.as<uint8_t>() : b->seqs.as<uint8_t>();
}
const uint8_t *codes_dev(const tsq_batch *b) {
  return b->input_owner ? b->input_owner->codes.as<uint8_t>() : b->codes.as<uint8_t>();
}
const uint8_t *ccodes_dev(const tsq_batch *b) {
  return b->input_owner ? b->input_owner->ccodes.as<uint8_t>() : b->ccodes.as<uint8_t>();
}

// Inside stream capture an event record becomes an external event-record
// node, so the event can still be timed after each graph launch.
cudaError_t record(tsq_batch *b, int k) {
  return b->capturing ? cudaEventRecordWithFlags(b->ev[k], b->stream, cudaEventRecordExternal)
                      : cudaEventRecord(b->ev[k], b->stream);
}

// Fill launch names for the trace ranges: [i16][out_mode].
const char *fill_range_name(const Launch &L, int out_mode) {
  if (L.cta && L.i16) return out_mode == kOutTrace ? "fill_cta16 trace" : "fill_cta16 score";
  if (L.cta) return out_mode == kOutTrace ? "fill_cta trace" : (out_mode == kOutIdent ? "fill_cta identity" : "fill_cta score");
  if (L.rerun) return "fill_i32 re-run of int16 overflows";
  if (L.i16 == 1) return "fill_i16 score";
  if (L.i16 == 2) return "fill_i16 score (checked)";
  return out_mode == kOutTrace ? "fill_i32 trace" : (out_mode == kOutIdent ? "fill_i32 identity" : "fill_i32 score");
}

int enqueue_run(tsq_batch *b) {
  TraceRange tr("enqueue run");
  cudaStream_t st = b->stream;
  const int nl = int(b->launches.size());
  TSQ_TRY(cudaMemsetAsync(b->counters.p, 0, sizeof(int32_t) * (size_t(nl) + 2), st));
  TSQ_TRY(record(b, 0));
  if (b->input_segmented) {
    // The residues this chunk reads were uploaded and encoded on the call's
    // input stream.
    TSQ_TRY(cudaStreamWaitEvent(st, b->input_ready, 0));
  } else if (b->input_owner) {
    // The owner encodes the residues on its stream.
    TSQ_TRY(cudaStreamWaitEvent(st, b->input_owner->ev_encoded, 0));
  } else {
    TraceRange er("encode");
    TSQ_TRY(launch_encode(b->seqs.as<uint8_t>(), b->seqs_len, b->lut.as<uint8_t>(), b->codes.as<uint8_t>(),
                          b->classes ? b->clut.as<uint8_t>() : nullptr, b->classes ? b->ccodes.as<uint8_t>() : nullptr,
                          st));
    if (!b->capturing) TSQ_TRY(cudaEventRecord(b->ev_encoded, st));
  }
  TSQ_TRY(record(b, 1));
  int32_t *rerun_count = b->counters.as<int32_t>() + nl + 1;
  // The CTA launch (long pairs) runs on a side stream next to the others.
  bool forked = false;
  for (const Launch &L : b->launches) forked |= L.cta;
  if (forked) {
    TSQ_TRY(cudaEventRecord(b->ev_fork, st));
    TSQ_TRY(cudaStreamWaitEvent(b->side, b->ev_fork, 0));
  }
  for (int l = 0; l < nl; ++l) {
    const Launch &L = b->launches[size_t(l)];
    TraceRange lr(fill_range_name(L, b->out_mode));
    if (L.cta) {
      FillArgs a{};
      a.codes = codes_dev(b);
      a.pairs = b->pairs.as<PairDev>();
      a.tasks = b->tasks.as<int32_t>() + L.task_begin;
      a.n_wtasks = L.n_wtasks;
      a.counter = b->counters.as<int32_t>() + l;
      a.matrix = b->matrix.as<int8_t>();
      a.gap_open = b->params.gap_open;
      a.gap_extend = b->params.gap_extend;
      a.res = b->res.as<ResultDev>();
      a.bnd = reinterpret_cast<int32_t *>(b->bnd.as<uint8_t>() + L.bnd_offset);
      a.bnd_cols = L.bnd_cols;
      a.planes = b->planes.as<uint8_t>();
      a.plane_off = b->plane_off.as<int64_t>();
      a.max_score = b->scheme.max_score;
      a.spin_limit = b->wait_polls;
      if (L.i16) {
        a.ccodes = ccodes_dev(b);
        a.cmatrix = b->cmatrix.as<int8_t>();
        a.nclasses = b->scheme.nclasses;
        TSQ_TRY(launch_cta16(b->out_mode, b->local, a, L.blocks, b->side));
      } else {
        TSQ_TRY(launch_cta(b->out_mode, b->local, a, L.blocks, b->side));
      }
      continue;
    }
    if (L.rerun) {
      // Pairs the checked int16x2 launch flagged, compacted on the device.
      TSQ_TRY(launch_collect_overflow(b->tasks.as<int32_t>() + b->checked_begin, int32_t(b->n_checked),
                                      b->overflow.as<int32_t>(), b->shape_g.as<int32_t>(),
                                      b->rerun_tasks.as<int32_t>(), b->rerun_wtasks.as<int2>(), rerun_count, st));
    }
    FillArgs a{};
    a.codes = codes_dev(b);
    a.pairs = b->pairs.as<PairDev>();
    a.tasks = L.rerun ? b->rerun_tasks.as<int32_t>() : b->tasks.as<int32_t>();
    a.wtasks = L.rerun ? b->rerun_wtasks.as<int2>() : b->wtasks.as<int2>() + L.wt_begin;
    a.n_wtasks = L.n_wtasks;
    a.n_wtasks_dev = L.rerun ? rerun_count : nullptr;
    a.counter = b->counters.as<int32_t>() + l;
    a.matrix = b->matrix.as<int8_t>();
    a.gap_open = b->params.gap_open;
    a.gap_extend = b->params.gap_extend;
    a.res = b->res.as<ResultDev>();
    a.bnd = reinterpret_cast<int32_t *>(b->bnd.as<uint8_t>() + L.bnd_offset);
    a.bnd_cols = L.bnd_cols;
    a.planes = b->planes.as<uint8_t>();
    a.plane_off = b->plane_off.as<int64_t>();
    a.overflow = b->overflow.as<int32_t>();
    a.max_score = b->scheme.max_score;
    if (L.i16) {
      a.ccodes = ccodes_dev(b);
      a.cmatrix = b->cmatrix.as<int8_t>();
      a.nclasses = b->scheme.nclasses;
    }
    TSQ_TRY(launch_fill(L.R, L.i16, b->out_mode, b->local, a, L.blocks, st));
  }
  if (forked) {
    TSQ_TRY(cudaEventRecord(b->ev_join, b->side));
    TSQ_TRY(cudaStreamWaitEvent(st, b->ev_join, 0));
  }
  if (b->n_checked > 0)
    TSQ_TRY(cudaMemcpyAsync(b->rerun_h.p, rerun_count, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  TSQ_TRY(record(b, 2));
  if (b->out_mode == kOutTrace) {
    WalkArgs w{};
    w.seqs = seqs_dev(b);
    w.codes = codes_dev(b);
    w.pairs = b->pairs.as<PairDev>();
    w.tasks = b->tasks.as<int32_t>();
    w.n_tasks = int32_t(b->n);
    w.planes = b->planes.as<uint8_t>();
    w.plane_off = b->plane_off.as<int64_t>();
    w.shape_G = b->shape_g.as<int32_t>();
    w.shape_R = b->shape_r.as<int32_t>();
    w.local = b->local ? 1 : 0;
    w.res = b->res.as<ResultDev>();
    w.aln = b->aln.as<char>();
    w.aln_off = b->aln_off.as<int64_t>();
    TraceRange wr("walk");
    TSQ_TRY(launch_walk(w, st));
  }
  TSQ_TRY(record(b, 3));
  return TSQ_OK;
}

}  // namespace

int batch_run_async(tsq_batch *b) {
  if (!b) return TSQ_E_INVALID_ARG;
  TraceRange tr(b->use_graph ? "batch run (graph)" : "batch run");
  TSQ_TRY(cudaSetDevice(b->device));
  if (!b->use_graph) {
    const int rc = enqueue_run(b);
    if (rc) return rc;
  } else {
    if (!b->gexec) {
      TSQ_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      b->capturing = true;
      const int rc = enqueue_run(b);
      b->capturing = false;
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      TSQ_TRY(e);
      b->graph = g;
      TSQ_TRY(cudaGraphInstantiate(&b->gexec, b->graph, 0));
    }
    TSQ_TRY(cudaEventRecord(b->ev[4], b->stream));
    TSQ_TRY(cudaGraphLaunch(b->gexec, b->stream));
    TSQ_TRY(cudaEventRecord(b->ev[5], b->stream));
  }
  b->has_run = true;
  return TSQ_OK;
}

int batch_sync(tsq_batch *b) {
  if (!b) return TSQ_E_INVALID_ARG;
  TraceRange tr("batch sync");
  TSQ_TRY(cudaStreamSynchronize(b->stream));
  if (!b->has_run) return TSQ_OK;
  b->stats.rerun_pairs = b->n_checked > 0 ? *b->rerun_h.as<int32_t>() : 0;
  float total = 0.f, fill = 0.f;
  if (cudaEventElapsedTime(&total, b->ev[0], b->ev[3]) == cudaSuccess) {
    b->stats.device_ms = total;
  } else if (b->use_graph && cudaEventElapsedTime(&total, b->ev[4], b->ev[5]) == cudaSuccess) {
    b->stats.device_ms = total;
  }
  if (cudaEventElapsedTime(&fill, b->ev[1], b->ev[2]) == cudaSuccess) {
    b->stats.fill_ms = fill;
  } else {
    b->stats.fill_ms = b->stats.device_ms;  // whole graph when nodes cannot be timed
  }
  cudaGetLastError();  // a failed elapsed-time query is not a sticky error
  return TSQ_OK;
}

int batch_fetch_async(tsq_batch *b) {
  if (!b || !b->has_run) return TSQ_E_INVALID_ARG;
  cudaStream_t st = b->stream;
  if (b->n > 0)
    TSQ_TRY(cudaMemcpyAsync(b->res_h.p, b->res.p, sizeof(ResultDev) * size_t(b->n), cudaMemcpyDeviceToHost, st));
  if (b->out_mode == kOutTrace && b->aln_bytes > 0)
    TSQ_TRY(cudaMemcpyAsync(b->aln_h.p, b->aln.p, size_t(b->aln_bytes), cudaMemcpyDeviceToHost, st));
  if (!b->ev_fetch) TSQ_TRY(cudaEventCreateWithFlags(&b->ev_fetch, cudaEventDisableTiming));
  TSQ_TRY(cudaEventRecord(b->ev_fetch, st));
  return TSQ_OK;
}

int batch_fetch_query(tsq_batch *b) {
  const cudaError_t e = cudaEventQuery(b->ev_fetch);
  if (e == cudaSuccess) return TSQ_OK;
  if (e == cudaErrorNotReady) return TSQ_E_PENDING;
  return cuda_status(e);
}

int64_t cost_order(const tsq_pair_desc *pairs, int64_t n, std::vector<uint8_t> &bin, tsq_pair_desc *out_pairs,
                   int32_t *out_index) {
  if (n <= 0) return 0;
  bin.resize(size_t(n));
  // Fixed slices, the same in both passes.
  const int slices = int(std::min<int64_t>({8, int64_t(WorkerPool::get().workers()) + 1, (n + 8191) / 8192}));
  const int64_t step = (n + slices - 1) / slices;
  std::vector<std::array<int64_t, 256>> hist(static_cast<size_t>(slices));
  std::vector<int64_t> cells(static_cast<size_t>(slices), 0);
  run_slices(slices, [&](int s) {
    std::array<int64_t, 256> &h = hist[size_t(s)];
    h.fill(0);
    int64_t c = 0;
    for (int64_t k = int64_t(s) * step, e = std::min(n, k + step); k < e; ++k) {
      const int64_t ck = int64_t(std::max(pairs[k].a_len, 0)) * std::max(pairs[k].b_len, 0);
      c += ck;
      const int bw = ck > 0 ? 64 - __builtin_clzll(uint64_t(ck)) : 0;
      const int b = 4 * bw + (bw >= 3 ? int((uint64_t(ck) >> (bw - 3)) & 3) : 0);
      bin[size_t(k)] = uint8_t(b);
      ++h[size_t(b)];
    }
    cells[size_t(s)] = c;
  });
  // Position of each (bin, slice) run: bins descending, slices in order.
  int64_t acc = 0;
  for (int b = 255; b >= 0; --b)
    for (int s = 0; s < slices; ++s) {
      const int64_t c = hist[size_t(s)][size_t(b)];
      hist[size_t(s)][size_t(b)] = acc;
      acc += c;
    }
  run_slices(slices, [&](int s) {
    std::array<int64_t, 256> &next = hist[size_t(s)];
    for (int64_t k = int64_t(s) * step, e = std::min(n, k + step); k < e; ++k) {
      const int64_t r = next[bin[size_t(k)]]++;
      out_pairs[r] = pairs[k];
      out_index[r] = int32_t(k);
    }
  });
  int64_t total = 0;
  for (int64_t c : cells) total += c;
  return total;
}

int batch_collect(tsq_batch *b, int64_t begin, int64_t count, tsq_result *out, const int32_t *dst) {
  if (!b || begin < 0 || count < 0 || begin + count > b->n || (count > 0 && !out)) return TSQ_E_INVALID_ARG;
  const ResultDev *r = b->res_h.as<ResultDev>();
  if (b->out_mode != kOutTrace && count >= 16384) {
    // Parallel over the pairs (a scattered collect is bound by its writes).
    // The status is what the serial loop below returns: the last pair's
    // error other than a residue error, else a residue error, else OK.
    struct Part {
      int last = TSQ_OK;
      bool residue = false;
    };
    Part parts[8];
    parallel_for(count, [&](int64_t lo, int64_t hi, int slot) {
      Part pt;
      for (int64_t q = lo; q < hi; ++q) {
        const ResultDev &d = r[begin + q];
        tsq_result &o = dst ? out[dst[q]] : out[q];
        o.score = d.score;
        o.a_begin = d.a_begin;
        o.a_end = d.a_end;
        o.b_begin = d.b_begin;
        o.b_end = d.b_end;
        o.n_ident = d.n_ident;
        o.n_cols = d.n_cols;
        o.status = d.status;
        o.aln_a = o.aln_b = nullptr;
        if (d.status == TSQ_E_INVALID_RESIDUE)
          pt.residue = true;
        else if (d.status != TSQ_OK)
          pt.last = d.status;
      }
      parts[slot] = pt;
    });
    int rc = TSQ_OK;
    for (const Part &pt : parts) {
      if (pt.residue && rc == TSQ_OK) rc = TSQ_E_INVALID_RESIDUE;
      if (pt.last != TSQ_OK) rc = pt.last;
    }
    return rc;
  }
  if (b->out_mode == kOutTrace && count >= 512) {
    // Each pair's rows take two allocations and two copies: parallel over
    // the pairs.  The status is the first failure to take rows (TSQ_E_CUDA,
    // TSQ_E_NOMEM) if any, else what the serial loop below returns.
    const int slices = int(std::min<int64_t>({8, int64_t(WorkerPool::get().workers()) + 1, count / 256}));
    const int64_t step = (count + slices - 1) / slices;
    struct Part {
      int fail = TSQ_OK;
      int last = TSQ_OK;
      bool residue = false;
    };
    std::vector<Part> parts(static_cast<size_t>(slices));
    run_slices(slices, [&](int sl) {
      Part pt;
      for (int64_t q = int64_t(sl) * step, e = std::min(count, q + step); q < e; ++q) {
        const int64_t k = begin + q;
        tsq_result &o = dst ? out[dst[q]] : out[q];
        const ResultDev &d = r[k];
        const PairDev &pd = b->pairs_h[size_t(k)];
        const int e2 = collect_one(d, d.status == TSQ_OK ? b->aln_h.as<char>() + b->aln_off_h[size_t(k)] : nullptr,
                                   int64_t(pd.a_len) + pd.b_len, o);
        if (e2 != TSQ_OK && pt.fail == TSQ_OK) pt.fail = e2;
        if (d.status == TSQ_E_INVALID_RESIDUE)
          pt.residue = true;
        else if (d.status != TSQ_OK)
          pt.last = d.status;
      }
      parts[size_t(sl)] = pt;
    });
    for (const Part &pt : parts)
      if (pt.fail != TSQ_OK) return pt.fail;
    int rc = TSQ_OK;
    for (const Part &pt : parts) {
      if (pt.residue && rc == TSQ_OK) rc = TSQ_E_INVALID_RESIDUE;
      if (pt.last != TSQ_OK) rc = pt.last;
    }
    return rc;
  }
  int rc = TSQ_OK;
  for (int64_t q = 0; q < count; ++q) {
    const int64_t k = begin + q;
    tsq_result &o = dst ? out[dst[q]] : out[q];
    const ResultDev &d = r[k];
    const bool rows = b->out_mode == kOutTrace && d.status == TSQ_OK;
    const PairDev &pd = b->pairs_h[size_t(k)];
    const int e = collect_one(d, rows ? b->aln_h.as<char>() + b->aln_off_h[size_t(k)] : nullptr,
                              int64_t(pd.a_len) + pd.b_len, o);
    if (e) return e;
    // A residue error is the caller's; anything else is the library's.
    if (d.status != TSQ_OK && (rc == TSQ_OK || d.status != TSQ_E_INVALID_RESIDUE)) rc = d.status;
  }
  return rc;
}

int batch_results(tsq_batch *b, tsq_result *out) { return batch_results(b, out, nullptr); }

int batch_results(tsq_batch *b, tsq_result *out, const int32_t *dst) {
  if (!b || (b->n > 0 && !out)) return TSQ_E_INVALID_ARG;
  int rc = batch_fetch_async(b);
  if (rc) return rc;
  TSQ_TRY(cudaStreamSynchronize(b->stream));
  return batch_collect(b, 0, b->n, out, dst);
}

int64_t batch_device_bytes(const tsq_batch *b) {
  const tsq::DevBuf *bufs[] = {&b->seqs, &b->codes, &b->pairs, &b->tasks, &b->wtasks, &b->res, &b->bnd,
                               &b->planes, &b->plane_off, &b->aln, &b->aln_off, &b->shape_g, &b->shape_r,
                               &b->counters, &b->lut, &b->matrix, &b->overflow, &b->rerun_tasks, &b->rerun_wtasks,
                               &b->ccodes, &b->clut, &b->cmatrix};
  int64_t total = 0;
  for (const tsq::DevBuf *d : bufs) total += int64_t(d->cap);
  return total;
}

}  // namespace tsq
