// resident.cu -- the device-resident request loop (see resident.h).
#include "resident.h"

#include <algorithm>
#include <cstring>

#include "fill_i16.cuh"
#include "fill_i32.cuh"
#include "trace.h"

namespace tsq {
namespace resident {
namespace {

constexpr int kBndCols = ((kMaxLen + 31) / 32 + 1) * 32;  // one staged chunk past the longest row
constexpr size_t kMatSlot = 704;                           // 26 x 26 int8, per warp
constexpr size_t kMatSlot16 = fill::kMatBytes16;           // class matrix of the int16x2 fill, per warp
constexpr int kWarps = fill::kThreads / 32;
static_assert(fill::kThreads == fill::kThreads16, "both fills index their profiles by the same thread");

// Each warp's private rings: one 32-lane group, as large as the int32
// fill's (top-row entries of up to 16 bytes, 128-byte code ring) or the
// int16x2 fill's (up to 16-byte entries, 256-byte code ring) need.
constexpr size_t kWarpRings32 = size_t(fill::kTopRing) * 16 + fill::kRingPad + fill::kCodeRing + fill::kRingPad;
constexpr size_t kWarpRings =
    kWarpRings32 > fill::warp_rings16_bytes(kOutIdent) ? kWarpRings32 : fill::warp_rings16_bytes(kOutIdent);

// Per-thread profile area: the int16x2 fill's (two 8-row words per class,
// 26 classes at most) holds the int32 fill's (one word per letter); a
// thread uses one of them at a time.  Then the identity match table.
constexpr size_t kProfBytes = fill::smem16_prof_bytes(kLetters);
constexpr size_t kMatchBytes = fill::smem16_match_bytes(kOutIdent, kLetters);

__host__ __device__ constexpr size_t smem_bytes() {
  return size_t(kWarps) * (kMatSlot + kMatSlot16) + kProfBytes + kMatchBytes + size_t(kWarps) * kWarpRings;
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Runs one pair with the int32 fill of fill_i32.cuh on a 32-lane group.
template <bool LOCAL, int OUT>
__device__ __forceinline__ void run_pair(const FillArgs &a, const int8_t *s_mat, uint2 *s_prof, uint8_t *s_rings,
                                         uint8_t *my_rings) {
  fill::fill_warp_task<32, 8, LOCAL, OUT>(a, s_mat, s_prof, s_rings, 0, 1, 0, my_rings);
}

// Runs one pair with the int16x2 fill of fill_i16.cuh on a 32-lane group.
template <bool LOCAL, bool CHECK, int OUT>
__device__ __forceinline__ void run_pair16(const FillArgs &a, const int8_t *s_mat16, uint2 *s_prof, uint32_t *s_match,
                                           uint8_t *my_rings) {
  fill::fill16_warp_task<LOCAL, CHECK, OUT>(a, s_mat16, s_prof, s_match, nullptr, 0, 1, 0, 32, 5, my_rings);
}

__global__ void __launch_bounds__(fill::kThreads, 1)
    resident_kernel(const ReqDesc *reqs, const Task *ring, Ctl *ctl, HostBlock *host, int32_t *bnd, int32_t idle_polls) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ int32_t s_pair[kWarps];  // the decoded pair index of each warp's task
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int8_t *s_mat = reinterpret_cast<int8_t *>(smem + size_t(w) * kMatSlot);
  int8_t *s_mat16 = reinterpret_cast<int8_t *>(smem + size_t(kWarps) * kMatSlot + size_t(w) * kMatSlot16);
  uint8_t *p = smem + size_t(kWarps) * (kMatSlot + kMatSlot16);
  uint2 *s_prof = reinterpret_cast<uint2 *>(p);
  uint32_t *s_match = reinterpret_cast<uint32_t *>(p + kProfBytes);
  uint8_t *s_rings = p + kProfBytes + kMatchBytes;
  uint8_t *my_rings = s_rings + size_t(w) * kWarpRings;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int32_t *my_bnd = bnd + size_t(warp) * kBndCols * 4;  // one row of int4 entries
  uint64_t cached = 0, cached16 = 0;  // publication whose matrices this warp holds (0: none)
  int idle = 0;
  bool stopped = false;
  for (;;) {
    long long idx = -1;
    int stop = 0;
    if (lane == 0) {
      stop = host->stop;
      if (!stop) {
        const unsigned long long h = *reinterpret_cast<volatile unsigned long long *>(&ctl->head);
        const unsigned long long t = ld_acquire(&ctl->tail);
        if (h < t) idx = atomicCAS(&ctl->head, h, h + 1) == h ? (long long)h : -2;
      }
    }
    idx = __shfl_sync(0xffffffffu, idx, 0);
    stop = __shfl_sync(0xffffffffu, stop, 0);
    if (stop) {
      stopped = true;
      break;
    }
    if (idx == -2) continue;  // another warp took that task: try again at once
    if (idx < 0) {
      // Empty queue: a bounded wait, then leave (the host relaunches).
      if (++idle >= idle_polls) break;
      __nanosleep(idle < 64 ? 32 : 1000);
      continue;
    }
    idle = 0;
    __threadfence();  // the task and its request were published before the tail
    const Task task = ring[idx & (kRingCap - 1)];
    const ReqDesc rq = reqs[task.req];
    const int32_t pair = task.pair & 0xFFFFFF, lane_type = task.pair >> 24;
    const bool packed = lane_type != kLaneI32;
    if (lane == 0) s_pair[w] = pair;
    if (rq.uid != cached) {
      for (int k = lane; k < kLetters * kLetters; k += 32) s_mat[k] = rq.matrix[k];
      cached = rq.uid;
    }
    if (packed && rq.uid != cached16) {
      // Class scores, one 32-byte row per class, then a zero row for the
      // padding rows (index nclasses).
      for (int k = lane; k < int(kMatSlot16); k += 32) {
        const int x = k / fill::kMatRow16, c = k % fill::kMatRow16;
        s_mat16[k] = (x < rq.nclasses && c < rq.nclasses) ? rq.cmatrix[x * rq.nclasses + c] : int8_t(0);
      }
      cached16 = rq.uid;
    }
    // The pair's letter codes (and, for the packed fill, class codes),
    // written by this warp (another warp coding a shared sequence writes the
    // same bytes); the fill reads them below.  The packed fill's staging
    // reads class codes up to 64 bytes past a sequence and uses them as
    // profile indices unchecked: those are written too, from the residues
    // and the buffer's padding (class 0 for any byte outside the scheme).
    {
      const PairDev pd = rq.pairs[pair];
      for (int k = lane; k < pd.a_len; k += 32) rq.codes[pd.a_off + k] = rq.lut[rq.seqs[pd.a_off + k]];
      for (int k = lane; k < pd.b_len; k += 32) rq.codes[pd.b_off + k] = rq.lut[rq.seqs[pd.b_off + k]];
      if (packed) {
        const int64_t lim = rq.seqs_len + 128;
        for (int64_t k = pd.a_off + lane; k < min(pd.a_off + pd.a_len + 64, lim); k += 32)
          rq.ccodes[k] = rq.clut[rq.seqs[k]];
        for (int64_t k = pd.b_off + lane; k < min(pd.b_off + pd.b_len + 64, lim); k += 32)
          rq.ccodes[k] = rq.clut[rq.seqs[k]];
        // The code ring may hold another fill's letter codes (up to 0xFF);
        // the packed step reads ring bytes as class indices unchecked.
        uint8_t *code_ring = my_rings + fill::smem16_top_stride(rq.out == kOutIdent ? kOutIdent : kOutScore);
        for (int k = lane; k < fill::kCodeRing16 + fill::kRingPad; k += 32) code_ring[k] = 0;
      }
      __syncwarp();
    }
    FillArgs a{};
    a.codes = rq.codes;
    a.pairs = rq.pairs;
    a.tasks = &s_pair[w];
    a.gap_open = rq.gap_open;
    a.gap_extend = rq.gap_extend;
    a.res = rq.res;
    a.bnd = my_bnd;
    a.bnd_cols = kBndCols;
    bool rerun = !packed;
    if (packed) {
      a.one = 1u;
      a.ccodes = rq.ccodes;
      a.nclasses = rq.nclasses;
      a.max_score = rq.max_score;
      a.overflow = rq.overflow;
      const bool check = lane_type == kLaneI16Checked;
      if (rq.out == kOutIdent) {
        if (check)
          run_pair16<false, true, kOutIdent>(a, s_mat16, s_prof, s_match, my_rings);
        else
          run_pair16<false, false, kOutIdent>(a, s_mat16, s_prof, s_match, my_rings);
      } else if (rq.local) {
        if (check)
          run_pair16<true, true, kOutScore>(a, s_mat16, s_prof, s_match, my_rings);
        else
          run_pair16<true, false, kOutScore>(a, s_mat16, s_prof, s_match, my_rings);
      } else {
        if (check)
          run_pair16<false, true, kOutScore>(a, s_mat16, s_prof, s_match, my_rings);
        else
          run_pair16<false, false, kOutScore>(a, s_mat16, s_prof, s_match, my_rings);
      }
      __syncwarp();
      // A checked pair that came near 32767 runs again in int32.
      if (check) rerun = *reinterpret_cast<volatile int32_t *>(&rq.overflow[pair]) != 0;
    }
    if (rerun) {
      if (rq.out == kOutIdent) {
        if (rq.local)
          run_pair<true, kOutIdent>(a, s_mat, s_prof, s_rings, my_rings);
        else
          run_pair<false, kOutIdent>(a, s_mat, s_prof, s_rings, my_rings);
      } else {
        if (rq.local)
          run_pair<true, kOutScore>(a, s_mat, s_prof, s_rings, my_rings);
        else
          run_pair<false, kOutScore>(a, s_mat, s_prof, s_rings, my_rings);
      }
    }
    __syncwarp();
    if (lane == 0) {
      __threadfence_system();  // the result is visible before the count is
      atomicAdd_system(const_cast<uint32_t *>(&host->done[task.req]), 1u);
    }
  }
  if (lane == 0 && atomicSub(&ctl->live, 1) == 1) {
    host->exit_status = stopped ? kStopped : kIdleExit;
    __threadfence_system();
  }
}

__global__ void publish_kernel(unsigned long long *tail, unsigned long long value) {
  __threadfence();
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(tail), "l"(value) : "memory");
}

int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

// Where a request's buffers sit in its arena range.  What the host sends
// comes first, in one block -- the residues (with 128 bytes of padding),
// the pair table, the 26 x 26 matrix (a 1 KiB slot), the letter table, the
// class scores (a 1 KiB slot) and the class table -- then what the kernel
// writes: the letter codes, the class codes, the results and the
// overflow flags of the checked int16x2 pairs.
struct Layout {
  uint8_t *seqs;
  PairDev *pairs;
  int8_t *mat;
  uint8_t *lut;
  int8_t *cmat;
  uint8_t *clut;
  uint8_t *codes;
  uint8_t *ccodes;
  ResultDev *res;
  int32_t *overflow;
  int64_t host_bytes;  // the block the host sends
};

Layout layout(uint8_t *arena, const Range &range, int64_t len, int64_t n) {
  Layout l;
  l.seqs = arena + range.off;
  l.pairs = reinterpret_cast<PairDev *>(l.seqs + align256(len + 128));
  l.mat = reinterpret_cast<int8_t *>(reinterpret_cast<uint8_t *>(l.pairs) + align256(24 * n));
  l.lut = reinterpret_cast<uint8_t *>(l.mat) + 1024;
  l.cmat = reinterpret_cast<int8_t *>(l.lut + 256);
  l.clut = reinterpret_cast<uint8_t *>(l.cmat) + 1024;
  l.codes = l.clut + 256;
  l.ccodes = l.codes + align256(len + 128);
  l.res = reinterpret_cast<ResultDev *>(l.ccodes + align256(len + 128));
  l.overflow = reinterpret_cast<int32_t *>(reinterpret_cast<uint8_t *>(l.res) + align256(32 * n));
  l.host_bytes = l.codes - l.seqs;
  return l;
}

}  // namespace

int64_t arena_need(int64_t seqs_len, int64_t n) {
  return 3 * align256(seqs_len + 128) + align256(24 * n) + align256(32 * n) + align256(4 * n) + 2 * (1024 + 256);
}

// Bytes of the page-locked block a request is staged in: the arena block
// the host sends, then the request descriptor and the tasks.
int64_t stage_bytes(int64_t seqs_len, int64_t n) {
  return align256(seqs_len + 128) + align256(24 * n) + 2 * (1024 + 256) + 256 + 8 * n;
}

Loop::~Loop() { shutdown(); }

int Loop::init(int device, int64_t arena_bytes, int32_t idle_polls) {
  device_ = device;
  idle_polls_ = idle_polls > 0 ? idle_polls : (1 << 20);
  if (cudaSetDevice(device) != cudaSuccess) return TSQ_E_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return TSQ_E_CUDA;
  // One block of 4 warps on every other SM: the loop leaves most of each
  // SM to the ticks that run beside it.
  blocks_ = std::max(1, sms / 2);
  warps_ = blocks_ * kWarps;
  if (cudaFuncSetAttribute(resident_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_bytes())) !=
      cudaSuccess)
    return TSQ_E_CUDA;
  arena_bytes_ = align256(std::max<int64_t>(arena_bytes, int64_t(64) << 20));
  if (cudaMalloc(&arena_, size_t(arena_bytes_)) != cudaSuccess) return TSQ_E_NOMEM;
  free_.assign(1, Range{0, arena_bytes_});
  if (cudaMalloc(&reqs_, sizeof(ReqDesc) * kMaxReqs) != cudaSuccess) return TSQ_E_NOMEM;
  if (cudaMalloc(&ring_, sizeof(Task) * size_t(kRingCap)) != cudaSuccess) return TSQ_E_NOMEM;
  if (cudaMalloc(&ctl_, sizeof(Ctl)) != cudaSuccess) return TSQ_E_NOMEM;
  if (cudaMalloc(&bnd_, size_t(warps_) * kBndCols * 16) != cudaSuccess) return TSQ_E_NOMEM;
  if (cudaMemset(ctl_, 0, sizeof(Ctl)) != cudaSuccess) return TSQ_E_CUDA;
  if (cudaHostAlloc(reinterpret_cast<void **>(&host_), sizeof(HostBlock), cudaHostAllocMapped) != cudaSuccess)
    return TSQ_E_NOMEM;
  std::memset(const_cast<HostBlock *>(host_), 0, sizeof(HostBlock));
  if (cudaHostGetDevicePointer(reinterpret_cast<void **>(&host_dev_), host_, 0) != cudaSuccess) return TSQ_E_CUDA;
  if (cudaStreamCreateWithFlags(&kstream_, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ustream_, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&kdone_, cudaEventDisableTiming) != cudaSuccess)
    return TSQ_E_CUDA;
  for (int32_t k = kMaxReqs - 1; k >= 0; --k) free_slots_.push_back(k);
  stages_.reset(new PinBuf[kMaxReqs]);
  return TSQ_OK;
}

bool Loop::eligible(const tsq_params &p, const std::vector<tsq_pair_desc> &pairs) {
  if (p.output != TSQ_OUT_SCORE && p.output != TSQ_OUT_IDENTITY) return false;
  if (pairs.empty() || int64_t(pairs.size()) > kMaxPairs) return false;
  int64_t lo = 3 * int64_t(p.gap_open) + 128;
  for (const tsq_pair_desc &d : pairs) {
    if (d.a_len > kMaxLen || d.b_len > kMaxLen) return false;
    if (p.output == TSQ_OUT_IDENTITY && int64_t(d.a_len) + d.b_len > 65535) return false;
    // The int32 fill's range: values stay far above its minus infinity.
    if (lo + (int64_t(d.a_len) + d.b_len + 1) * p.gap_extend >= (int64_t(1) << 28)) return false;
  }
  return true;
}

int Loop::admit(int64_t seqs_len, int64_t n, int32_t *slot, Range *range) {
  if (free_slots_.empty()) return TSQ_E_PENDING;
  const int64_t need = arena_need(seqs_len, n);
  for (size_t k = 0; k < free_.size(); ++k)
    if (free_[k].bytes >= need) {
      range->off = free_[k].off;
      range->bytes = need;
      free_[k].off += need;
      free_[k].bytes -= need;
      if (free_[k].bytes == 0) free_.erase(free_.begin() + int64_t(k));
      *slot = free_slots_.back();
      free_slots_.pop_back();
      return TSQ_OK;
    }
  return need > arena_bytes_ ? TSQ_E_REJECTED : TSQ_E_PENDING;
}

void Loop::release(int32_t slot, const Range &range) {
  free_slots_.push_back(slot);
  stages_[size_t(slot)].release();
  // Insert by offset and merge with the neighbours.
  auto it = std::lower_bound(free_.begin(), free_.end(), range,
                             [](const Range &a, const Range &b) { return a.off < b.off; });
  it = free_.insert(it, range);
  if (it + 1 != free_.end() && it->off + it->bytes == (it + 1)->off) {
    it->bytes += (it + 1)->bytes;
    free_.erase(it + 1);
  }
  if (it != free_.begin() && (it - 1)->off + (it - 1)->bytes == it->off) {
    (it - 1)->bytes += it->bytes;
    free_.erase(it);
  }
}

int Loop::publish(int32_t slot, const Range &range, const std::vector<uint8_t> &seqs,
                  const std::vector<tsq_pair_desc> &pairs, const tsq_params &p, const int8_t *custom_score,
                  const uint8_t *custom_valid) {
  TraceRange tr("resident publish");
  tsq_params q = p;
  if (q.matrix == TSQ_MATRIX_CUSTOM) {
    q.custom_score = custom_score;
    q.custom_valid = custom_valid;
  }
  Scheme sc;
  int rc = build_scheme(&q, &sc);
  if (rc) return rc;
  const int64_t len = int64_t(seqs.size()), n = int64_t(pairs.size());
  const Layout l = layout(arena_, range, len, n);
  // Everything goes into one page-locked block, kept until the slot is
  // released (by then the kernel has finished the request, so the copies
  // from it are long done): the arena block, the descriptor, the tasks.
  PinBuf &stage = stages_[size_t(slot)];
  if (stage.ensure(size_t(stage_bytes(len, n))) != cudaSuccess) return TSQ_E_NOMEM;
  uint8_t *h = stage.as<uint8_t>();
  const int64_t off_pairs = reinterpret_cast<uint8_t *>(l.pairs) - l.seqs;
  const int64_t off_mat = reinterpret_cast<uint8_t *>(l.mat) - l.seqs;
  const int64_t off_lut = l.lut - l.seqs;
  const int64_t off_cmat = reinterpret_cast<uint8_t *>(l.cmat) - l.seqs;
  const int64_t off_clut = l.clut - l.seqs;
  if (len > 0) std::memcpy(h, seqs.data(), size_t(len));
  // The 128 bytes of padding past the residues: the packed fill's class
  // codes are written from them (any byte outside the scheme is class 0).
  std::memset(h + len, 0, 128);
  std::memcpy(h + off_pairs, pairs.data(), size_t(24 * n));
  std::memcpy(h + off_mat, sc.score, sizeof(sc.score));
  build_lut(sc, h + off_lut);
  std::memcpy(h + off_cmat, sc.cscore, size_t(sc.nclasses) * size_t(sc.nclasses));
  build_class_lut(sc, h + off_clut);
  static_assert(sizeof(PairDev) == sizeof(tsq_pair_desc), "pair layouts must match");
  const int out_mode = q.output == TSQ_OUT_IDENTITY ? int32_t(kOutIdent) : int32_t(kOutScore);
  ReqDesc *desc = reinterpret_cast<ReqDesc *>(h + l.host_bytes);
  *desc = ReqDesc{l.seqs,     l.codes,       l.lut,      l.pairs,       l.res,        l.mat,
                  q.gap_open, q.gap_extend,  q.mode == TSQ_LOCAL ? 1 : 0, out_mode,    l.ccodes,
                  l.clut,     l.cmat,        l.overflow, len,           sc.nclasses,  sc.max_score,
                  ++published_};
  // Lane type per pair, by the batch planner's range rules: int16x2 where
  // every value provably fits, checked int16x2 where only the lower bound
  // is proven (or lane TSQ_LANE_I16 asks for it), int32 otherwise (and for
  // local identity, which has no int16x2 fill).
  const bool try16 = q.lane != TSQ_LANE_I32 && !(out_mode == kOutIdent && q.mode == TSQ_LOCAL);
  const int64_t go = q.gap_open, ge = q.gap_extend;
  const int64_t smax = std::max<int32_t>(sc.max_score, 0), sneg = std::max<int64_t>(0, -int64_t(sc.min_score));
  Task *tasks = reinterpret_cast<Task *>(h + l.host_bytes + 256);
  for (int64_t k = 0; k < n; ++k) {
    const tsq_pair_desc &d = pairs[size_t(k)];
    int32_t lt = kLaneI32;
    if (try16) {
      const int64_t lowest = 3 * go + (int64_t(d.a_len) + 512 + d.b_len + 1) * ge + go + ge + 128 + sneg;
      const bool lower_ok = lowest + go + ge < 31000 && ge <= 700;
      const bool upper_ok = smax * std::min(d.a_len, d.b_len) + smax < 32767;
      if (lower_ok) lt = (upper_ok && q.lane == TSQ_LANE_AUTO) ? kLaneI16 : kLaneI16Checked;
    }
    tasks[k] = Task{slot, int32_t(k) | (lt << 24)};
  }
  host_->done[slot] = 0;
  cudaStream_t st = ustream_;
  if (cudaMemcpyAsync(l.seqs, h, size_t(l.host_bytes), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(reqs_ + slot, desc, sizeof(ReqDesc), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return TSQ_E_CUDA;
  // The tasks, in one or two pieces around the ring's end.
  const int64_t at = int64_t(tail_ & (kRingCap - 1));
  const int64_t first = std::min<int64_t>(n, kRingCap - at);
  if (cudaMemcpyAsync(ring_ + at, tasks, sizeof(Task) * size_t(first), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return TSQ_E_CUDA;
  if (first < n &&
      cudaMemcpyAsync(ring_, tasks + first, sizeof(Task) * size_t(n - first), cudaMemcpyHostToDevice, st) !=
          cudaSuccess)
    return TSQ_E_CUDA;
  tail_ += static_cast<unsigned long long>(n);
  publish_kernel<<<1, 1, 0, st>>>(&ctl_->tail, tail_);
  if (cudaGetLastError() != cudaSuccess) return TSQ_E_CUDA;
  outstanding_ += n;
  return tend();
}

int Loop::launch() {
  TraceRange tr("resident launch");
  const int32_t live = warps_;
  host_->exit_status = kRunning;
  if (cudaMemcpyAsync(&ctl_->live, &live, sizeof(live), cudaMemcpyHostToDevice, kstream_) != cudaSuccess)
    return TSQ_E_CUDA;
  resident_kernel<<<blocks_, fill::kThreads, smem_bytes(), kstream_>>>(reqs_, ring_, ctl_, host_dev_, bnd_,
                                                                       idle_polls_);
  if (cudaGetLastError() != cudaSuccess) return TSQ_E_CUDA;
  if (cudaEventRecord(kdone_, kstream_) != cudaSuccess) return TSQ_E_CUDA;
  running_ = true;
  ++launches_;
  return TSQ_OK;
}

int Loop::tend() {
  if (running_) {
    const cudaError_t q = cudaEventQuery(kdone_);
    if (q == cudaErrorNotReady) return TSQ_OK;
    if (q != cudaSuccess) return TSQ_E_CUDA;
    running_ = false;
    if (host_->exit_status == kIdleExit) ++idle_exits_;
  }
  // Tasks published and not all done: the loop must be on the device.
  if (outstanding_ > 0 && !host_->stop) return launch();
  return TSQ_OK;
}

int Loop::fetch(const Range &range, int64_t seqs_len, int64_t n, tsq_result *out) {
  TraceRange tr("resident fetch");
  const Layout l = layout(arena_, range, seqs_len, n);
  std::vector<ResultDev> res(static_cast<size_t>(n));
  if (cudaSetDevice(device_) != cudaSuccess) return TSQ_E_CUDA;
  if (n > 0 && cudaMemcpy(res.data(), l.res, sizeof(ResultDev) * size_t(n), cudaMemcpyDeviceToHost) != cudaSuccess)
    return TSQ_E_CUDA;
  // The same status rule as a batch: a residue error is the caller's, any
  // other error is reported over it.
  int rc = TSQ_OK;
  for (int64_t k = 0; k < n; ++k) {
    const ResultDev &d = res[size_t(k)];
    tsq_result &o = out[k];
    o.score = d.score;
    o.a_begin = d.a_begin;
    o.a_end = d.a_end;
    o.b_begin = d.b_begin;
    o.b_end = d.b_end;
    o.n_ident = d.n_ident;
    o.n_cols = d.n_cols;
    o.status = d.status;
    o.aln_a = o.aln_b = nullptr;
    if (d.status != TSQ_OK && (rc == TSQ_OK || d.status != TSQ_E_INVALID_RESIDUE)) rc = d.status;
  }
  return rc;
}

void Loop::shutdown() {
  if (host_) {
    host_->stop = 1;
    if (running_) cudaEventSynchronize(kdone_);
    running_ = false;
  }
  if (kdone_) cudaEventDestroy(kdone_);
  if (kstream_) cudaStreamDestroy(kstream_);
  if (ustream_) cudaStreamDestroy(ustream_);
  if (arena_) cudaFree(arena_);
  if (reqs_) cudaFree(reqs_);
  if (ring_) cudaFree(ring_);
  if (ctl_) cudaFree(ctl_);
  if (bnd_) cudaFree(bnd_);
  if (host_) cudaFreeHost(const_cast<HostBlock *>(host_));
  kdone_ = nullptr;
  kstream_ = ustream_ = nullptr;
  arena_ = nullptr;
  reqs_ = nullptr;
  ring_ = nullptr;
  ctl_ = nullptr;
  bnd_ = nullptr;
  host_ = nullptr;
}

}  // namespace resident
}  // namespace tsq
