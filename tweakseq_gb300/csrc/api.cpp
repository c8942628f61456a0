// api.cpp -- the extern "C" entry points declared in include/tweakseq_gb300.h.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <memory>
#include <new>
#include <vector>

#include "engine.h"
#include "trace.h"

namespace {

// One cached engine object per host thread and device, so that repeated
// plain or batch calls reuse their device buffers instead of allocating.
struct ThreadCache {
  tsq::PairPath pair_path;  // tsq_align_pair's one-pair path
  std::unique_ptr<tsq_batch> pair_engine;
  std::unique_ptr<tsq_batch> batch_engine;
  std::vector<std::unique_ptr<tsq_batch>> chunk_engines;  // chunks 1.. of a large call
  int pair_dev = -1, batch_dev = -1;
  // A chunked call's residue segments go up on this stream.
  cudaStream_t input_stream = nullptr;
  std::vector<cudaEvent_t> seg_events;
  int input_dev = -1;
  // A chunked call's cost order: each pair's cost bin, the pairs in cost
  // order and their input positions.
  std::vector<uint8_t> order_bin;
  std::vector<tsq_pair_desc> order_pairs;
  std::vector<int32_t> order_index;
  ~ThreadCache() {
    for (cudaEvent_t e : seg_events) cudaEventDestroy(e);
    if (input_stream) cudaStreamDestroy(input_stream);
  }
};

// A score or identity call of at least 2 * kChunkPairs pairs runs as up to
// kMaxChunks chunks (see align_in_chunks).
constexpr int64_t kChunkPairs = 16384;
constexpr int kMaxChunks = 3;

ThreadCache &cache() {
  thread_local ThreadCache c;
  return c;
}

int current_device(const tsq_batch_opts *opts, int *dev) {
  if (opts && opts->device >= 0) {
    *dev = opts->device;
    return TSQ_OK;
  }
  const cudaError_t e = cudaGetDevice(dev);
  return e == cudaSuccess ? TSQ_OK : TSQ_E_CUDA;
}

template <class F>
int guarded(F &&f) {
  try {
    return f();
  } catch (const std::bad_alloc &) {
    return TSQ_E_NOMEM;
  } catch (...) {
    return TSQ_E_CUDA;
  }
}

// A large score or identity call runs as a few chunks, each planned by its
// own batch object and run on its own stream; each later chunk is planned on
// the host while the earlier ones run, and the chunks' persistent launches
// fill each other's tails on the device.  Each pair's result does not depend
// on the chunking.  Two ways of cutting and feeding the chunks:
// - Input the device can read in place (page-locked, 16-byte aligned): one
//   kernel encodes the residues straight from host memory while the host
//   plans the first chunk.  Chunks are cut by cost: chunk 0 takes the
//   costliest tenth of the pairs (cells, binned at four steps per octave, in
//   input order within a bin), chunk 1 the next three tenths, chunk 2 the
//   rest.  The first plan is small, its long pairs keep the device busy
//   while the host plans the rest, and the last chunk -- launched last --
//   holds the short pairs, so the call ends with a short tail.  Results go
//   back to their input positions.  (Chunks of consecutive pairs left the
//   longest pairs of the last chunk to start late: 5.4 ms of fills for
//   4.97 ms of work on the 100,000-pair batch.)
// - Other (pageable) input: chunks of consecutive pairs growing in size
//   (1/6, 2/6, 3/6 with three chunks), the residues uploaded in segments on
//   an input stream -- segment k holds what chunk k reads beyond the earlier
//   segments -- so a chunk waits only for the residues up to its own, and
//   the host copies the next segment while the device fills earlier chunks.
int align_in_chunks(ThreadCache &c, tsq_batch *e, const uint8_t *seqs, int64_t seqs_len, const tsq_pair_desc *pairs,
                    int64_t n, const tsq_params *p, const tsq_batch_opts *opts, tsq_result *out) {
  if (n > INT32_MAX / 2) return TSQ_E_TOO_LARGE;
  const int K = int(std::min<int64_t>(kMaxChunks, n / kChunkPairs));
  while (int(c.chunk_engines.size()) < K - 1) c.chunk_engines.emplace_back(new tsq_batch());
  std::vector<tsq_batch *> eng(static_cast<size_t>(K));
  eng[0] = e;
  for (int k = 1; k < K; ++k) eng[size_t(k)] = c.chunk_engines[size_t(k - 1)].get();
  int dev = 0;
  if (opts && opts->device >= 0)
    dev = opts->device;
  else if (cudaGetDevice(&dev) != cudaSuccess)
    return TSQ_E_CUDA;
  if (cudaSetDevice(dev) != cudaSuccess) return TSQ_E_CUDA;
  if (c.input_dev != dev) {
    for (cudaEvent_t ev : c.seg_events) cudaEventDestroy(ev);
    c.seg_events.clear();
    if (c.input_stream) cudaStreamDestroy(c.input_stream);
    c.input_stream = nullptr;
    if (cudaStreamCreateWithFlags(&c.input_stream, cudaStreamNonBlocking) != cudaSuccess) return TSQ_E_CUDA;
    c.input_dev = dev;
  }
  while (int(c.seg_events.size()) < K) {
    cudaEvent_t ev;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return TSQ_E_CUDA;
    c.seg_events.push_back(ev);
  }
  const tsq_batch_opts o{dev, 0, opts ? opts->autotune : 0, opts ? opts->wait_polls : 0};

  cudaPointerAttributes attr{};
  const bool in_place = seqs_len > 0 && cudaPointerGetAttributes(&attr, seqs) == cudaSuccess &&
                        attr.type == cudaMemoryTypeHost && attr.devicePointer != nullptr &&
                        reinterpret_cast<uintptr_t>(attr.devicePointer) % 16 == 0;
  cudaGetLastError();  // (a pointer CUDA does not know leaves an error behind)
  int rc = TSQ_OK;
  if (in_place) {  // the encode runs while the host orders and plans
    rc = tsq::input_prepare(e, seqs_len, p, &o);
    if (rc == TSQ_OK)
      rc = tsq::input_encode_mapped(e, static_cast<const uint8_t *>(attr.devicePointer), c.input_stream);
    if (rc == TSQ_OK && cudaEventRecord(c.seg_events[0], c.input_stream) != cudaSuccess) rc = TSQ_E_CUDA;
  }

  // Chunk k covers positions [cut[k], cut[k+1]) of the chunk order: the
  // input order, or (in place) the cost order held in c.order_pairs with the
  // input index of each position in c.order_index.
  std::vector<int64_t> cut(static_cast<size_t>(K) + 1);
  int64_t cells = 0;
  const tsq_pair_desc *chunk_pairs = pairs;
  const int32_t *chunk_index = nullptr;
  if (in_place) {
    static const double kCut3[] = {0.0, 0.1, 0.4, 1.0}, kCut2[] = {0.0, 0.2, 1.0};
    for (int k = 0; k <= K; ++k) cut[size_t(k)] = int64_t(double(n) * (K == 3 ? kCut3[k] : kCut2[k]));
    cut[size_t(K)] = n;
    c.order_pairs.resize(size_t(n));
    c.order_index.resize(size_t(n));
    cells = tsq::cost_order(pairs, n, c.order_bin, c.order_pairs.data(), c.order_index.data());
    chunk_pairs = c.order_pairs.data();
    chunk_index = c.order_index.data();
  } else {
    // Chunk k ends at n * (1 + 2 + ... + (k+1)) / (1 + 2 + ... + K).
    const int64_t tri = int64_t(K) * (K + 1) / 2;
    for (int k = 0; k <= K; ++k) cut[size_t(k)] = n * (int64_t(k) * (k + 1) / 2) / tri;
    for (int64_t k = 0; k < n; ++k) cells += int64_t(std::max(pairs[k].a_len, 0)) * std::max(pairs[k].b_len, 0);
  }

  int launched = 0;
  int64_t uploaded = 0;  // (pageable) residues [0, uploaded) are on their way
  for (int k = 0; k < K && rc == TSQ_OK; ++k) {
    const int64_t b0 = cut[size_t(k)], nk = cut[size_t(k) + 1] - b0;
    const tsq_pair_desc *pk = chunk_pairs + b0;
    rc = tsq::batch_plan_chunk(eng[size_t(k)], k == 0 ? nullptr : e, seqs, seqs_len, pk, nk, p, &o, n, cells, true);
    if (rc != TSQ_OK) break;
    if (!in_place) {
      // This chunk's segment: whole 16-byte blocks, plus the 64 bytes past
      // a sequence end that the fills' staging reads; the last chunk takes
      // the rest of the buffer.
      int64_t hi = uploaded;
      for (int64_t q = 0; q < nk; ++q)
        hi = std::max({hi, pk[q].a_off + pk[q].a_len, pk[q].b_off + pk[q].b_len});
      hi = k == K - 1 ? seqs_len : std::min(seqs_len, (hi + 64 + 15) / 16 * 16);
      rc = tsq::input_segment(e, seqs, uploaded, hi, c.input_stream);
      if (rc == TSQ_OK && cudaEventRecord(c.seg_events[size_t(k)], c.input_stream) != cudaSuccess) rc = TSQ_E_CUDA;
      if (rc != TSQ_OK) break;
      uploaded = hi;
    }
    eng[size_t(k)]->input_ready = c.seg_events[in_place ? 0 : size_t(k)];
    rc = tsq::batch_run_async(eng[size_t(k)]);
    if (rc == TSQ_OK) ++launched;
  }
  int status = rc;
  for (int k = 0; k < launched; ++k) {
    const int sync_rc = tsq::batch_sync(eng[size_t(k)]);
    if (status != TSQ_OK && status != TSQ_E_INVALID_RESIDUE) continue;  // drain the rest, report the first error
    int r = sync_rc;
    if (r == TSQ_OK)
      r = chunk_index ? tsq::batch_results(eng[size_t(k)], out, chunk_index + cut[size_t(k)])
                      : tsq::batch_results(eng[size_t(k)], out + cut[size_t(k)]);
    if (r != TSQ_OK && (status == TSQ_OK || r != TSQ_E_INVALID_RESIDUE)) status = r;
  }
  // The input stream reads the caller's residues: done before return.
  cudaStreamSynchronize(c.input_stream);
  e->input_prepared = false;
  if (in_place && (rc == TSQ_E_INVALID_ARG || rc == TSQ_E_TOO_LARGE)) {
    // A chunk in cost order found a bad pair: report what one plan of the
    // whole call reports (the first bad pair in input order).
    const int whole = tsq::batch_plan(e, seqs, seqs_len, pairs, n, p, &o, false);
    if (whole != TSQ_OK) status = whole;
  }
  return status;
}

// Runs an alignment batch wave by wave (see tsq_align_batch).
int align_in_waves(tsq_batch *e, const uint8_t *seqs, int64_t seqs_len, const tsq_pair_desc *pairs, int64_t n,
                   const tsq_params *p, const tsq_batch_opts *opts, tsq_result *out,
                   const std::vector<int64_t> &bytes, int64_t budget) {
  std::vector<int64_t> order(static_cast<size_t>(n));
  for (int64_t k = 0; k < n; ++k) order[size_t(k)] = k;
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t x, int64_t y) { return bytes[size_t(x)] > bytes[size_t(y)]; });
  std::memset(out, 0, sizeof(tsq_result) * size_t(n));
  std::vector<tsq_pair_desc> wave;
  std::vector<tsq_result> res;
  int status = TSQ_OK;
  // Long pairs run one per CTA (the CTA fill): a wave that holds more of them
  // than one round of resident CTAs is cut at a whole number of rounds, or
  // its last few long pairs would start only when the first ones finish.
  const int slots = tsq::cta_blocks(tsq::kOutTrace, p->mode == TSQ_LOCAL);
  auto is_long = [&](int64_t k) {
    const tsq_pair_desc &d = pairs[k];
    return d.a_len > 0 && d.b_len > 0 && double((d.a_len + 255) / 256) * double(d.b_len + 31) > 20000.0;
  };
  int64_t begin = 0;
  while (begin < n) {
    int64_t end = begin, used = 0;
    while (end < n && (end == begin || used + bytes[size_t(order[size_t(end)])] <= budget))
      used += bytes[size_t(order[size_t(end++)])];
    if (slots > 0 && used <= budget) {
      int64_t nlong = 0;
      for (int64_t k = begin; k < end; ++k) nlong += is_long(order[size_t(k)]);
      if (nlong > slots && nlong % slots != 0) {
        const int64_t keep = nlong / slots * slots;
        int64_t seen = 0, cut = end;
        for (int64_t k = begin; k < end; ++k)
          if (is_long(order[size_t(k)]) && seen++ == keep) {
            cut = k;
            break;
          }
        end = cut;
      }
    }
    if (used > budget) {  // one pair alone is larger than the budget
      for (int64_t k = begin; k < end; ++k) out[order[size_t(k)]].status = TSQ_E_TOO_LARGE;
      status = status ? status : TSQ_E_TOO_LARGE;
      begin = end;
      continue;
    }
    wave.resize(size_t(end - begin));
    res.assign(size_t(end - begin), tsq_result{});
    for (int64_t k = begin; k < end; ++k) wave[size_t(k - begin)] = pairs[order[size_t(k)]];
    int rc = tsq::batch_plan(e, seqs, seqs_len, wave.data(), end - begin, p, opts, false);
    if (rc == TSQ_OK) rc = tsq::batch_run_async(e);
    if (rc == TSQ_OK) rc = tsq::batch_sync(e);
    if (rc == TSQ_OK || rc == TSQ_E_INVALID_RESIDUE) {
      const int rr = tsq::batch_results(e, res.data());
      rc = rc ? rc : rr;
    }
    if (rc != TSQ_OK && rc != TSQ_E_INVALID_RESIDUE) {
      tsq_results_free(res.data(), int64_t(res.size()));
      tsq_results_free(out, n);
      return rc;
    }
    if (rc) status = status ? status : rc;
    for (int64_t k = begin; k < end; ++k) out[order[size_t(k)]] = res[size_t(k - begin)];  // strings move over
    begin = end;
  }
  return status;
}

}  // namespace

extern "C" {

int tsq_version(int32_t *abi_version, const char **build) {
  if (abi_version) *abi_version = TSQ_ABI_VERSION;
  if (build) *build = "tweakseq_gb300 sm_103a int32 group-striped Gotoh fill + traceback";
  return TSQ_OK;
}

void tsq_result_free(tsq_result *r) {
  if (!r) return;
  std::free(r->aln_a);
  std::free(r->aln_b);
  r->aln_a = r->aln_b = nullptr;
}

void tsq_results_free(tsq_result *r, int64_t n) {
  if (!r) return;
  for (int64_t k = 0; k < n; ++k) tsq_result_free(&r[k]);
}

int64_t tsq_results_strings(const tsq_result *r, int64_t n, char *buf, int64_t buf_len) {
  if (n < 0 || (n > 0 && !r) || buf_len < 0) return TSQ_E_INVALID_ARG;
  int64_t total = 0;
  for (int64_t k = 0; k < n; ++k) {
    if (!r[k].aln_a || !r[k].aln_b) continue;
    if (r[k].n_cols < 0) return TSQ_E_INVALID_ARG;
    total += 2 * int64_t(r[k].n_cols);
  }
  if (!buf || buf_len < total) return total;
  char *o = buf;
  for (int64_t k = 0; k < n; ++k) {
    if (!r[k].aln_a || !r[k].aln_b) continue;
    const size_t L = size_t(r[k].n_cols);
    std::memcpy(o, r[k].aln_a, L);
    std::memcpy(o + L, r[k].aln_b, L);
    o += 2 * L;
  }
  return total;
}

int tsq_align_pair(const uint8_t *a, int32_t la, const uint8_t *b, int32_t lb, const tsq_params *p,
                   tsq_result *out) {
  tsq::TraceRange tr("tsq_align_pair");
  return guarded([&]() -> int {
    if (!out || !p || la < 0 || lb < 0 || (la > 0 && !a) || (lb > 0 && !b)) return TSQ_E_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    ThreadCache &c = cache();
    const int lean = tsq::pair_align(&c.pair_path, a, la, b, lb, p, out);
    if (lean != tsq::kPairNotTaken) return lean;
    // Calls the one-pair path leaves to the batch engine (forced checked
    // int16x2 lanes, pairs beyond its limits, bad parameters).
    int dev = 0;
    if (current_device(nullptr, &dev)) return TSQ_E_CUDA;
    if (!c.pair_engine || c.pair_dev != dev) {
      c.pair_engine.reset(new tsq_batch());
      c.pair_dev = dev;
    }
    // The pair's residues go up as one buffer: a then b.
    std::unique_ptr<uint8_t[]> buf(new uint8_t[size_t(la) + size_t(lb) + 1]);
    if (la) std::memcpy(buf.get(), a, size_t(la));
    if (lb) std::memcpy(buf.get() + la, b, size_t(lb));
    tsq_pair_desc d{0, la, la, lb};
    tsq_batch *e = c.pair_engine.get();
    int rc = tsq::batch_plan(e, buf.get(), int64_t(la) + lb, &d, 1, p, nullptr, true);
    if (rc) return rc;
    if ((rc = tsq::batch_run_async(e))) return rc;
    if ((rc = tsq::batch_sync(e))) return rc;
    return tsq::batch_results(e, out);
  });
}

int tsq_align_batch(const uint8_t *seqs, int64_t seqs_len, const tsq_pair_desc *pairs, int64_t n,
                    const tsq_params *p, const tsq_batch_opts *opts, tsq_result *out) {
  tsq::TraceRange tr("tsq_align_batch");
  return guarded([&]() -> int {
    if (n > 0 && !out) return TSQ_E_INVALID_ARG;
    int dev = 0;
    if (current_device(opts, &dev)) return TSQ_E_CUDA;
    ThreadCache &c = cache();
    if (!c.batch_engine || c.batch_dev != dev) {
      c.batch_engine.reset(new tsq_batch());
      c.batch_dev = dev;
    }
    tsq_batch *e = c.batch_engine.get();
    if (p && p->output == TSQ_OUT_ALIGNMENT && n > 1 && pairs) {
      // Traceback planes take about m*n/2 bytes per pair.  A batch whose
      // planes do not fit in the device memory that is free runs in waves:
      // pairs by plane size, largest first (so that the pairs of a wave are
      // alike and no wave waits on one long pair), each wave as many pairs as
      // fit in 85 % of the free memory less 2 GiB (the rest of the batch
      // object: residues, rows, results, strings).  Results land at the pairs' own
      // positions; a pair too large for any wave is TSQ_E_TOO_LARGE.
      if (cudaSetDevice(dev) != cudaSuccess) return TSQ_E_CUDA;
      std::vector<int64_t> bytes(static_cast<size_t>(n));
      int64_t total = 0;
      for (int64_t k = 0; k < n; ++k) {
        const tsq_pair_desc &d = pairs[k];
        bytes[size_t(k)] = (std::max<int64_t>(d.a_len, 0) + 255) * (std::max<int64_t>(d.b_len, 0) + 31) / 2 +
                           2 * (int64_t(std::max(d.a_len, 0)) + std::max(d.b_len, 0)) + 512;
        total += bytes[size_t(k)];
      }
      auto wave_budget = [&](int64_t *budget) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return false;
        const double avail = double(free_b + e->planes.cap + e->aln.cap);
        *budget = std::max(int64_t(0.85 * avail) - (int64_t(2) << 30), int64_t(0.5 * avail));
        // TSQ_WAVE_BUDGET_BYTES lowers the budget (tests use it to force waves).
        if (const char *env = std::getenv("TSQ_WAVE_BUDGET_BYTES")) {
          const long long v = std::atoll(env);
          if (v > 0) *budget = std::min<int64_t>(*budget, v);
        }
        return true;
      };
      int64_t budget = 0;
      if (!wave_budget(&budget)) return TSQ_E_CUDA;
      if (total > budget) {
        // Memory the engine's pool keeps mapped but does not use goes back
        // first (only when the batch would not fit: unmapping costs about as
        // much as mapping).
        tsq::trim_engine_pool(dev);
        if (!wave_budget(&budget)) return TSQ_E_CUDA;
      }
      if (total > budget) return align_in_waves(e, seqs, seqs_len, pairs, n, p, opts, out, bytes, budget);
    }
    if (p && p->output != TSQ_OUT_ALIGNMENT && n >= 2 * kChunkPairs && pairs)
      return align_in_chunks(c, e, seqs, seqs_len, pairs, n, p, opts, out);
    int rc = tsq::batch_plan(e, seqs, seqs_len, pairs, n, p, opts, false);
    if (rc) return rc;
    if ((rc = tsq::batch_run_async(e))) return rc;
    if ((rc = tsq::batch_sync(e))) return rc;
    return tsq::batch_results(e, out);
  });
}

int tsq_batch_create(const uint8_t *seqs, int64_t seqs_len, const tsq_pair_desc *pairs, int64_t n,
                     const tsq_params *p, const tsq_batch_opts *opts, tsq_batch **out) {
  return guarded([&]() -> int {
    if (!out) return TSQ_E_INVALID_ARG;
    *out = nullptr;
    std::unique_ptr<tsq_batch> b(new tsq_batch());
    const int rc = tsq::batch_plan(b.get(), seqs, seqs_len, pairs, n, p, opts, false);
    if (rc) return rc;
    *out = b.release();
    return TSQ_OK;
  });
}

int tsq_batch_run(tsq_batch *b) {
  return guarded([&]() -> int {
    const int rc = tsq::batch_run_async(b);
    return rc ? rc : tsq::batch_sync(b);
  });
}

int tsq_batch_run_async(tsq_batch *b) {
  return guarded([&]() -> int { return tsq::batch_run_async(b); });
}

int tsq_batch_sync(tsq_batch *b) {
  return guarded([&]() -> int { return tsq::batch_sync(b); });
}

int tsq_batch_results(tsq_batch *b, tsq_result *out) {
  return guarded([&]() -> int { return tsq::batch_results(b, out); });
}

int tsq_batch_get_stats(const tsq_batch *b, tsq_batch_stats *st) {
  if (!b || !st) return TSQ_E_INVALID_ARG;
  *st = b->stats;
  return TSQ_OK;
}

int tsq_batch_stream(const tsq_batch *b, void **stream) {
  if (!b || !stream) return TSQ_E_INVALID_ARG;
  *stream = static_cast<void *>(b->stream);
  return TSQ_OK;
}

void tsq_batch_destroy(tsq_batch *b) {
  if (!b) return;
  cudaSetDevice(b->device);
  delete b;
}

}  // extern "C"
