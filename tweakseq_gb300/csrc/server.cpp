// server.cpp -- continuous-batching alignment server on one GPU.
//
// Requests of any size (one pair from an editor realignment up to an
// all-vs-all distance batch) are submitted from any host thread and return
// at once with an id.  A scheduler thread turns waiting requests into
// *ticks*: consecutive waiting requests with the same scoring parameters,
// up to a cell budget per tick, admitted only while the device memory they
// need (residues, codes, pair table, results, band-boundary rows and, for
// alignments, traceback planes and gapped rows) fits what is left of the
// server's HBM budget.  Each tick is planned and launched on one of several
// stream slots, so ticks that are admitted while others still run overlap on
// the device; requests that arrive meanwhile join the next tick as soon as a
// slot and memory free up.  The scheduler only polls CUDA events from the
// host -- no kernel waits on anything -- and a finished tick's results go
// back to their requests, whose latency (submit to completion) feeds the
// p50/p99 statistics.
//
// Each request's results are exactly what tsq_align_batch returns for that
// request alone: the kernels compute every pair independently, so neither
// the other requests of a tick nor the lane width a pair gets change a
// score, a coordinate or a string.
#include <algorithm>
#include <cstdint>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "engine.h"
#include "resident.h"
#include "trace.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id = 0;
  tsq_params params{};
  int8_t custom_score[26 * 26];
  uint8_t custom_valid[26];
  std::vector<uint8_t> seqs;
  std::vector<tsq_pair_desc> pairs;
  int64_t cells = 0;
  int64_t bytes = 0;      // device bytes without the boundary rows
  int32_t max_n = 0;
  Clock::time_point t_submit, t_done;
  enum State { kPending, kRunning, kDone, kCancelled } state = kPending;
  int32_t status = TSQ_OK;
  std::vector<tsq_result> results;
  // Served by the device-resident loop: its slot and arena range, and
  // whether its results are still in the arena.
  bool resident = false;
  int32_t rslot = -1;
  tsq::resident::Range rrange;
  bool on_device = false;
};

struct Slot {
  std::unique_ptr<tsq_batch> batch;
  std::vector<std::shared_ptr<Request>> reqs;
  std::vector<int64_t> first;  // first pair of each request in the tick
  int64_t bytes = 0;           // reserved against the budget
  bool busy = false;
  // The tick's residues: page-locked, so that their upload is a direct
  // copy (a pageable vector when page-locked memory cannot be had).
  std::unique_ptr<tsq::PinBuf> seqpin;
  std::vector<uint8_t> seqbuf;
  std::vector<tsq_pair_desc> pairbuf;
};

bool same_params(const Request &a, const Request &b) {
  const tsq_params &x = a.params, &y = b.params;
  if (x.matrix != y.matrix || x.gap_open != y.gap_open || x.gap_extend != y.gap_extend || x.mode != y.mode ||
      x.output != y.output || x.lane != y.lane)
    return false;
  if (x.matrix == TSQ_MATRIX_CUSTOM)
    return std::memcmp(a.custom_score, b.custom_score, sizeof(a.custom_score)) == 0 &&
           std::memcmp(a.custom_valid, b.custom_valid, sizeof(a.custom_valid)) == 0;
  return true;
}

double percentile(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * double(v.size() - 1);
  const size_t lo = size_t(pos);
  const size_t hi = std::min(v.size() - 1, lo + 1);
  return v[lo] + (v[hi] - v[lo]) * (pos - double(lo));
}

}  // namespace

struct tsq_server {
  tsq_server_opts opts{};
  int device = 0;
  int resident_warps = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Request>> pending;
  std::map<uint64_t, std::shared_ptr<Request>> requests;
  std::vector<Slot> slots;
  uint64_t next_id = 1;
  int64_t reserved = 0;  // bytes of the ticks in flight
  bool stop = false;
  std::thread worker;
  // statistics
  int64_t submitted = 0, completed = 0, rejected = 0, cancelled = 0, ticks = 0, cells_done = 0;
  int64_t peak_reserved = 0, admission_waits = 0;
  std::vector<double> latencies_ms;
  Clock::time_point t_first_submit, t_last_done;
  bool any_submit = false;
  // The device-resident request loop (opts.resident).
  std::unique_ptr<tsq::resident::Loop> loop;
  std::deque<std::shared_ptr<Request>> rpending;     // waiting for arena room
  std::vector<std::shared_ptr<Request>> rrunning;    // published, not done
  int64_t resident_requests = 0;
  int64_t r_outstanding_pairs = 0;
  int tend_resident();                               // called with the lock held

  // Boundary rows a tick of npairs pairs needs for sequences up to max_n
  // columns: 8 group rows per warp of the launch (no more warps than pairs,
  // no more than fit on the device), at the largest entry size (16 bytes).
  int64_t boundary_bytes(int32_t max_n, int64_t npairs) const {
    const int64_t warps = std::min<int64_t>(resident_warps, npairs + 8);
    return warps * 8 * (int64_t(max_n) + 64) * 16;
  }

  void run();
  int launch(Slot &s, std::vector<std::shared_ptr<Request>> &&reqs, int64_t bytes);
  void finish(Slot &s, int rc);
};

// Plans and enqueues one tick (called without the lock; only the scheduler
// thread touches slots).  Returns the status of the launch.
int tsq_server::launch(Slot &s, std::vector<std::shared_ptr<Request>> &&reqs, int64_t bytes) {
  tsq::TraceRange tr("server tick launch");
  s.reqs = std::move(reqs);
  // The tick's residues and pair table: each request's at its offsets,
  // copied on the host worker pool (a tick can hold tens of megabytes).
  const size_t nr = s.reqs.size();
  std::vector<int64_t> seq_at(nr + 1, 0);
  s.first.assign(nr + 1, 0);
  for (size_t q = 0; q < nr; ++q) {
    seq_at[q + 1] = seq_at[q] + int64_t(s.reqs[q]->seqs.size());
    s.first[q + 1] = s.first[q] + int64_t(s.reqs[q]->pairs.size());
  }
  const int64_t seq_len = seq_at[nr];
  uint8_t *seqs = nullptr;
  if (!s.seqpin) s.seqpin.reset(new tsq::PinBuf());
  if (s.seqpin->ensure(size_t(seq_len)) == cudaSuccess) {
    seqs = s.seqpin->as<uint8_t>();
  } else {
    cudaGetLastError();
    s.seqbuf.resize(size_t(seq_len));
    seqs = s.seqbuf.data();
  }
  s.pairbuf.resize(size_t(s.first[nr]));
  tsq::run_tasks(int(nr), [&](int q) {
    const Request &r = *s.reqs[size_t(q)];
    const int64_t base = seq_at[size_t(q)];
    if (!r.seqs.empty()) std::memcpy(seqs + base, r.seqs.data(), r.seqs.size());
    tsq_pair_desc *dst = s.pairbuf.data() + s.first[size_t(q)];
    for (size_t k = 0; k < r.pairs.size(); ++k) {
      tsq_pair_desc d = r.pairs[k];
      d.a_off += base;
      d.b_off += base;
      dst[k] = d;
    }
  });
  s.first.pop_back();
  if (!s.batch) {
    s.batch.reset(new tsq_batch());
    s.batch->async_max = SIZE_MAX;  // growth never waits for the other slots
  }
  tsq_params p = s.reqs.front()->params;
  if (p.matrix == TSQ_MATRIX_CUSTOM) {
    p.custom_score = s.reqs.front()->custom_score;
    p.custom_valid = s.reqs.front()->custom_valid;
  }
  tsq_batch_opts o{};
  o.device = device;
  o.use_graph = 0;  // every tick is a different plan
  o.autotune = opts.autotune;
  int rc = tsq::batch_plan(s.batch.get(), seqs, seq_len, s.pairbuf.data(),
                           int64_t(s.pairbuf.size()), &p, &o, false);
  if (!rc) rc = tsq::batch_run_async(s.batch.get());
  if (!rc) rc = tsq::batch_fetch_async(s.batch.get());
  s.bytes = std::max(bytes, tsq::batch_device_bytes(s.batch.get()));
  return rc;
}

// Called with the lock held.
void tsq_server::finish(Slot &s, int rc) {
  const auto now = Clock::now();
  // Each request's results (and strings) are copied out of the tick's
  // result blocks on the host worker pool.
  tsq::run_tasks(int(s.reqs.size()), [&](int q) {
    Request &r = *s.reqs[size_t(q)];
    r.results.assign(r.pairs.size(), tsq_result{});
    r.status = rc ? rc : tsq::batch_collect(s.batch.get(), s.first[size_t(q)], int64_t(r.pairs.size()), r.results.data());
  });
  for (size_t q = 0; q < s.reqs.size(); ++q) {
    Request &r = *s.reqs[q];
    r.state = Request::kDone;
    r.t_done = now;
    ++completed;
    cells_done += r.cells;
    latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r.t_submit).count());
  }
  t_last_done = now;
  reserved -= s.bytes;
  s.reqs.clear();
  s.busy = false;
  // Keep the slot's cached buffers only while they fit its share of the
  // budget, so idle slots do not hold HBM the budget gave to others.
  if (s.batch && tsq::batch_device_bytes(s.batch.get()) > opts.hbm_budget_bytes / int64_t(slots.size()))
    s.batch.reset();
  cv_done.notify_all();
}

// The resident loop's side of the scheduler (lock held): finished
// requests, admission and publication of waiting ones, and a relaunch of
// the loop's kernel when it has ended with work outstanding.  Returns
// whether resident requests are in flight.
int tsq_server::tend_resident() {
  if (!loop) return 0;
  const auto now = Clock::now();
  for (size_t k = 0; k < rrunning.size();) {
    Request &r = *rrunning[k];
    const int64_t n = int64_t(r.pairs.size());
    if (!loop->done(r.rslot, n)) {
      ++k;
      continue;
    }
    loop->retired(n);
    r_outstanding_pairs -= n;
    r.state = Request::kDone;
    r.on_device = true;
    r.t_done = now;
    ++completed;
    cells_done += r.cells;
    latencies_ms.push_back(std::chrono::duration<double, std::milli>(now - r.t_submit).count());
    t_last_done = now;
    rrunning.erase(rrunning.begin() + int64_t(k));
    cv_done.notify_all();
  }
  while (!rpending.empty() && !stop) {
    const std::shared_ptr<Request> r = rpending.front();
    const int64_t n = int64_t(r->pairs.size());
    if (r_outstanding_pairs + n > tsq::resident::kRingCap) break;
    int32_t slot = -1;
    tsq::resident::Range range;
    const int rc = loop->admit(int64_t(r->seqs.size()), n, &slot, &range);
    if (rc == TSQ_E_PENDING) {
      ++admission_waits;
      break;
    }
    rpending.pop_front();
    if (rc) {
      r->status = rc;
      r->state = Request::kDone;
      ++completed;
      cv_done.notify_all();
      continue;
    }
    r->rslot = slot;
    r->rrange = range;
    r->state = Request::kRunning;
    const int prc = loop->publish(slot, range, r->seqs, r->pairs, r->params, r->custom_score, r->custom_valid);
    if (prc) {
      loop->release(slot, range);
      r->status = prc;
      r->state = Request::kDone;
      ++completed;
      cv_done.notify_all();
      continue;
    }
    r_outstanding_pairs += n;
    rrunning.push_back(r);
  }
  loop->tend();
  return rrunning.empty() ? 0 : 1;
}

void tsq_server::run() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lock(mu);
  for (;;) {
    const int resident_busy = tend_resident();
    // Completed ticks.
    for (Slot &s : slots)
      if (s.busy) {
        const int q = tsq::batch_fetch_query(s.batch.get());
        if (q != TSQ_E_PENDING) finish(s, q);
      }
    if (stop) {
      bool busy = resident_busy != 0;
      for (Slot &s : slots) busy |= s.busy;
      if (!busy) break;
    }
    // Admission: the oldest waiting request heads the next tick; later
    // requests with the same parameters join while the tick stays under
    // its cell budget and the memory left in the budget.
    Slot *free_slot = nullptr;
    for (Slot &s : slots)
      if (!s.busy) {
        free_slot = &s;
        break;
      }
    bool launched = false;
    if (free_slot && !pending.empty() && !stop) {
      const std::shared_ptr<Request> head = pending.front();
      const int64_t room = opts.hbm_budget_bytes - reserved;
      std::vector<std::shared_ptr<Request>> take;
      int64_t bytes = 0, cells = 0, npairs = 0;
      int32_t max_n = 0;
      for (auto it = pending.begin(); it != pending.end();) {
        const auto &r = *it;
        if (!same_params(*r, *head)) {
          ++it;
          continue;
        }
        const int32_t mn = std::max(max_n, r->max_n);
        const int64_t np = npairs + int64_t(r->pairs.size());
        const int64_t need = bytes + r->bytes + boundary_bytes(mn, np);
        const bool first = take.empty();
        if (need > room || (!first && cells + r->cells > opts.max_tick_cells)) {
          if (first) ++admission_waits;
          break;  // the head (or the tick) waits for memory
        }
        take.push_back(r);
        bytes += r->bytes;
        cells += r->cells;
        npairs = np;
        max_n = mn;
        r->state = Request::kRunning;
        it = pending.erase(it);
      }
      if (!take.empty()) {
        const int64_t tick_bytes = bytes + boundary_bytes(max_n, npairs);
        reserved += tick_bytes;
        peak_reserved = std::max(peak_reserved, reserved);
        ++ticks;
        Slot &s = *free_slot;
        s.busy = true;
        s.bytes = tick_bytes;
        lock.unlock();
        const int rc = launch(s, std::move(take), tick_bytes);
        lock.lock();
        // The slot may have grown past the estimate; account what it holds.
        reserved += s.bytes - tick_bytes;
        peak_reserved = std::max(peak_reserved, reserved);
        if (rc) finish(s, rc);
        launched = true;
      }
    }
    if (!launched) {
      bool busy = resident_busy != 0 || !rpending.empty();
      for (Slot &s : slots) busy |= s.busy;
      // Poll in-flight work often (resident requests most often: their
      // completion is one read of mapped memory); sleep longer when idle.
      cv_work.wait_for(lock, resident_busy ? std::chrono::microseconds(10)
                                           : (busy ? std::chrono::microseconds(50) : std::chrono::milliseconds(2)));
    }
  }
}

extern "C" {

int tsq_server_create(const tsq_server_opts *opts, tsq_server **out) {
  if (!out) return TSQ_E_INVALID_ARG;
  *out = nullptr;
  try {
    std::unique_ptr<tsq_server> s(new tsq_server());
    if (opts) s->opts = *opts;
    int dev = s->opts.device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return TSQ_E_CUDA;
    if (cudaSetDevice(dev) != cudaSuccess) return TSQ_E_CUDA;
    s->device = dev;
    if (s->opts.slots <= 0) s->opts.slots = 4;
    if (s->opts.slots > 64) return TSQ_E_INVALID_ARG;
    if (s->opts.max_tick_cells <= 0) s->opts.max_tick_cells = int64_t(4e10);
    if (s->opts.hbm_budget_bytes <= 0) {
      size_t free_b = 0, total_b = 0;
      if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return TSQ_E_CUDA;
      s->opts.hbm_budget_bytes = int64_t(free_b / 2);
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return TSQ_E_CUDA;
    s->resident_warps = sms * 16;  // most warps any fill kernel keeps resident per SM
    if (s->opts.resident) {
      // The loop's arena comes out of the budget: a quarter of it, at most
      // 4 GiB.
      const int64_t arena = std::min<int64_t>(s->opts.hbm_budget_bytes / 4, int64_t(4) << 30);
      s->loop.reset(new tsq::resident::Loop());
      const int rc = s->loop->init(dev, arena, s->opts.resident_idle_polls);
      if (rc) return rc;
      s->opts.hbm_budget_bytes -= arena;
    }
    s->slots.resize(size_t(s->opts.slots));
    tsq_server *raw = s.get();
    s->worker = std::thread([raw]() { raw->run(); });
    *out = s.release();
    return TSQ_OK;
  } catch (...) {
    return TSQ_E_NOMEM;
  }
}

int tsq_server_submit(tsq_server *s, const uint8_t *seqs, int64_t seqs_len, const tsq_pair_desc *pairs, int64_t n,
                      const tsq_params *p, uint64_t *request_id) {
  if (!s || !p || !request_id || n < 0 || seqs_len < 0 || (n > 0 && !pairs) || (seqs_len > 0 && !seqs))
    return TSQ_E_INVALID_ARG;
  if (p->mode != TSQ_GLOBAL && p->mode != TSQ_LOCAL) return TSQ_E_INVALID_ARG;
  if (p->output < TSQ_OUT_SCORE || p->output > TSQ_OUT_ALIGNMENT) return TSQ_E_INVALID_ARG;
  if (p->lane < TSQ_LANE_AUTO || p->lane > TSQ_LANE_I32 || p->gap_open < 0 || p->gap_extend < 0)
    return TSQ_E_INVALID_ARG;
  if (p->matrix == TSQ_MATRIX_CUSTOM && (!p->custom_score || !p->custom_valid)) return TSQ_E_INVALID_ARG;
  try {
    auto r = std::make_shared<Request>();
    r->params = *p;
    r->params.custom_score = nullptr;
    r->params.custom_valid = nullptr;
    if (p->matrix == TSQ_MATRIX_CUSTOM) {
      std::memcpy(r->custom_score, p->custom_score, sizeof(r->custom_score));
      std::memcpy(r->custom_valid, p->custom_valid, sizeof(r->custom_valid));
    }
    r->seqs.assign(seqs, seqs + seqs_len);
    r->pairs.assign(pairs, pairs + n);
    int64_t bytes = 2 * seqs_len + 256 + n * 80;
    for (const tsq_pair_desc &d : r->pairs) {
      if (d.a_len < 0 || d.b_len < 0 || d.a_off < 0 || d.b_off < 0 || d.a_off > seqs_len - d.a_len ||
          d.b_off > seqs_len - d.b_len)
        return TSQ_E_INVALID_ARG;
      r->cells += int64_t(d.a_len) * d.b_len;
      r->max_n = std::max(r->max_n, d.b_len);
      if (p->output == TSQ_OUT_ALIGNMENT)
        bytes += tsq::plane_bytes(d.a_len, d.b_len, tsq::Shape{32, 8, 0}) + 2 * (int64_t(d.a_len) + d.b_len);
    }
    r->bytes = bytes;
    r->resident = s->loop && tsq::resident::Loop::eligible(r->params, r->pairs);
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return TSQ_E_CANCELLED;
    if (!r->resident && r->bytes + s->boundary_bytes(r->max_n, n) > s->opts.hbm_budget_bytes) {
      ++s->rejected;
      return TSQ_E_REJECTED;
    }
    r->id = s->next_id++;
    r->t_submit = Clock::now();
    if (!s->any_submit) {
      s->any_submit = true;
      s->t_first_submit = r->t_submit;
    }
    ++s->submitted;
    s->requests[r->id] = r;
    if (r->resident) {
      ++s->resident_requests;
      s->rpending.push_back(r);
    } else {
      s->pending.push_back(r);
    }
    *request_id = r->id;
    s->cv_work.notify_one();
    return TSQ_OK;
  } catch (...) {
    return TSQ_E_NOMEM;
  }
}

int tsq_server_poll(tsq_server *s, uint64_t id, int32_t wait_ms, tsq_result *out, int64_t n) {
  if (!s) return TSQ_E_INVALID_ARG;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->requests.find(id);
  if (it == s->requests.end()) return TSQ_E_NOT_FOUND;
  std::shared_ptr<Request> r = it->second;
  if (r->state != Request::kDone && r->state != Request::kCancelled && wait_ms != 0) {
    auto done = [&]() { return r->state == Request::kDone || r->state == Request::kCancelled; };
    if (wait_ms < 0)
      s->cv_done.wait(lock, done);
    else
      s->cv_done.wait_for(lock, std::chrono::milliseconds(wait_ms), done);
  }
  if (r->state == Request::kCancelled) {
    s->requests.erase(id);
    return TSQ_E_CANCELLED;
  }
  if (r->state != Request::kDone) return TSQ_E_PENDING;
  if (r->on_device) {
    // A resident request's results leave the device arena when polled.
    const int64_t np = int64_t(r->pairs.size());
    if (n != np || (n > 0 && !out)) return TSQ_E_INVALID_ARG;
    r->on_device = false;
    lock.unlock();
    const int st = s->loop->fetch(r->rrange, int64_t(r->seqs.size()), np, out);
    lock.lock();
    s->loop->release(r->rslot, r->rrange);
    s->requests.erase(id);
    s->cv_work.notify_one();  // arena room for waiting requests
    return st;
  }
  if (n != int64_t(r->results.size()) || (n > 0 && !out)) return TSQ_E_INVALID_ARG;
  // The strings move to the caller, who frees them with tsq_results_free.
  std::copy(r->results.begin(), r->results.end(), out);
  const int st = r->status;
  s->requests.erase(id);
  return st;
}

int tsq_server_cancel(tsq_server *s, uint64_t id) {
  if (!s) return TSQ_E_INVALID_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->requests.find(id);
  if (it == s->requests.end()) return TSQ_E_NOT_FOUND;
  Request &r = *it->second;
  if (r.state != Request::kPending) return TSQ_E_PENDING;  // already on the device (or done)
  for (auto *q : {&s->pending, &s->rpending})
    for (auto p = q->begin(); p != q->end(); ++p)
      if ((*p)->id == id) {
        q->erase(p);
        break;
      }
  r.state = Request::kCancelled;
  ++s->cancelled;
  s->cv_done.notify_all();
  return TSQ_OK;
}

int tsq_server_get_stats(tsq_server *s, tsq_server_stats *st) {
  if (!s || !st) return TSQ_E_INVALID_ARG;
  std::lock_guard<std::mutex> lock(s->mu);
  std::memset(st, 0, sizeof(*st));
  st->submitted = s->submitted;
  st->completed = s->completed;
  st->rejected = s->rejected;
  st->cancelled = s->cancelled;
  st->ticks = s->ticks;
  st->cells_completed = s->cells_done;
  st->peak_reserved_bytes = s->peak_reserved;
  st->admission_waits = s->admission_waits;
  st->p50_ms = percentile(s->latencies_ms, 0.50);
  st->p99_ms = percentile(s->latencies_ms, 0.99);
  st->max_ms = s->latencies_ms.empty() ? 0.0 : *std::max_element(s->latencies_ms.begin(), s->latencies_ms.end());
  if (s->any_submit && s->completed > 0)
    st->span_s = std::chrono::duration<double>(s->t_last_done - s->t_first_submit).count();
  st->resident_requests = s->resident_requests;
  if (s->loop) {
    st->resident_launches = s->loop->launches();
    st->resident_idle_exits = s->loop->idle_exits();
  }
  return TSQ_OK;
}

int tsq_server_destroy(tsq_server *s) {
  if (!s) return TSQ_E_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
    for (auto *q : {&s->pending, &s->rpending}) {
      for (auto &r : *q) {
        r->state = Request::kCancelled;
        ++s->cancelled;
      }
      q->clear();
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  for (auto &kv : s->requests) tsq_results_free(kv.second->results.data(), int64_t(kv.second->results.size()));
  cudaSetDevice(s->device);
  s->loop.reset();  // stops the loop's kernel, frees its arena
  delete s;
  return TSQ_OK;
}

}  // extern "C"
