// tune.cpp -- the length-bucket autotuner.
//
// For each output kind (score, identity, alignment) and each length bucket
// (by the longer sequence of a pair), tsq_tune_run times the candidates on
// seeded synthetic protein pairs that fill the GPU and keeps the fastest in
// cells per second:
//   - the lane width G (4, 8, 16 or 32 lanes per pair);
//   - for score output, the lane type: int16x2 (proven or overflow-checked
//     with the exact int32 re-run) against int32;
//   - for buckets of 1,024 residues and more, the CTA fill (one pair per
//     8-warp CTA, the pair's bands striped over the warps) against one pair
//     per warp group.
// The table is written as JSON and read back by tsq_tune_load; batches
// created with opts.autotune consult it.  Few-pair batches still get at
// least enough lanes per pair to keep every SM busy (the planner takes the
// larger of the tuned and the occupancy G), and a pair too long for any
// warp group keeps the CTA fill whatever the table says.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "engine.h"

namespace tsq {
namespace {

struct Entry {
  int out, lo, hi;
  Shape sh;  // G, R, and i16 (1: int16x2 lanes where their range allows, 0: int32)
  int cta;   // 1: int32 pairs of the bucket take the CTA fill
  double gcups;
};

std::mutex g_mu;
std::vector<Entry> g_table;
bool g_loaded = false;

// Half-octave length buckets.
constexpr int kEdges[] = {0, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096, 6144, 8192, 1 << 21};
constexpr int kNumBuckets = int(sizeof(kEdges) / sizeof(kEdges[0])) - 1;
constexpr int kWidths[] = {4, 8, 16, 32};
constexpr int kCtaFrom = 1024;  // buckets from this length also try the CTA fill
const char *kOutNames[] = {"score", "identity", "alignment"};

int find_int(const std::string &obj, const char *key, int *v) {
  const std::string k = std::string("\"") + key + "\"";
  const size_t p = obj.find(k);
  if (p == std::string::npos) return -1;
  size_t q = obj.find(':', p + k.size());
  if (q == std::string::npos) return -1;
  *v = std::atoi(obj.c_str() + q + 1);
  return 0;
}

int find_str(const std::string &obj, const char *key, std::string *v) {
  const std::string k = std::string("\"") + key + "\"";
  const size_t p = obj.find(k);
  if (p == std::string::npos) return -1;
  size_t q = obj.find('"', obj.find(':', p + k.size()) + 1);
  if (q == std::string::npos) return -1;
  size_t r = obj.find('"', q + 1);
  if (r == std::string::npos) return -1;
  *v = obj.substr(q + 1, r - q - 1);
  return 0;
}

}  // namespace

bool tune_table_loaded() {
  std::lock_guard<std::mutex> g(g_mu);
  return g_loaded;
}

bool tune_table_pick(int out_mode, int m, int n, TunedChoice *c) {
  std::lock_guard<std::mutex> g(g_mu);
  const int L = std::max(m, n);
  for (const Entry &e : g_table)
    if (e.out == out_mode && L >= e.lo && L < e.hi) {
      c->sh = e.sh;
      c->cta = e.cta;
      return true;
    }
  return false;
}

}  // namespace tsq

extern "C" int tsq_tune_load(const char *json_path) {
  if (!json_path) return TSQ_E_INVALID_ARG;
  FILE *f = std::fopen(json_path, "rb");
  if (!f) return TSQ_E_INVALID_ARG;
  std::string text;
  char buf[4096];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
  std::fclose(f);
  std::vector<tsq::Entry> table;
  const size_t list = text.find("\"entries\"");
  if (list == std::string::npos) return TSQ_E_INVALID_ARG;
  size_t pos = text.find('[', list);
  while (pos != std::string::npos) {
    const size_t a = text.find('{', pos);
    if (a == std::string::npos) break;
    const size_t b = text.find('}', a);
    if (b == std::string::npos) return TSQ_E_INVALID_ARG;
    const std::string obj = text.substr(a, b - a + 1);
    tsq::Entry e{};
    std::string out;
    if (tsq::find_str(obj, "out", &out) || tsq::find_int(obj, "lo", &e.lo) || tsq::find_int(obj, "hi", &e.hi) ||
        tsq::find_int(obj, "G", &e.sh.G) || tsq::find_int(obj, "R", &e.sh.R) || tsq::find_int(obj, "i16", &e.sh.i16))
      return TSQ_E_INVALID_ARG;
    if (tsq::find_int(obj, "cta", &e.cta)) e.cta = 0;  // tables written before the CTA choice
    e.out = -1;
    for (int k = 0; k < 3; ++k)
      if (out == tsq::kOutNames[k]) e.out = k;
    if (e.out < 0 || e.lo < 0 || e.hi <= e.lo || (e.cta != 0 && e.cta != 1) || (e.sh.i16 != 0 && e.sh.i16 != 1))
      return TSQ_E_INVALID_ARG;
    if (!tsq::shape_supported(e.sh, e.out, false)) return TSQ_E_INVALID_ARG;
    table.push_back(e);
    pos = b + 1;
  }
  std::lock_guard<std::mutex> g(tsq::g_mu);
  tsq::g_table = table;
  tsq::g_loaded = !table.empty();
  return TSQ_OK;
}

extern "C" int tsq_tune_run(const char *json_path, int32_t quick) {
  using namespace tsq;
  if (!json_path) return TSQ_E_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TSQ_E_CUDA;
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return TSQ_E_CUDA;
  std::mt19937_64 rng(20261203);
  const char *aa = "ARNDCQEGHILKMFPSTWYV";
  std::vector<Entry> table;
  const int outs[] = {kOutScore, kOutIdent, kOutTrace};
  for (int out : outs) {
    for (int bk = 0; bk < kNumBuckets; ++bk) {
      const int lo = std::max(kEdges[bk], 16);
      const int hi = std::min(kEdges[bk + 1], quick ? 2048 : 8192);
      if (lo >= hi) continue;
      if (out == kOutIdent && hi > 32768) continue;
      // Enough pairs for eight rounds of 4-lane groups filling every SM
      // about 24 warps deep (the planner's occupancy target), so that a
      // candidate wins by its throughput in a large batch, not by a shorter
      // tail; at most about 5e10 cells per run (2e11 when not quick), and
      // for alignment output at most about 20 GB of traceback planes.
      const double mid = 0.5 * (lo + hi);
      const int64_t fill_pairs = int64_t(prop.multiProcessorCount) * 24 * 32 / 4;
      int64_t np = std::min<int64_t>(8 * fill_pairs, std::max<int64_t>(64, int64_t((quick ? 5e10 : 2e11) / (mid * mid))));
      if (out == kOutTrace) np = std::min<int64_t>(np, std::max<int64_t>(64, int64_t(4e10 / (mid * mid))));
      std::vector<uint8_t> seqs;
      std::vector<tsq_pair_desc> pairs(static_cast<size_t>(np));
      std::uniform_int_distribution<int> len(lo, hi - 1), let(0, 19);
      for (int64_t k = 0; k < np; ++k) {
        const int m = len(rng), n = len(rng);
        pairs[size_t(k)] = tsq_pair_desc{int64_t(seqs.size()), int64_t(seqs.size()) + m, m, n};
        for (int q = 0; q < m + n; ++q) seqs.push_back(uint8_t(aa[let(rng)]));
      }
      tsq_params p{};
      p.matrix = TSQ_MATRIX_BLOSUM62;
      p.gap_open = 11;
      p.gap_extend = 1;
      p.mode = TSQ_GLOBAL;
      p.output = out == kOutScore ? TSQ_OUT_SCORE : (out == kOutIdent ? TSQ_OUT_IDENTITY : TSQ_OUT_ALIGNMENT);
      // Candidates: (lane width, lane type, CTA fill).  Each is timed as the
      // fill time of one planned run (device events), the best of several.
      // The first candidate is the planner's own choice (nothing forced);
      // a forced candidate replaces it only when it is at least 3 % faster,
      // so a table never moves a batch off the default for noise.
      struct Cand {
        int G, i16, cta;
        bool free;
      };
      std::vector<Cand> cands;
      cands.push_back(Cand{4, 1, 0, true});
      for (int G : kWidths) {
        cands.push_back(Cand{G, 0, 0, false});
        cands.push_back(Cand{G, 1, 0, false});
      }
      if (kEdges[bk] >= kCtaFrom) cands.push_back(Cand{32, 0, 1, false});
      Entry best{out, kEdges[bk], kEdges[bk + 1], Shape{32, 8, 0}, 0, 0.0};
      for (const Cand &cand : cands) {
        tsq_batch b;
        tsq_batch_opts o{};
        o.device = dev;
        p.lane = cand.i16 ? TSQ_LANE_AUTO : TSQ_LANE_I32;
        b.tune_force.shape = !cand.free;
        b.tune_force.sh = Shape{cand.G, 8, 0};
        b.tune_force.cta = cand.cta != 0;
        int rc = batch_plan(&b, seqs.data(), int64_t(seqs.size()), pairs.data(), np, &p, &o, false);
        if (rc) return rc;
        double best_ms = 1e30;
        for (int it = 0; it < (quick ? 2 : 4); ++it) {
          if ((rc = batch_run_async(&b)) || (rc = batch_sync(&b))) return rc;
          // Alignment output: the whole run, since the walker's speed
          // depends on the plane layout the lane width sets.
          if (it > 0) best_ms = std::min(best_ms, out == kOutTrace ? b.stats.device_ms : b.stats.fill_ms);
        }
        const double gcups = double(b.cells) / (best_ms * 1e-3) / 1e9;
        if (cand.free) {
          best.gcups = gcups;  // the baseline, kept unless beaten by 3 %
          best.sh = Shape{cand.G, 8, cand.i16};
          best.cta = 0;
        } else if (gcups > 1.03 * best.gcups) {
          best.gcups = gcups;
          best.sh = Shape{cand.G, 8, cand.i16};
          best.cta = cand.cta;
        }
      }
      table.push_back(best);
    }
  }
  FILE *f = std::fopen(json_path, "wb");
  if (!f) return TSQ_E_INVALID_ARG;
  std::fprintf(f, "{\n \"device\": \"%s\",\n \"sm\": \"%d.%d\",\n \"entries\": [\n", prop.name, prop.major,
               prop.minor);
  for (size_t k = 0; k < table.size(); ++k) {
    const Entry &e = table[k];
    std::fprintf(f,
                 "  {\"out\": \"%s\", \"lo\": %d, \"hi\": %d, \"G\": %d, \"R\": %d, \"i16\": %d, \"cta\": %d, "
                 "\"gcups\": %.1f}%s\n",
                 kOutNames[e.out], e.lo, e.hi, e.sh.G, e.sh.R, e.sh.i16, e.cta, e.gcups, k + 1 < table.size() ? "," : "");
  }
  std::fprintf(f, " ]\n}\n");
  std::fclose(f);
  std::lock_guard<std::mutex> g(g_mu);
  g_table = table;
  g_loaded = true;
  return TSQ_OK;
}
