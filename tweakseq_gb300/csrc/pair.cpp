// pair.cpp -- the plain form's one-pair path (tsq_align_pair).
//
// A lone pair needs none of the batch planner's passes (per-pair checks
// over worker threads, lane types, radix sorts, warp-task lists) nor its
// dozen separate uploads and three host synchronisations.  This path packs
// everything the kernels read -- the pair record, its task entries, the
// zeroed work counter, the code tables, the score matrices and the
// residues -- into one page-locked block and sends it with one copy; runs
// the encoder, the fill (one warp task, or the CTA fill for a long int32
// pair) and, for alignments, the walker; and brings the result record and
// the aligned rows back with one copy: one host synchronisation per call.
//
// Lane choice: the batch planner's, with one difference.  A pair whose
// int16x2 range is not proven (range16: lower bound only) runs in int32 at
// once (or, when long, on the int16x2 CTA fill), where the planner would
// run the overflow-checked int16x2 fill and re-run a flagged pair in int32
// -- a second round trip for one pair.
// Scores, coordinates and rows are the same in every lane type.  Calls
// that force the checked int16x2 lane (TSQ_LANE_I16) and pairs outside
// pair_limits go to the batch engine (kPairNotTaken), which owns those
// cases and their error codes.
//
// The entry point this serves is the plain aligner call of the editor's
// "Align selection" (tweakseq/UI/SeqEditMainWin.cpp:1616-1663), one pair
// at a time.
#include <algorithm>
#include <cstring>

#include "engine.h"
#include "trace.h"

namespace tsq {

namespace {

#define PAIR_TRY(expr)                                  \
  do {                                                  \
    const cudaError_t e_ = (expr);                      \
    if (e_ != cudaSuccess) return cuda_status(e_);      \
  } while (0)

constexpr int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

// The upload block (byte offsets).  The device keeps a copy of it at the
// start of PairPath::dev; the kernels read every table there.
constexpr size_t kOffPair = 0;        // PairDev: a at kOffSeqs, b right after it
constexpr size_t kOffTask = 32;       // int32 pair id 0
constexpr size_t kOffCounter = 36;    // int32 work-queue head, zero
constexpr size_t kOffWtask = 48;      // int2 warp task {0, (G << 16) | 1}
constexpr size_t kOffShapeG = 56;     // int32 G of the traceback planes
constexpr size_t kOffShapeR = 60;     // int32 R of the traceback planes
constexpr size_t kOffPlaneOff = 64;   // int64 0
constexpr size_t kOffAlnOff = 72;     // int64 0
constexpr size_t kOffLut = 128;       // letter codes by byte
constexpr size_t kOffClut = 384;      // score classes by byte
constexpr size_t kOffMatrix = 640;    // 26 x 26 scores
constexpr size_t kOffCmatrix = 1344;  // nclasses x nclasses class scores
constexpr size_t kOffSeqs = 2048;     // residues of a, then b, then kPad zero bytes
// The fills' staging reads up to 64 bytes past a sequence; the zero bytes
// there encode to class 0 (and an invalid letter code, which no check
// reads past a sequence's end).
constexpr int64_t kPad = 128;
static_assert(kOffCmatrix + kLetters * kLetters <= kOffSeqs, "tables overlap the residues");
static_assert(sizeof(PairDev) <= kOffTask && sizeof(ResultDev) == 32, "record sizes");

}  // namespace

void PairPath::reset() {
  if (stream) cudaStreamSynchronize(stream);
  dev.release();
  up.release();
  down.release();
  if (stream) cudaStreamDestroy(stream);
  stream = nullptr;
  device = -1;
}

int pair_align(PairPath *pp, const uint8_t *a, int32_t la, const uint8_t *b, int32_t lb, const tsq_params *p,
               tsq_result *out) {
  if (!pp || !p || !out) return kPairNotTaken;
  if (check_params(p) != TSQ_OK || p->lane == TSQ_LANE_I16) return kPairNotTaken;
  Scheme sc;
  if (build_scheme(p, &sc) != TSQ_OK) return kPairNotTaken;
  const int out_mode = out_mode_of(p);
  const bool local = p->mode == TSQ_LOCAL;
  if (pair_limits(p, sc, out_mode, la, lb) != TSQ_OK) return kPairNotTaken;
  TraceRange tr("align pair (one-pair path)");

  int devno = 0;
  PAIR_TRY(cudaGetDevice(&devno));
  if (pp->device != devno) {
    pp->reset();
    PAIR_TRY(cudaStreamCreateWithFlags(&pp->stream, cudaStreamNonBlocking));
    PAIR_TRY(cudaDeviceGetAttribute(&pp->sms, cudaDevAttrMultiProcessorCount, devno));
    pp->device = devno;
  }
  cudaStream_t st = pp->stream;
  // Whatever this call returns, its copies have landed before the next call
  // rewrites the page-locked blocks.
  struct SyncOnExit {
    cudaStream_t st;
    ~SyncOnExit() { cudaStreamSynchronize(st); }
  } sync_on_exit{st};

  // ---- lane type and shape: the planner's rules for a lone pair ----------
  // 0 int32 warp task, 1 int16x2 warp task, 3 CTA fill (int32), 4 CTA fill
  // (int16x2, rebased values).
  int lt = 0;
  if (lanes16_possible(out_mode, local, p->lane)) {
    const Range16 r16 = range16(p, sc, la, lb);
    if (r16.lower && r16.upper && p->lane == TSQ_LANE_AUTO) lt = 1;
  }
  const bool cta16 = p->lane == TSQ_LANE_AUTO && cta16_supported(out_mode, local, sc, p->gap_open, p->gap_extend);
  if (lt == 0 && la > 0 && lb > 0) {
    const double steps32 = double((la + 255) / 256) * double(lb + 31);
    if (steps32 > 20000.0) lt = cta16 ? 4 : 3;
  } else if (lt == 1 && cta16) {
    const double steps16 = double((la + 511) / 512) * double(lb + 63);
    if (steps16 > 20000.0) lt = 4;
  }
  ShapeChooser ch;
  ch.out_mode = out_mode;
  ch.local = local;
  ch.sms = pp->sms;
  ch.npairs = 1;
  ch.prepare();
  Shape shp = ch.pick(la, lb, lt == 1 ? 2 * kFillRows : kFillRows);
  if (lt >= 3) shp = Shape{32, kFillRows, 0};
  if (!shape_supported(shp, out_mode, local)) return kPairNotTaken;
  const int i16 = lt == 1 || lt == 4 ? 1 : 0;  // class codes and class matrix in use

  // Resident blocks of the kernel: the query also opts it into its shared
  // memory (answered from a cache after the first call).
  const int blocks_avail = lt == 4   ? cta16_blocks(out_mode, local, sc.nclasses)
                           : lt == 3 ? cta_blocks(out_mode, local)
                                     : fill_blocks(kFillRows, i16, out_mode, local, i16 ? sc.nclasses : kLetters);
  if (blocks_avail <= 0) return TSQ_E_CUDA;

  // ---- device layout ---------------------------------------------------
  const int64_t len = int64_t(la) + lb;
  const int64_t up_bytes = int64_t(kOffSeqs) + len + kPad;
  const int64_t off_codes = align256(up_bytes);
  const int64_t off_ccodes = off_codes + align256(len + kPad);
  const int64_t off_res = off_ccodes + (i16 ? align256(len + kPad) : 0);
  const bool trace = out_mode == kOutTrace;
  const int64_t down_bytes = int64_t(sizeof(ResultDev)) + (trace ? 2 * len : 0);  // record, then a and b rows
  const int64_t off_bnd = off_res + align256(down_bytes);
  const int32_t bnd_cols = ((std::max(lb, 1) + 31) / 32 + 1) * 32;
  const int64_t bnd_bytes =
      lt >= 3 ? int64_t(bnd_cols) * int64_t(cta_bnd_entry_bytes(out_mode))
              : int64_t(fill_threads_for(i16) / 32) * 8 * bnd_cols * int64_t(fill_bnd_entry_bytes(i16, out_mode));
  const int64_t off_planes = off_bnd + align256(bnd_bytes);
  const int64_t plane_total = trace ? plane_bytes(la, lb, Shape{shp.G, shp.R, 0}) : 0;
  const int64_t dev_bytes = off_planes + std::max<int64_t>(plane_total, 16);

  auto grow = [](size_t need, size_t cap) { return need <= cap ? need : need + need / 2; };
  // (A pair whose traceback planes do not fit in device memory fails here
  // with TSQ_E_NOMEM, as it does on the batch engine's one-pair plan.)
  PAIR_TRY(pp->dev.ensure(grow(size_t(dev_bytes), pp->dev.cap), st));
  PAIR_TRY(pp->up.ensure(grow(size_t(up_bytes), pp->up.cap)));
  PAIR_TRY(pp->down.ensure(grow(size_t(down_bytes), pp->down.cap)));

  // ---- the upload block --------------------------------------------------
  uint8_t *h = pp->up.as<uint8_t>();
  std::memset(h, 0, kOffSeqs);
  const PairDev pd{0, la, la, lb};  // offsets into the residues
  std::memcpy(h + kOffPair, &pd, sizeof(pd));
  const int2 wt = make_int2(0, (shp.G << 16) | 1);
  std::memcpy(h + kOffWtask, &wt, sizeof(wt));
  std::memcpy(h + kOffShapeG, &shp.G, sizeof(int32_t));
  std::memcpy(h + kOffShapeR, &shp.R, sizeof(int32_t));
  build_lut(sc, h + kOffLut);
  if (i16) {
    build_class_lut(sc, h + kOffClut);
    std::memcpy(h + kOffCmatrix, sc.cscore, size_t(sc.nclasses) * size_t(sc.nclasses));
  }
  std::memcpy(h + kOffMatrix, sc.score, size_t(kLetters) * kLetters);
  if (la) std::memcpy(h + kOffSeqs, a, size_t(la));
  if (lb) std::memcpy(h + kOffSeqs + la, b, size_t(lb));
  std::memset(h + kOffSeqs + len, 0, size_t(kPad));

  uint8_t *d = pp->dev.as<uint8_t>();
  const uint8_t *seqs = d + kOffSeqs;
  uint8_t *codes = d + off_codes;
  uint8_t *ccodes = i16 ? d + off_ccodes : nullptr;
  ResultDev *res = reinterpret_cast<ResultDev *>(d + off_res);
  PAIR_TRY(cudaMemcpyAsync(d, h, size_t(up_bytes), cudaMemcpyHostToDevice, st));
  PAIR_TRY(launch_encode(seqs, len + kPad, d + kOffLut, codes, i16 ? d + kOffClut : nullptr, ccodes, st));

  // ---- fill ----------------------------------------------------------------
  FillArgs fa{};
  fa.codes = codes;
  fa.pairs = reinterpret_cast<const PairDev *>(d + kOffPair);
  fa.tasks = reinterpret_cast<const int32_t *>(d + kOffTask);
  fa.wtasks = reinterpret_cast<const int2 *>(d + kOffWtask);
  fa.n_wtasks = 1;
  fa.counter = reinterpret_cast<int32_t *>(d + kOffCounter);
  fa.matrix = reinterpret_cast<const int8_t *>(d + kOffMatrix);
  fa.gap_open = p->gap_open;
  fa.gap_extend = p->gap_extend;
  fa.res = res;
  fa.bnd = reinterpret_cast<int32_t *>(d + off_bnd);
  fa.bnd_cols = bnd_cols;
  fa.planes = d + off_planes;
  fa.plane_off = reinterpret_cast<const int64_t *>(d + kOffPlaneOff);
  fa.max_score = sc.max_score;
  if (i16) {
    fa.ccodes = ccodes;
    fa.cmatrix = reinterpret_cast<const int8_t *>(d + kOffCmatrix);
    fa.nclasses = sc.nclasses;
  }
  if (lt == 4) {
    PAIR_TRY(launch_cta16(out_mode, local, fa, 1, st));
  } else if (lt == 3) {
    PAIR_TRY(launch_cta(out_mode, local, fa, 1, st));
  } else {
    PAIR_TRY(launch_fill(kFillRows, i16, out_mode, local, fa, 1, st));
  }

  // ---- traceback ---------------------------------------------------------
  char *rows = reinterpret_cast<char *>(d + off_res + sizeof(ResultDev));
  if (trace) {
    WalkArgs w{};
    w.seqs = seqs;
    w.codes = codes;
    w.pairs = fa.pairs;
    w.tasks = fa.tasks;
    w.n_tasks = 1;
    w.planes = fa.planes;
    w.plane_off = fa.plane_off;
    w.shape_G = reinterpret_cast<const int32_t *>(d + kOffShapeG);
    w.shape_R = reinterpret_cast<const int32_t *>(d + kOffShapeR);
    w.local = local ? 1 : 0;
    w.res = res;
    w.aln = rows;
    w.aln_off = reinterpret_cast<const int64_t *>(d + kOffAlnOff);
    PAIR_TRY(launch_walk(w, st));
  }
  PAIR_TRY(cudaMemcpyAsync(pp->down.p, res, size_t(down_bytes), cudaMemcpyDeviceToHost, st));
  PAIR_TRY(cudaStreamSynchronize(st));

  const ResultDev rd = *pp->down.as<ResultDev>();
  const char *hrows = pp->down.as<char>() + sizeof(ResultDev);
  const int e = collect_one(rd, trace && rd.status == TSQ_OK ? hrows : nullptr, len, *out);
  if (e) return e;
  return rd.status;
}

}  // namespace tsq
