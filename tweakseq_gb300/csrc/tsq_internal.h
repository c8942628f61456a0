// tsq_internal.h -- shared declarations of the GB300 alignment library.
//
// Device data layout (all in HBM, one allocation pool per context):
//   codes      uint8 per residue: 'A'..'Z' -> 0..25 when the scheme accepts
//              the letter, kBadCode otherwise (converted once per batch).
//   ccodes     score batches: uint8 score class per residue, 0 for bytes
//              the scheme rejects (their codes entry marks them), and 128
//              bytes of class 0 past the residues: every entry indexes the
//              int16x2 fill's profile.
//   pairs      PairDev per pair (offsets into codes, lengths).
//   tasks      int32 pair ids of one launch, sorted so that the groups of a
//              warp get pairs of nearly the same shape.
//   results    ResultDev per pair.
//   boundary   per group slot, two rows of (H, F) of max_n + 1 columns: the
//              bottom row of one band of rows is the top row of the next.
//   planes     traceback nibbles (TB mode), diagonal-major per band so the
//              lanes of a group store one contiguous run per step.
#pragma once

#include <cstdint>
#include <cstddef>

#include <cuda_runtime.h>

#include "../../include/tweakseq_gb300.h"

namespace tsq {

constexpr uint8_t kBadCode = 0xFF;
constexpr int kLetters = 26;
constexpr int32_t kNegInf = -(1 << 29);  // "minus infinity" for int32 E/F

// Output modes of the fill kernels.
enum : int { kOutScore = 0, kOutIdent = 1, kOutTrace = 2 };
// Traceback nibble: bits 0-1 H source, bit 2 E opened, bit 3 F opened.
enum : int { kDirDiag = 0, kDirE = 1, kDirF = 2, kDirStop = 3 };

struct Scheme {
  int8_t score[kLetters][kLetters];
  uint8_t valid[kLetters];
  int32_t max_score, min_score;
  bool symmetric;
  // Score classes: valid letters with the same row and column of scores
  // (BLOSUM62: J, O, U and X) share a class; the int16x2 fills index their
  // profile by class, which keeps the profile small.  For identity output
  // every valid letter is its own class (identical = same class).
  int32_t nclasses;
  uint8_t cls[kLetters];               // class of each letter, kBadCode if invalid
  int8_t cscore[kLetters * kLetters];  // nclasses x nclasses class scores
};

struct PairDev {
  int64_t a_off, b_off;
  int32_t a_len, b_len;
};

struct ResultDev {
  int32_t score;
  int32_t a_begin, a_end, b_begin, b_end;
  int32_t n_ident, n_cols;
  int32_t status;
};

// Kernel shape of the group-striped fill: G lanes per pair, R rows per lane,
// int32 or int16x2 values.
struct Shape {
  int G, R, i16;
};

// A warp task: up to 32/G pairs of one lane width G, processed by one warp
// (x = first index into the task list, y = (G << 16) | number of pairs).
// The planner orders warp tasks longest first; warps of one persistent
// launch pull them from a single counter.
struct FillArgs {
  const uint8_t *codes;
  const PairDev *pairs;
  const int32_t *tasks;  // pair ids, grouped by warp task
  const int2 *wtasks;
  int32_t n_wtasks;
  const int32_t *n_wtasks_dev;  // when set, the warp-task count is read here (int32 re-run)
  int32_t *counter;      // work-queue head, zero before the launch
  const int8_t *matrix;  // 26*26 device copy of the scheme
  int32_t gap_open, gap_extend;
  ResultDev *res;
  int32_t *bnd;          // boundary scratch: per warp, 8 group rows
  int32_t bnd_cols;      // entries per group row (max n over the launch, even)
  uint8_t *planes;       // TB planes (kOutTrace)
  const int64_t *plane_off;  // byte offset of each pair's planes
  int32_t *overflow;     // int16 CHECK: per pair, 1 when a lane came near 32767
  int32_t max_score;     // largest substitution score of the scheme
  uint32_t one;          // int16x2 fill: 1, an opaque multiplier for packed subtractions on the IMAD pipe
  const uint8_t *ccodes;  // int16x2 fill: class code per residue (0 for invalid ones), same offsets as codes
  const int8_t *cmatrix;  // int16x2 fill: nclasses x nclasses class scores
  int32_t nclasses;
  int32_t spin_limit;     // CTA fill: polls per bounded wait (0 = the compiled default)
};

// Compacts the pairs an int16 CHECK launch flagged into a warp-task list
// for the int32 re-run (one pair per warp task, same lane width).
cudaError_t launch_collect_overflow(const int32_t *checked, int32_t n_checked, const int32_t *overflow,
                                    const int32_t *pair_g, int32_t *rerun_tasks, int2 *rerun_wtasks,
                                    int32_t *rerun_count, cudaStream_t st);

struct WalkArgs {
  const uint8_t *seqs;  // ASCII residues (for the emitted strings)
  const uint8_t *codes;
  const PairDev *pairs;
  const int32_t *tasks;
  int32_t n_tasks;
  const uint8_t *planes;
  const int64_t *plane_off;
  const int32_t *shape_G;  // per pair: the G and R its planes were written with
  const int32_t *shape_R;
  int32_t local;
  ResultDev *res;
  char *aln;                 // per pair: 2 * cap bytes (a row then b row)
  const int64_t *aln_off;
};

// Host-side helpers (scheme.cpp).
int build_scheme(const tsq_params *p, Scheme *out);
// BLOSUM62 entry by row index in the order ARNDCQEGHILKMFPSTWYVBZX.
int8_t blosum62_by_row(int x, int y);
void build_lut(const Scheme &s, uint8_t lut[256]);
// Byte -> score class (0 for bytes the scheme rejects, which their letter
// code marks invalid).
void build_class_lut(const Scheme &s, uint8_t lut[256]);

// Kernel launchers (fill_dispatch.cu, fill_i16.cu, fill_cta.cu, walk_kernel.cu).
// Returns the number of thread blocks a persistent launch of this shape uses.
// A launch covers every lane width G of one row height R and lane type
// (i16: 0 int32, 1 int16x2, 2 int16x2 with overflow check).
// Blocks of a fill launch resident on the device; nclasses sizes the int16x2
// fill's profile (ignored by the int32 fills).
int fill_blocks(int R, int i16, int out_mode, bool local, int nclasses = kLetters);
size_t fill_smem_bytes(int R, int i16, int out_mode, int nclasses = kLetters);
int fill_threads();
int fill_threads_for(int i16);
size_t fill_bnd_entry_bytes(int i16, int out_mode);
cudaError_t launch_fill(int R, int i16, int out_mode, bool local, const FillArgs &a, int blocks,
                        cudaStream_t st);
bool shape_supported(const Shape &sh, int out_mode, bool local);
// One long pair per CTA (fill_cta.cu): FillArgs.tasks / n_wtasks hold the
// pair list, bnd one wrap-around row of bnd_cols entries per block.
int cta_blocks(int out_mode, bool local);
size_t cta_bnd_entry_bytes(int out_mode);
cudaError_t launch_cta(int out_mode, bool local, const FillArgs &a, int blocks, cudaStream_t st);
// The same in int16x2 lanes with rebased values (fill_cta16.cu): score and
// traceback output, global or local, open + ext + max_score <= 40.
// FillArgs also carries the class codes, class matrix and class count.
bool cta16_supported(int out_mode, bool local, const Scheme &sc, int32_t gap_open, int32_t gap_extend);
int cta16_blocks(int out_mode, bool local, int nclasses);
cudaError_t launch_cta16(int out_mode, bool local, const FillArgs &a, int blocks, cudaStream_t st);
cudaError_t launch_walk(const WalkArgs &a, cudaStream_t st);
// Residues -> letter codes and, when clut_dev / ccodes are set, score
// classes.
cudaError_t launch_encode(const uint8_t *seqs, int64_t len, const uint8_t *lut_dev, uint8_t *codes,
                          const uint8_t *clut_dev, uint8_t *ccodes, cudaStream_t st);

// Bytes of traceback planes a pair needs under a shape.
inline int64_t plane_bytes(int m, int n, const Shape &sh) {
  if (m <= 0 || n <= 0) return 0;
  const int64_t P = (int64_t)sh.G * sh.R;
  const int64_t passes = (m + P - 1) / P;
  const int64_t entry = sh.R / 2;  // R nibbles per lane per step
  int64_t b = passes * (int64_t)(n + sh.G - 1) * sh.G * entry;
  return (b + 15) & ~int64_t(15);
}

}  // namespace tsq
