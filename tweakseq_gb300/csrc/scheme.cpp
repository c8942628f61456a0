// scheme.cpp -- scoring schemes and the residue lookup table.
//
// BLOSUM62 values and row order (ARNDCQEGHILKMFPSTWYVBZX) are the ones of
// tweakseq/Core/Annotations/Consensus.cpp:34-59, and letters map to rows as
// in Consensus.cpp:61-69 (J, O and U have no row and score as X).  The
// reference maps any other byte to a "gap" code (Consensus.cpp:96-106); for
// DP input that has no meaning, so such bytes are rejected with
// TSQ_E_INVALID_RESIDUE.
#include <cstring>

#include "tsq_internal.h"

namespace tsq {
namespace {

constexpr char kRowOrder[] = "ARNDCQEGHILKMFPSTWYVBZX";

// clang-format off
constexpr int8_t kBlosum62[23][23] = {
  { 4,-1,-2,-2, 0,-1,-1, 0,-2,-1,-1,-1,-1,-2,-1, 1, 0,-3,-2, 0,-2,-1, 0},
  {-1, 5, 0,-2,-3, 1, 0,-2, 0,-3,-2, 2,-1,-3,-2,-1,-1,-3,-2,-3,-1, 0,-1},
  {-2, 0, 6, 1,-3, 0, 0, 0, 1,-3,-3, 0,-2,-3,-2, 1, 0,-4,-2,-3, 3, 0,-1},
  {-2,-2, 1, 6,-3, 0, 2,-1,-1,-3,-4,-1,-3,-3,-1, 0,-1,-4,-3,-3, 4, 1,-1},
  { 0,-3,-3,-3, 9,-3,-4,-3,-3,-1,-1,-3,-1,-2,-3,-1,-1,-2,-2,-1,-3,-3,-2},
  {-1, 1, 0, 0,-3, 5, 2,-2, 0,-3,-2, 1, 0,-3,-1, 0,-1,-2,-1,-2, 0, 3,-1},
  {-1, 0, 0, 2,-4, 2, 5,-2, 0,-3,-3, 1,-2,-3,-1, 0,-1,-3,-2,-2, 1, 4,-1},
  { 0,-2, 0,-1,-3,-2,-2, 6,-2,-4,-4,-2,-3,-3,-2, 0,-2,-2,-3,-3,-1,-2,-1},
  {-2, 0, 1,-1,-3, 0, 0,-2, 8,-3,-3,-1,-2,-1,-2,-1,-2,-2, 2,-3, 0, 0,-1},
  {-1,-3,-3,-3,-1,-3,-3,-4,-3, 4, 2,-3, 1, 0,-3,-2,-1,-3,-1, 3,-3,-3,-1},
  {-1,-2,-3,-4,-1,-2,-3,-4,-3, 2, 4,-2, 2, 0,-3,-2,-1,-2,-1, 1,-4,-3,-1},
  {-1, 2, 0,-1,-3, 1, 1,-2,-1,-3,-2, 5,-1,-3,-1, 0,-1,-3,-2,-2, 0, 1,-1},
  {-1,-1,-2,-3,-1, 0,-2,-3,-2, 1, 2,-1, 5, 0,-2,-1,-1,-1,-1, 1,-3,-1,-1},
  {-2,-3,-3,-3,-2,-3,-3,-3,-1, 0, 0,-3, 0, 6,-4,-2,-2, 1, 3,-1,-3,-3,-1},
  {-1,-2,-2,-1,-3,-1,-1,-2,-2,-3,-3,-1,-2,-4, 7,-1,-1,-4,-3,-2,-2,-1,-2},
  { 1,-1, 1, 0,-1, 0, 0, 0,-1,-2,-2, 0,-1,-2,-1, 4, 1,-3,-2,-2, 0, 0, 0},
  { 0,-1, 0,-1,-1,-1,-1,-2,-2,-1,-1,-1,-1,-2,-1, 1, 5,-2,-2, 0,-1,-1, 0},
  {-3,-3,-4,-4,-2,-2,-3,-2,-2,-3,-2,-3,-1, 1,-4,-3,-2,11, 2,-3,-4,-3,-2},
  {-2,-2,-2,-3,-2,-1,-2,-3, 2,-1,-1,-2,-1, 3,-3,-2,-2, 2, 7,-1,-3,-2,-1},
  { 0,-3,-3,-3,-1,-2,-2,-3,-3, 3, 1,-2, 1,-1,-2,-2, 0,-3,-1, 4,-3,-2,-1},
  {-2,-1, 3, 4,-3, 0, 1,-1, 0,-3,-4, 0,-3,-3,-2, 0,-1,-4,-3,-3, 4, 1,-1},
  {-1, 0, 0, 1,-3, 3, 4,-2, 0,-3,-3, 1,-1,-3,-1, 0,-1,-3,-2,-2, 1, 4,-1},
  { 0,-1,-1,-1,-2,-1,-1,-1,-1,-1,-1,-1,-1,-1,-2, 0, 0,-2,-1,-1,-1,-1,-1},
};
// clang-format on

}  // namespace

int8_t blosum62_by_row(int x, int y) { return kBlosum62[x][y]; }

namespace {

int blosum_row(char letter) {
  if (letter == 'J' || letter == 'O' || letter == 'U') letter = 'X';
  const char *p = std::strchr(kRowOrder, letter);
  return p ? int(p - kRowOrder) : -1;
}

// letters: every valid letter its own class (identity fills test letter
// equality on class codes).
void finish(Scheme *s, bool letters) {
  s->max_score = -128;
  s->min_score = 127;
  s->symmetric = true;
  for (int x = 0; x < kLetters; ++x)
    for (int y = 0; y < kLetters; ++y) {
      if (!s->valid[x] || !s->valid[y]) continue;
      const int v = s->score[x][y];
      if (v > s->max_score) s->max_score = v;
      if (v < s->min_score) s->min_score = v;
      if (s->score[x][y] != s->score[y][x]) s->symmetric = false;
    }
  if (s->max_score < s->min_score) s->max_score = s->min_score = 0;
  // Score classes, numbered in letter order of their first letter (or of
  // their only letter).
  int rep[kLetters];
  s->nclasses = 0;
  for (int x = 0; x < kLetters; ++x) {
    s->cls[x] = kBadCode;
    if (!s->valid[x]) continue;
    for (int c = 0; !letters && c < s->nclasses && s->cls[x] == kBadCode; ++c) {
      const int r = rep[c];
      bool same = true;
      for (int y = 0; y < kLetters && same; ++y)
        if (s->valid[y]) same = s->score[x][y] == s->score[r][y] && s->score[y][x] == s->score[y][r];
      if (same) s->cls[x] = uint8_t(c);
    }
    if (s->cls[x] == kBadCode) {
      rep[s->nclasses] = x;
      s->cls[x] = uint8_t(s->nclasses++);
    }
  }
  for (int a = 0; a < s->nclasses; ++a)
    for (int b = 0; b < s->nclasses; ++b) s->cscore[a * s->nclasses + b] = s->score[rep[a]][rep[b]];
}

}  // namespace

int build_scheme(const tsq_params *p, Scheme *out) {
  std::memset(out, 0, sizeof(*out));
  switch (p->matrix) {
    case TSQ_MATRIX_BLOSUM62:
      for (int x = 0; x < kLetters; ++x) {
        out->valid[x] = 1;
        for (int y = 0; y < kLetters; ++y)
          out->score[x][y] = kBlosum62[blosum_row(char('A' + x))][blosum_row(char('A' + y))];
      }
      break;
    case TSQ_MATRIX_DNA: {
      // IUPAC nucleotide letters; identical A/C/G/T/U score +2, anything
      // else (ambiguity codes included, N vs N too) scores -3.
      for (const char *c = "ACGTURYKMSWBDHVN"; *c; ++c) out->valid[*c - 'A'] = 1;
      for (int x = 0; x < kLetters; ++x)
        for (int y = 0; y < kLetters; ++y) out->score[x][y] = -3;
      for (const char *c = "ACGTU"; *c; ++c) out->score[*c - 'A'][*c - 'A'] = 2;
      break;
    }
    case TSQ_MATRIX_CUSTOM:
      if (!p->custom_score || !p->custom_valid) return TSQ_E_INVALID_ARG;
      std::memcpy(out->score, p->custom_score, sizeof(out->score));
      for (int x = 0; x < kLetters; ++x) out->valid[x] = p->custom_valid[x] ? 1 : 0;
      break;
    default:
      return TSQ_E_INVALID_ARG;
  }
  finish(out, p->output == TSQ_OUT_IDENTITY);
  return TSQ_OK;
}

void build_lut(const Scheme &s, uint8_t lut[256]) {
  for (int c = 0; c < 256; ++c) lut[c] = kBadCode;
  for (int x = 0; x < kLetters; ++x)
    if (s.valid[x]) lut['A' + x] = uint8_t(x);
}

void build_class_lut(const Scheme &s, uint8_t lut[256]) {
  // Bytes the scheme rejects get class 0 (their letter code marks them
  // invalid): every class code is a valid profile index.
  for (int c = 0; c < 256; ++c) lut[c] = 0;
  for (int x = 0; x < kLetters; ++x)
    if (s.valid[x]) lut['A' + x] = s.cls[x];
}

}  // namespace tsq
