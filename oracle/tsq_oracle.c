/*
 * tsq_oracle.c -- scalar CPU restatement of Gotoh (1982) affine-gap global
 * and local alignment with traceback.  TEST INFRASTRUCTURE ONLY: the checker
 * for the CUDA library and the timed CPU baseline.  The conventions it fixes
 * are written at the top of tsq_oracle.h; parity is unpinned (the reference,
 * groundstate/tweakseq, delegates all DP to external programs).
 *
 * Deliberately plain: one cell at a time, int32 everywhere, no SIMD, so that
 * each line can be checked against the recurrences by reading.
 */
#include "tsq_oracle.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define NEG_INF (INT32_MIN / 4)

/* BLOSUM62 in the published row order ARNDCQEGHILKMFPSTWYVBZX.  The values
 * and the order are those of tweakseq/Core/Annotations/Consensus.cpp:34-59
 * (checked by tests/test_oracle.py against a fixture extracted from that
 * file). */
static const char kB62Order[23] = {'A', 'R', 'N', 'D', 'C', 'Q', 'E', 'G',
                                   'H', 'I', 'L', 'K', 'M', 'F', 'P', 'S',
                                   'T', 'W', 'Y', 'V', 'B', 'Z', 'X'};
static const int8_t kB62[23][23] = {
    {4, -1, -2, -2, 0, -1, -1, 0, -2, -1, -1, -1, -1, -2, -1, 1, 0, -3, -2, 0, -2, -1, 0},
    {-1, 5, 0, -2, -3, 1, 0, -2, 0, -3, -2, 2, -1, -3, -2, -1, -1, -3, -2, -3, -1, 0, -1},
    {-2, 0, 6, 1, -3, 0, 0, 0, 1, -3, -3, 0, -2, -3, -2, 1, 0, -4, -2, -3, 3, 0, -1},
    {-2, -2, 1, 6, -3, 0, 2, -1, -1, -3, -4, -1, -3, -3, -1, 0, -1, -4, -3, -3, 4, 1, -1},
    {0, -3, -3, -3, 9, -3, -4, -3, -3, -1, -1, -3, -1, -2, -3, -1, -1, -2, -2, -1, -3, -3, -2},
    {-1, 1, 0, 0, -3, 5, 2, -2, 0, -3, -2, 1, 0, -3, -1, 0, -1, -2, -1, -2, 0, 3, -1},
    {-1, 0, 0, 2, -4, 2, 5, -2, 0, -3, -3, 1, -2, -3, -1, 0, -1, -3, -2, -2, 1, 4, -1},
    {0, -2, 0, -1, -3, -2, -2, 6, -2, -4, -4, -2, -3, -3, -2, 0, -2, -2, -3, -3, -1, -2, -1},
    {-2, 0, 1, -1, -3, 0, 0, -2, 8, -3, -3, -1, -2, -1, -2, -1, -2, -2, 2, -3, 0, 0, -1},
    {-1, -3, -3, -3, -1, -3, -3, -4, -3, 4, 2, -3, 1, 0, -3, -2, -1, -3, -1, 3, -3, -3, -1},
    {-1, -2, -3, -4, -1, -2, -3, -4, -3, 2, 4, -2, 2, 0, -3, -2, -1, -2, -1, 1, -4, -3, -1},
    {-1, 2, 0, -1, -3, 1, 1, -2, -1, -3, -2, 5, -1, -3, -1, 0, -1, -3, -2, -2, 0, 1, -1},
    {-1, -1, -2, -3, -1, 0, -2, -3, -2, 1, 2, -1, 5, 0, -2, -1, -1, -1, -1, 1, -3, -1, -1},
    {-2, -3, -3, -3, -2, -3, -3, -3, -1, 0, 0, -3, 0, 6, -4, -2, -2, 1, 3, -1, -3, -3, -1},
    {-1, -2, -2, -1, -3, -1, -1, -2, -2, -3, -3, -1, -2, -4, 7, -1, -1, -4, -3, -2, -2, -1, -2},
    {1, -1, 1, 0, -1, 0, 0, 0, -1, -2, -2, 0, -1, -2, -1, 4, 1, -3, -2, -2, 0, 0, 0},
    {0, -1, 0, -1, -1, -1, -1, -2, -2, -1, -1, -1, -1, -2, -1, 1, 5, -2, -2, 0, -1, -1, 0},
    {-3, -3, -4, -4, -2, -2, -3, -2, -2, -3, -2, -3, -1, 1, -4, -3, -2, 11, 2, -3, -4, -3, -2},
    {-2, -2, -2, -3, -2, -1, -2, -3, 2, -1, -1, -2, -1, 3, -3, -2, -2, 2, 7, -1, -3, -2, -1},
    {0, -3, -3, -3, -1, -2, -2, -3, -3, 3, 1, -2, 1, -1, -2, -2, 0, -3, -1, 4, -3, -2, -1},
    {-2, -1, 3, 4, -3, 0, 1, -1, 0, -3, -4, 0, -3, -3, -2, 0, -1, -4, -3, -3, 4, 1, -1},
    {-1, 0, 0, 1, -3, 3, 4, -2, 0, -3, -3, 1, -1, -3, -1, 0, -1, -3, -2, -2, 1, 4, -1},
    {0, -1, -1, -1, -2, -1, -1, -1, -1, -1, -1, -1, -1, -1, -2, 0, 0, -2, -1, -1, -1, -1, -1}};

/* Index of a letter in kB62Order; J, O and U have no row of their own and
 * score as X, as the reference's letter map does (Consensus.cpp:61-69). */
static int b62_index(char c) {
  if (c == 'J' || c == 'O' || c == 'U') c = 'X';
  for (int k = 0; k < 23; ++k)
    if (kB62Order[k] == c) return k;
  return -1;
}

int tsqo_builtin_scheme(int id, tsqo_scheme *out) {
  if (!out) return TSQO_E_INVALID_ARG;
  memset(out, 0, sizeof(*out));
  if (id == TSQO_MATRIX_BLOSUM62) {
    for (int x = 0; x < 26; ++x) {
      out->valid[x] = 1;
      for (int y = 0; y < 26; ++y)
        out->score[x][y] = kB62[b62_index((char)('A' + x))][b62_index((char)('A' + y))];
    }
    return TSQO_OK;
  }
  if (id == TSQO_MATRIX_DNA) {
    /* IUPAC nucleotide letters are accepted.  Identical A, C, G, T or U
     * score +2; every other combination, ambiguity codes included (N vs N),
     * scores -3. */
    const char *iupac = "ACGTURYKMSWBDHVN";
    const char *bases = "ACGTU";
    for (const char *p = iupac; *p; ++p) out->valid[*p - 'A'] = 1;
    for (int x = 0; x < 26; ++x)
      for (int y = 0; y < 26; ++y) out->score[x][y] = -3;
    for (const char *p = bases; *p; ++p) out->score[*p - 'A'][*p - 'A'] = 2;
    return TSQO_OK;
  }
  return TSQO_E_INVALID_ARG;
}

/* Converts residues to 0..25 letter indices; returns 0 or an error. */
static int encode(const uint8_t *s, int32_t len, const tsqo_scheme *sc,
                  uint8_t *code) {
  for (int32_t k = 0; k < len; ++k) {
    uint8_t c = s[k];
    if (c < 'A' || c > 'Z' || !sc->valid[c - 'A']) return TSQO_E_INVALID_RESIDUE;
    code[k] = (uint8_t)(c - 'A');
  }
  return TSQO_OK;
}

static int check_args(const uint8_t *a, int32_t m, const uint8_t *b, int32_t n,
                      const tsqo_scheme *sc, int32_t go, int32_t ge,
                      tsqo_result *out) {
  if (!sc || !out || m < 0 || n < 0 || go < 0 || ge < 0) return TSQO_E_INVALID_ARG;
  if ((m > 0 && !a) || (n > 0 && !b)) return TSQO_E_INVALID_ARG;
  return TSQO_OK;
}

/* Direction codes of the H plane. */
enum { DIR_DIAG = 0, DIR_E = 1, DIR_F = 2, DIR_STOP = 3 };
#define BIT_EOPEN 4
#define BIT_FOPEN 8

int tsqo_align(const uint8_t *a, int32_t m, const uint8_t *b, int32_t n,
               const tsqo_scheme *sc, int32_t go, int32_t ge, int32_t local,
               char *aln_a, char *aln_b, tsqo_result *out) {
  int rc = check_args(a, m, b, n, sc, go, ge, out);
  if (rc) return rc;
  const int32_t oe = go + ge;
  const size_t W = (size_t)n + 1;
  uint8_t *ca = malloc((size_t)m + 1), *cb = malloc((size_t)n + 1);
  int32_t *H = malloc(sizeof(int32_t) * W * 2);
  int32_t *F = malloc(sizeof(int32_t) * W);
  uint8_t *dir = malloc(((size_t)m + 1) * W);
  char *ra = malloc((size_t)m + n + 1), *rb = malloc((size_t)m + n + 1);
  if (!ca || !cb || !H || !F || !dir || !ra || !rb) {
    rc = TSQO_E_NOMEM;
    goto done;
  }
  if ((rc = encode(a, m, sc, ca)) || (rc = encode(b, n, sc, cb))) goto done;

  int32_t *Hprev = H, *Hcur = H + W;
  int32_t best = 0, bi = 0, bj = 0;
  /* Row 0. */
  Hprev[0] = 0;
  for (int32_t j = 1; j <= n; ++j) {
    Hprev[j] = local ? 0 : -(go + j * ge);
    F[j] = NEG_INF;
    dir[j] = DIR_E; /* only read by the walk for global, where it is a gap run */
  }
  for (int32_t i = 1; i <= m; ++i) {
    Hcur[0] = local ? 0 : -(go + i * ge);
    int32_t E = NEG_INF;
    uint8_t *drow = dir + (size_t)i * W;
    drow[0] = DIR_F;
    const int8_t *srow = sc->score[ca[i - 1]];
    for (int32_t j = 1; j <= n; ++j) {
      uint8_t d = 0;
      /* E from the left neighbour in this row. */
      int32_t e_open = Hcur[j - 1] - oe, e_ext = E - ge;
      if (e_open >= e_ext) {
        E = e_open;
        d |= BIT_EOPEN;
      } else {
        E = e_ext;
      }
      /* F from the cell above. */
      int32_t f_open = Hprev[j] - oe, f_ext = F[j] - ge;
      if (f_open >= f_ext) {
        F[j] = f_open;
        d |= BIT_FOPEN;
      } else {
        F[j] = f_ext;
      }
      int32_t h = Hprev[j - 1] + srow[cb[j - 1]];
      uint8_t hd = DIR_DIAG;
      if (E > h) {
        h = E;
        hd = DIR_E;
      }
      if (F[j] > h) {
        h = F[j];
        hd = DIR_F;
      }
      if (local && h <= 0) {
        h = 0;
        hd = DIR_STOP;
      }
      Hcur[j] = h;
      drow[j] = (uint8_t)(d | hd);
      if (local && h > best) {
        best = h;
        bi = i;
        bj = j;
      }
    }
    int32_t *t = Hprev;
    Hprev = Hcur;
    Hcur = t;
  }

  int32_t i, j;
  if (local) {
    out->score = best;
    i = bi;
    j = bj;
  } else {
    out->score = Hprev[n];
    i = m;
    j = n;
  }
  out->a_end = i;
  out->b_end = j;

  /* Walk.  state 0 = H, 1 = E, 2 = F. */
  int state = 0;
  int32_t L = 0, ident = 0;
  for (;;) {
    if (state == 0) {
      if (local && (i == 0 || j == 0 || (dir[(size_t)i * W + j] & 3) == DIR_STOP)) break;
      if (!local && i == 0 && j == 0) break;
      if (i == 0) { /* global top row: one horizontal gap run */
        ra[L] = '-';
        rb[L] = (char)b[j - 1];
        ++L;
        --j;
        continue;
      }
      if (j == 0) { /* global left column: one vertical gap run */
        ra[L] = (char)a[i - 1];
        rb[L] = '-';
        ++L;
        --i;
        continue;
      }
      int hd = dir[(size_t)i * W + j] & 3;
      if (hd == DIR_DIAG) {
        ra[L] = (char)a[i - 1];
        rb[L] = (char)b[j - 1];
        if (a[i - 1] == b[j - 1]) ++ident;
        ++L;
        --i;
        --j;
      } else {
        state = hd; /* DIR_E == 1, DIR_F == 2 */
      }
    } else if (state == 1) {
      uint8_t d = dir[(size_t)i * W + j];
      ra[L] = '-';
      rb[L] = (char)b[j - 1];
      ++L;
      --j;
      if (d & BIT_EOPEN) state = 0;
    } else {
      uint8_t d = dir[(size_t)i * W + j];
      ra[L] = (char)a[i - 1];
      rb[L] = '-';
      ++L;
      --i;
      if (d & BIT_FOPEN) state = 0;
    }
  }
  out->a_begin = i;
  out->b_begin = j;
  if (local && out->score == 0) {
    out->a_begin = out->a_end = out->b_begin = out->b_end = 0;
  }
  out->n_cols = L;
  out->n_ident = ident;
  if (aln_a) {
    for (int32_t k = 0; k < L; ++k) aln_a[k] = ra[L - 1 - k];
    aln_a[L] = 0;
  }
  if (aln_b) {
    for (int32_t k = 0; k < L; ++k) aln_b[k] = rb[L - 1 - k];
    aln_b[L] = 0;
  }
  rc = TSQO_OK;
done:
  free(ca);
  free(cb);
  free(H);
  free(F);
  free(dir);
  free(ra);
  free(rb);
  return rc;
}

int tsqo_score(const uint8_t *a, int32_t m, const uint8_t *b, int32_t n,
               const tsqo_scheme *sc, int32_t go, int32_t ge, int32_t local,
               tsqo_result *out) {
  int rc = check_args(a, m, b, n, sc, go, ge, out);
  if (rc) return rc;
  const int32_t oe = go + ge;
  uint8_t *ca = malloc((size_t)m + 1), *cb = malloc((size_t)n + 1);
  int32_t *H = malloc(sizeof(int32_t) * ((size_t)n + 1));
  int32_t *F = malloc(sizeof(int32_t) * ((size_t)n + 1));
  if (!ca || !cb || !H || !F) {
    rc = TSQO_E_NOMEM;
    goto done;
  }
  if ((rc = encode(a, m, sc, ca)) || (rc = encode(b, n, sc, cb))) goto done;
  H[0] = 0;
  for (int32_t j = 1; j <= n; ++j) {
    H[j] = local ? 0 : -(go + j * ge);
    F[j] = NEG_INF;
  }
  int32_t best = 0, bi = 0, bj = 0;
  for (int32_t i = 1; i <= m; ++i) {
    int32_t diag = H[0];
    H[0] = local ? 0 : -(go + i * ge);
    int32_t E = NEG_INF;
    const int8_t *srow = sc->score[ca[i - 1]];
    for (int32_t j = 1; j <= n; ++j) {
      int32_t e_open = H[j - 1] - oe, e_ext = E - ge;
      E = e_open >= e_ext ? e_open : e_ext;
      int32_t f_open = H[j] - oe, f_ext = F[j] - ge;
      F[j] = f_open >= f_ext ? f_open : f_ext;
      int32_t h = diag + srow[cb[j - 1]];
      if (E > h) h = E;
      if (F[j] > h) h = F[j];
      if (local && h < 0) h = 0;
      diag = H[j];
      H[j] = h;
      if (local && h > best) {
        best = h;
        bi = i;
        bj = j;
      }
    }
  }
  if (local) {
    out->score = best;
    out->a_end = bi;
    out->b_end = bj;
    out->a_begin = out->b_begin = best > 0 ? -1 : 0;
  } else {
    out->score = H[n];
    out->a_begin = 0;
    out->a_end = m;
    out->b_begin = 0;
    out->b_end = n;
  }
  out->n_ident = out->n_cols = -1;
  rc = TSQO_OK;
done:
  free(ca);
  free(cb);
  free(H);
  free(F);
  return rc;
}

/* Counts of the tie-break path packed as (ident << 16) | cols would overflow
 * for long DNA, so the two are carried as separate int32 arrays. */
int tsqo_score_ident(const uint8_t *a, int32_t m, const uint8_t *b, int32_t n,
                     const tsqo_scheme *sc, int32_t go, int32_t ge,
                     int32_t local, tsqo_result *out) {
  int rc = check_args(a, m, b, n, sc, go, ge, out);
  if (rc) return rc;
  const int32_t oe = go + ge;
  const size_t W = (size_t)n + 1;
  uint8_t *ca = malloc((size_t)m + 1), *cb = malloc((size_t)n + 1);
  int32_t *H = malloc(sizeof(int32_t) * W), *F = malloc(sizeof(int32_t) * W);
  int32_t *hI = malloc(sizeof(int32_t) * W), *hC = malloc(sizeof(int32_t) * W);
  int32_t *fI = malloc(sizeof(int32_t) * W), *fC = malloc(sizeof(int32_t) * W);
  if (!ca || !cb || !H || !F || !hI || !hC || !fI || !fC) {
    rc = TSQO_E_NOMEM;
    goto done;
  }
  if ((rc = encode(a, m, sc, ca)) || (rc = encode(b, n, sc, cb))) goto done;
  H[0] = 0;
  hI[0] = hC[0] = 0;
  for (int32_t j = 1; j <= n; ++j) {
    H[j] = local ? 0 : -(go + j * ge);
    hI[j] = 0;
    hC[j] = local ? 0 : j;
    F[j] = NEG_INF;
    fI[j] = fC[j] = 0;
  }
  int32_t best = 0, bi = 0, bj = 0, bI = 0, bC = 0;
  for (int32_t i = 1; i <= m; ++i) {
    int32_t diag = H[0], dI = hI[0], dC = hC[0];
    H[0] = local ? 0 : -(go + i * ge);
    hI[0] = 0;
    hC[0] = local ? 0 : i;
    int32_t E = NEG_INF, eI = 0, eC = 0;
    const int8_t *srow = sc->score[ca[i - 1]];
    for (int32_t j = 1; j <= n; ++j) {
      /* E: from (i, j-1). */
      int32_t e_open = H[j - 1] - oe, e_ext = E - ge;
      if (e_open >= e_ext) {
        E = e_open;
        eI = hI[j - 1];
        eC = hC[j - 1] + 1;
      } else {
        E = e_ext;
        eC = eC + 1;
      }
      /* F: from (i-1, j). */
      int32_t f_open = H[j] - oe, f_ext = F[j] - ge;
      if (f_open >= f_ext) {
        F[j] = f_open;
        fI[j] = hI[j];
        fC[j] = hC[j] + 1;
      } else {
        F[j] = f_ext;
        fC[j] = fC[j] + 1;
      }
      int32_t h = diag + srow[cb[j - 1]];
      int32_t nI = dI + (a[i - 1] == b[j - 1]), nC = dC + 1;
      if (E > h) {
        h = E;
        nI = eI;
        nC = eC;
      }
      if (F[j] > h) {
        h = F[j];
        nI = fI[j];
        nC = fC[j];
      }
      if (local && h <= 0) {
        h = 0;
        nI = nC = 0;
      }
      diag = H[j];
      dI = hI[j];
      dC = hC[j];
      H[j] = h;
      hI[j] = nI;
      hC[j] = nC;
      if (local && h > best) {
        best = h;
        bi = i;
        bj = j;
        bI = nI;
        bC = nC;
      }
    }
  }
  if (local) {
    out->score = best;
    out->a_end = bi;
    out->b_end = bj;
    out->a_begin = out->b_begin = -1;
    out->n_ident = bI;
    out->n_cols = bC;
    if (best == 0) out->a_end = out->b_end = out->a_begin = out->b_begin = 0;
  } else {
    out->score = H[n];
    out->a_begin = 0;
    out->a_end = m;
    out->b_begin = 0;
    out->b_end = n;
    out->n_ident = hI[n];
    out->n_cols = hC[n];
  }
  rc = TSQO_OK;
done:
  free(ca);
  free(cb);
  free(H);
  free(F);
  free(hI);
  free(hC);
  free(fI);
  free(fC);
  return rc;
}

/* Last row (H and F) of a global fill of codes x (len p) against y (len q). */
static void global_last_row(const uint8_t *x, int32_t p, const uint8_t *y,
                            int32_t q, const tsqo_scheme *sc, int32_t go,
                            int32_t ge, int32_t *H, int32_t *F) {
  const int32_t oe = go + ge;
  H[0] = 0;
  F[0] = NEG_INF;
  for (int32_t j = 1; j <= q; ++j) {
    H[j] = -(go + j * ge);
    F[j] = NEG_INF;
  }
  for (int32_t i = 1; i <= p; ++i) {
    int32_t diag = H[0];
    H[0] = -(go + i * ge);
    F[0] = H[0]; /* column 0 is one vertical gap run */
    int32_t E = NEG_INF;
    for (int32_t j = 1; j <= q; ++j) {
      int32_t e_open = H[j - 1] - oe, e_ext = E - ge;
      E = e_open >= e_ext ? e_open : e_ext;
      int32_t f_open = H[j] - oe, f_ext = F[j] - ge;
      F[j] = f_open >= f_ext ? f_open : f_ext;
      int32_t h = diag + sc->score[x[i - 1]][y[j - 1]];
      if (E > h) h = E;
      if (F[j] > h) h = F[j];
      diag = H[j];
      H[j] = h;
    }
  }
}

int tsqo_score_global_midpoint(const uint8_t *a, int32_t m, const uint8_t *b,
                               int32_t n, const tsqo_scheme *sc, int32_t go,
                               int32_t ge, int32_t *score) {
  if (!sc || !score || m < 2 || n < 0) return TSQO_E_INVALID_ARG;
  int rc = TSQO_OK;
  uint8_t *ca = malloc((size_t)m), *cb = malloc((size_t)n + 1);
  uint8_t *ra = malloc((size_t)m), *rb = calloc((size_t)n + 1, 1);
  int32_t *Hf = malloc(sizeof(int32_t) * ((size_t)n + 1));
  int32_t *Ff = malloc(sizeof(int32_t) * ((size_t)n + 1));
  int32_t *Hr = malloc(sizeof(int32_t) * ((size_t)n + 1));
  int32_t *Fr = malloc(sizeof(int32_t) * ((size_t)n + 1));
  if (!ca || !cb || !ra || !rb || !Hf || !Ff || !Hr || !Fr) {
    rc = TSQO_E_NOMEM;
    goto done;
  }
  if ((rc = encode(a, m, sc, ca)) || (rc = encode(b, n, sc, cb))) goto done;
  int32_t mid = m / 2;
  for (int32_t k = 0; k < m; ++k) ra[k] = ca[m - 1 - k];
  for (int32_t k = 0; k < n; ++k) rb[k] = cb[n - 1 - k];
  global_last_row(ca, mid, cb, n, sc, go, ge, Hf, Ff);
  global_last_row(ra, m - mid, rb, n, sc, go, ge, Hr, Fr);
  int32_t best = NEG_INF;
  for (int32_t j = 0; j <= n; ++j) {
    int32_t through_h = Hf[j] + Hr[n - j];
    int32_t through_f = Ff[j] + Fr[n - j] + go; /* one gap run, one open */
    if (through_h > best) best = through_h;
    if (through_f > best) best = through_f;
  }
  *score = best;
done:
  free(ca);
  free(cb);
  free(ra);
  free(rb);
  free(Hf);
  free(Ff);
  free(Hr);
  free(Fr);
  return rc;
}

int tsqo_num_cores(void) {
  long c = sysconf(_SC_NPROCESSORS_ONLN);
  return c > 0 ? (int)c : 1;
}

typedef struct {
  const uint8_t *seqs;
  const int64_t *a_off, *b_off, *aln_off;
  const int32_t *a_len, *b_len;
  int64_t npairs;
  const tsqo_scheme *sc;
  int32_t go, ge, local, mode;
  char *aln_a, *aln_b;
  tsqo_result *out;
  atomic_llong next;
  atomic_int status;
} batch_job;

static void *batch_worker(void *arg) {
  batch_job *J = (batch_job *)arg;
  for (;;) {
    int64_t k = atomic_fetch_add(&J->next, 1);
    if (k >= J->npairs) break;
    const uint8_t *a = J->seqs + J->a_off[k], *b = J->seqs + J->b_off[k];
    int32_t m = J->a_len[k], n = J->b_len[k];
    int rc;
    if (J->mode == 0)
      rc = tsqo_score(a, m, b, n, J->sc, J->go, J->ge, J->local, &J->out[k]);
    else if (J->mode == 1)
      rc = tsqo_score_ident(a, m, b, n, J->sc, J->go, J->ge, J->local, &J->out[k]);
    else
      rc = tsqo_align(a, m, b, n, J->sc, J->go, J->ge, J->local,
                      J->aln_a ? J->aln_a + J->aln_off[k] : NULL,
                      J->aln_b ? J->aln_b + J->aln_off[k] : NULL, &J->out[k]);
    if (rc) {
      int zero = 0;
      atomic_compare_exchange_strong(&J->status, &zero, rc);
    }
  }
  return NULL;
}

int tsqo_batch(const uint8_t *seqs, const int64_t *a_off, const int32_t *a_len,
               const int64_t *b_off, const int32_t *b_len, int64_t npairs,
               const tsqo_scheme *sc, int32_t go, int32_t ge, int32_t local,
               int32_t mode, int32_t nthreads, char *aln_a, char *aln_b,
               const int64_t *aln_off, tsqo_result *out) {
  if (npairs < 0 || !sc || !out || mode < 0 || mode > 2) return TSQO_E_INVALID_ARG;
  if ((aln_a || aln_b) && !aln_off) return TSQO_E_INVALID_ARG;
  if (npairs == 0) return TSQO_OK;
  if (nthreads <= 0) nthreads = tsqo_num_cores();
  if (nthreads > npairs) nthreads = (int32_t)npairs;
  batch_job J;
  memset(&J, 0, sizeof(J));
  J.seqs = seqs;
  J.a_off = a_off;
  J.b_off = b_off;
  J.aln_off = aln_off;
  J.a_len = a_len;
  J.b_len = b_len;
  J.npairs = npairs;
  J.sc = sc;
  J.go = go;
  J.ge = ge;
  J.local = local;
  J.mode = mode;
  J.aln_a = aln_a;
  J.aln_b = aln_b;
  J.out = out;
  atomic_init(&J.next, 0);
  atomic_init(&J.status, 0);
  pthread_t *th = malloc(sizeof(pthread_t) * (size_t)nthreads);
  if (!th) return TSQO_E_NOMEM;
  int started = 0;
  for (int t = 1; t < nthreads; ++t)
    if (pthread_create(&th[started], NULL, batch_worker, &J) == 0) ++started;
  /* The calling thread works too. */
  batch_worker(&J);
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  free(th);
  return atomic_load(&J.status);
}

/* ------------------------------------------------------------------------
 * Consensus of a gapped alignment: Consensus::calculate restated loop for
 * loop (tweakseq/Core/Annotations/Consensus.cpp:80-161), O(ncols * nseq^2),
 * doubles as there, one column per task over POSIX threads.
 * ---------------------------------------------------------------------- */

/* Residue byte -> BLOSUM62 row, 99 for anything outside 'A'..'Z'
 * (Consensus.cpp:96-106; the map of :61-69 sends J, O, U, X to 22). */
static int consensus_class(uint8_t byte) {
  const int idx = (int)byte - 65;
  if (idx < 0 || idx > 25) return 99;
  return b62_index((char)byte);
}

typedef struct {
  const uint8_t *rows;
  int32_t nseq, ncols;
  int64_t stride;
  double plurality;
  uint8_t *out;
  int32_t *best_score, *best_matches;
  atomic_llong next;
} consensus_job;

static void consensus_column(const consensus_job *J, int32_t c) {
  double hi_score = 0.0, ri_matches = 0.0;
  int32_t ri_hi = 0;
  for (int32_t ri = 0; ri < J->nseq; ++ri) {
    double score = 0.0, matches = 0.0;
    const int resi = consensus_class(J->rows[(int64_t)ri * J->stride + c]);
    for (int32_t rj = 0; rj < J->nseq; ++rj) {
      if (ri == rj) continue;
      const double weight = 1.0;
      const int resj = consensus_class(J->rows[(int64_t)rj * J->stride + c]);
      if (resi == 99 && resj == 99) {
        score += weight;
        if (weight > 0) matches += weight;
      } else if (resi == 99 || resj == 99) {
        score += -4 * weight;
      } else {
        const double tmp = kB62[resi][resj] * weight;
        score += tmp;
        if (tmp > 0) matches += weight;
      }
    }
    if (ri == 0 || score > hi_score) {
      hi_score = score;
      ri_hi = ri;
      ri_matches = matches;
    }
  }
  J->out[c] = ri_matches >= J->plurality ? J->rows[(int64_t)ri_hi * J->stride + c] : (uint8_t)'?';
  if (J->best_score) J->best_score[c] = (int32_t)hi_score;
  if (J->best_matches) J->best_matches[c] = (int32_t)ri_matches;
}

static void *consensus_worker(void *arg) {
  consensus_job *J = (consensus_job *)arg;
  for (;;) {
    const int64_t c = atomic_fetch_add(&J->next, 1);
    if (c >= J->ncols) break;
    consensus_column(J, (int32_t)c);
  }
  return NULL;
}

int tsqo_consensus(const uint8_t *rows, int32_t nseq, int32_t ncols, int64_t stride, double plurality,
                   int32_t nthreads, uint8_t *out, int32_t *best_score, int32_t *best_matches) {
  if (nseq <= 0 || ncols < 0 || stride < ncols || !rows || (!out && ncols)) return TSQO_E_INVALID_ARG;
  consensus_job J;
  memset(&J, 0, sizeof(J));
  J.rows = rows;
  J.nseq = nseq;
  J.ncols = ncols;
  J.stride = stride;
  /* Consensus::setSequences: plurality = (sum of unit weights) / 2. */
  J.plurality = plurality < 0 ? nseq / 2.0 : plurality;
  J.out = out;
  J.best_score = best_score;
  J.best_matches = best_matches;
  atomic_init(&J.next, 0);
  if (nthreads <= 0) nthreads = tsqo_num_cores();
  if (nthreads > ncols) nthreads = ncols > 0 ? ncols : 1;
  pthread_t *th = malloc(sizeof(pthread_t) * (size_t)nthreads);
  if (!th) return TSQO_E_NOMEM;
  int started = 0;
  for (int t = 1; t < nthreads; ++t)
    if (pthread_create(&th[started], NULL, consensus_worker, &J) == 0) ++started;
  consensus_worker(&J);
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  free(th);
  return TSQO_OK;
}

/* ------------------------------------------------------------------------
 * Guide tree from all-vs-all identities: UPGMA (Sokal & Michener 1958) or
 * neighbour joining (Saitou & Nei 1987, in the Studier & Keppler 1988 form)
 * over integer fixed-point distances, with the conventions of
 * tsq_oracle.h.  Plain O(n^3): every step scans every active pair.
 * ---------------------------------------------------------------------- */

int64_t tsqo_identity_distance(int32_t n_ident, int32_t n_cols) {
  if (n_cols <= 0) return TSQO_DIST_ONE;
  return (int64_t)(((uint64_t)(uint32_t)(n_cols - n_ident) << 32) / (uint64_t)(uint32_t)n_cols);
}

static int64_t floor_div(int64_t a, int64_t b) {
  int64_t q = a / b;
  if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
  return q;
}

int tsqo_guide_tree(int32_t n, const int64_t *dist, int32_t method, tsqo_tree_node *out) {
  if (n < 1 || !dist || (method != TSQO_TREE_UPGMA && method != TSQO_TREE_NJ) || (!out && n > 1))
    return TSQO_E_INVALID_ARG;
  int64_t *D = malloc(sizeof(int64_t) * (size_t)n * (size_t)n);
  int64_t *r = malloc(sizeof(int64_t) * (size_t)n);
  int64_t *height = malloc(sizeof(int64_t) * (size_t)n);
  int32_t *node = malloc(sizeof(int32_t) * (size_t)n), *size = malloc(sizeof(int32_t) * (size_t)n);
  uint8_t *active = malloc((size_t)n);
  if (!D || !r || !height || !node || !size || !active) {
    free(D), free(r), free(height), free(node), free(size), free(active);
    return TSQO_E_NOMEM;
  }
  memcpy(D, dist, sizeof(int64_t) * (size_t)n * (size_t)n);
  for (int32_t i = 0; i < n; ++i) {
    node[i] = i;
    size[i] = 1;
    height[i] = 0;
    active[i] = 1;
    r[i] = 0;
    for (int32_t k = 0; k < n; ++k)
      if (k != i) r[i] += D[(int64_t)i * n + k];
  }
  int32_t m = n;
  for (int32_t t = 0; t < n - 1; ++t, --m) {
    int32_t bi = -1, bj = -1;
    int64_t best = 0;
    for (int32_t i = 0; i < n; ++i) {
      if (!active[i]) continue;
      for (int32_t j = i + 1; j < n; ++j) {
        if (!active[j]) continue;
        const int64_t dij = D[(int64_t)i * n + j];
        const int64_t c = method == TSQO_TREE_UPGMA ? dij : (int64_t)(m - 2) * dij - r[i] - r[j];
        if (bi < 0 || c < best) { /* strict: the first pair in (i, j) order wins ties */
          best = c;
          bi = i;
          bj = j;
        }
      }
    }
    const int64_t dij = D[(int64_t)bi * n + bj];
    tsqo_tree_node *o = &out[t];
    o->left = node[bi];
    o->right = node[bj];
    o->size = size[bi] + size[bj];
    o->pos = bi;
    o->dist = dij;
    if (method == TSQO_TREE_UPGMA) {
      const int64_t h = dij >> 1;
      o->height = h;
      o->left_length = h - height[bi];
      o->right_length = h - height[bj];
      height[bi] = h;
    } else {
      o->height = 0;
      if (m > 2) {
        o->left_length = floor_div((int64_t)(m - 2) * dij + r[bi] - r[bj], 2 * (int64_t)(m - 2));
      } else {
        o->left_length = dij >> 1;
      }
      o->right_length = dij - o->left_length;
    }
    /* Join: the new cluster takes position bi, position bj leaves. */
    int64_t r_new = 0;
    for (int32_t k = 0; k < n; ++k) {
      if (!active[k] || k == bi || k == bj) continue;
      const int64_t dik = D[(int64_t)bi * n + k], djk = D[(int64_t)bj * n + k];
      int64_t du;
      if (method == TSQO_TREE_UPGMA)
        du = floor_div((int64_t)size[bi] * dik + (int64_t)size[bj] * djk, (int64_t)(size[bi] + size[bj]));
      else
        du = (dik + djk - dij) >> 1;
      r[k] += du - dik - djk;
      r_new += du;
      D[(int64_t)bi * n + k] = du;
      D[(int64_t)k * n + bi] = du;
    }
    r[bi] = r_new;
    node[bi] = n + t;
    size[bi] += size[bj];
    active[bj] = 0;
  }
  free(D), free(r), free(height), free(node), free(size), free(active);
  return TSQO_OK;
}
