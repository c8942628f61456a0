/*
 * tsq_oracle.h -- CPU oracle for the pairwise affine-gap alignment path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * library under tweakseq_gb300/ and the timed CPU baseline of bench.py.  The
 * product never links, loads or calls it.
 *
 * PARITY UNPINNED.  groundstate/tweakseq has no pairwise DP of its own: its
 * "Align" action exports FASTA and runs an external program (ClustalO, MAFFT
 * or MUSCLE) through QProcess (tweakseq/UI/SeqEditMainWin.cpp:1616-1663,
 * tweakseq/Core/AlignmentTool.h:36-71).  Those programs are neither vendored
 * nor installed, and the reference ships no tests or golden vectors.  This
 * oracle therefore restates the published method -- Gotoh, O. (1982) "An
 * improved algorithm for matching biological sequences", J. Mol. Biol.
 * 162:705-708, with the local variant of Smith & Waterman (1981) -- and fixes
 * the conventions below.  What IS pinned against the reference is the
 * scoring data: the BLOSUM62 table and its A..Z index map are checked against
 * tweakseq/Core/Annotations/Consensus.cpp:34-69 by a committed fixture.
 *
 * Conventions (the CUDA library must reproduce every one bit for bit):
 *   - Residues are uppercase ASCII 'A'..'Z'.  A scoring scheme is a 26x26
 *     int8 matrix indexed by letter-'A' plus a validity flag per letter; a
 *     residue whose flag is 0, or any byte outside 'A'..'Z', is rejected
 *     with TSQO_E_INVALID_RESIDUE (the reference maps such bytes to a "gap"
 *     code, Consensus.cpp:96-106, which has no meaning for DP input).
 *   - Row i (1..m) consumes a[i-1]; column j (1..n) consumes b[j-1].
 *   - A gap of length k costs gap_open + k * gap_extend.
 *   - E (horizontal move, consumes b[j-1], '-' in the aligned a):
 *       E(i,j) = max(E(i,j-1) - ext, H(i,j-1) - open - ext)
 *     F (vertical move, consumes a[i-1], '-' in the aligned b):
 *       F(i,j) = max(F(i-1,j) - ext, H(i-1,j) - open - ext)
 *     H(i,j) = max(H(i-1,j-1) + s(a[i-1], b[j-1]), E(i,j), F(i,j) [, 0 local])
 *   - Global boundaries: H(0,0)=0, H(i,0) = -(open + i*ext), H(0,j) =
 *     -(open + j*ext); E(i,0) and F(0,j) are minus infinity.  End gaps are
 *     charged.  Local boundaries: H(i,0) = H(0,j) = 0.
 *   - Tie-breaks.  H: diagonal beats E beats F.  E and F: opening beats
 *     extending when the two candidates are equal.  Local: any cell whose
 *     best candidate is <= 0 gets H = 0 and direction STOP; the alignment
 *     ends at the FIRST cell in row-major order (smallest i, then smallest j)
 *     holding the maximum H, and the walk stops on entering a STOP cell or
 *     row/column 0.  If no cell is positive the local alignment is empty.
 *   - Identity: n_ident counts aligned columns whose two letters are equal;
 *     n_cols counts all columns of the alignment (gap columns included).
 *   - Coordinates are 0-based half-open: a[a_begin:a_end] is aligned against
 *     b[b_begin:b_end].  A global alignment spans [0,m) x [0,n).
 */
#ifndef TSQ_ORACLE_H_
#define TSQ_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TSQO_OK 0
#define TSQO_E_INVALID_ARG (-1)
#define TSQO_E_INVALID_RESIDUE (-2)
#define TSQO_E_NOMEM (-3)

/* Builtin schemes. */
#define TSQO_MATRIX_BLOSUM62 0
#define TSQO_MATRIX_DNA 1 /* +2 / -3, see tsqo_builtin_scheme */

typedef struct {
  int8_t score[26][26]; /* score[x][y] for letters 'A'+x vs 'A'+y */
  uint8_t valid[26];    /* 1 if letter 'A'+k is accepted */
} tsqo_scheme;

typedef struct {
  int32_t score;
  int32_t a_begin, a_end, b_begin, b_end;
  int32_t n_ident, n_cols;
} tsqo_result;

/* Fills *out with a builtin scheme; returns TSQO_E_INVALID_ARG for an
 * unknown id. */
int tsqo_builtin_scheme(int id, tsqo_scheme *out);

/* Full-matrix fill plus traceback.  aln_a / aln_b receive the gapped strings
 * (NUL terminated); each needs capacity m + n + 1.  Either may be NULL, in
 * which case the walk still runs (for identity and coordinates) but emits
 * nothing. */
int tsqo_align(const uint8_t *a, int32_t m, const uint8_t *b, int32_t n,
               const tsqo_scheme *sc, int32_t gap_open, int32_t gap_extend,
               int32_t local, char *aln_a, char *aln_b, tsqo_result *out);

/* Linear-space score-only fill.  Global: score only (coordinates set to the
 * full span, counts to -1).  Local: score and end coordinates a_end/b_end of
 * the first maximal cell (begins -1, or 0 when the alignment is empty;
 * counts -1). */
int tsqo_score(const uint8_t *a, int32_t m, const uint8_t *b, int32_t n,
               const tsqo_scheme *sc, int32_t gap_open, int32_t gap_extend,
               int32_t local, tsqo_result *out);

/* Linear-space fill that carries (n_ident, n_cols) of the tie-break path
 * forward, so that it equals what tsqo_align's walk reports, without
 * direction storage.  Begin coordinates are -1 for local. */
int tsqo_score_ident(const uint8_t *a, int32_t m, const uint8_t *b, int32_t n,
                     const tsqo_scheme *sc, int32_t gap_open,
                     int32_t gap_extend, int32_t local, tsqo_result *out);

/* Hirschberg / Myers-Miller style cross-check: global score via forward and
 * reverse half fills meeting in the middle row.  Used only to check the
 * oracle against itself. */
int tsqo_score_global_midpoint(const uint8_t *a, int32_t m, const uint8_t *b,
                               int32_t n, const tsqo_scheme *sc,
                               int32_t gap_open, int32_t gap_extend,
                               int32_t *score);

/* Batch over pairs stored in one residue buffer.  mode 0: tsqo_score,
 * 1: tsqo_score_ident, 2: tsqo_align (aln buffers may be NULL; when given,
 * pair k's strings go to aln_a + aln_off[k] and aln_b + aln_off[k], each
 * with capacity a_len[k] + b_len[k] + 1).  Pairs are scheduled dynamically
 * over nthreads POSIX threads (nthreads <= 0: all online cores).  Returns the
 * first non-zero status of any pair (others still run). */
int tsqo_batch(const uint8_t *seqs, const int64_t *a_off, const int32_t *a_len,
               const int64_t *b_off, const int32_t *b_len, int64_t npairs,
               const tsqo_scheme *sc, int32_t gap_open, int32_t gap_extend,
               int32_t local, int32_t mode, int32_t nthreads, char *aln_a,
               char *aln_b, const int64_t *aln_off, tsqo_result *out);

/* Number of online cores the batch driver uses by default. */
int tsqo_num_cores(void);

/* Consensus of a gapped alignment, restated loop for loop from
 * Consensus::calculate (tweakseq/Core/Annotations/Consensus.cpp:80-161):
 * rows holds nseq rows of ncols bytes (row k at rows + k*stride).  For each
 * column, every row ri scores the sum over the other rows rj of: +1 when
 * both bytes are outside 'A'..'Z' (a "gap" pair, counted as a match), -4
 * when exactly one is, else BLOSUM62[ri][rj] (counted as a match when
 * positive; J, O, U, X share the X row).  The first row with the highest
 * score wins; the column's consensus is that row's byte when its match count
 * is >= plurality, else '?'.  plurality < 0 means the reference's default,
 * nseq / 2 (Consensus::setSequences, Consensus.cpp:163-172).  best_score and
 * best_matches (either may be NULL) receive the winning row's figures. */
int tsqo_consensus(const uint8_t *rows, int32_t nseq, int32_t ncols, int64_t stride, double plurality,
                   int32_t nthreads, uint8_t *out, int32_t *best_score, int32_t *best_matches);

/* Guide trees from all-vs-all identities.
 *
 * Conventions (the CUDA library reproduces every one bit for bit):
 *   - Distances are integers in units of 2^-32: d = floor((n_cols - n_ident)
 *     * 2^32 / n_cols), 2^32 when n_cols is 0 (tsqo_identity_distance).
 *     Integer arithmetic makes every step exact and order-independent.
 *   - Clusters sit at positions 0..n-1 (leaf k at position k).  Each step
 *     joins the active pair (i < j) with the smallest criterion; ties go to
 *     the smallest i, then the smallest j.  The join takes position i, j
 *     leaves.  Join t (0-based) is node n + t; leaves are nodes 0..n-1.
 *   - UPGMA: criterion D(i,j); D(u,k) = floor((s_i D(i,k) + s_j D(j,k)) /
 *     (s_i + s_j)) with s the cluster sizes; height(u) = floor(D(i,j) / 2);
 *     branch length = height(u) - height(child).
 *   - NJ: with m active clusters and r_k = sum over active l != k of D(k,l),
 *     criterion (m - 2) D(i,j) - r_i - r_j; D(u,k) = floor((D(i,k) + D(j,k)
 *     - D(i,j)) / 2); branch length of i = floor(((m - 2) D(i,j) + r_i -
 *     r_j) / (2 (m - 2))) (floor(D(i,j) / 2) when m = 2), of j = D(i,j) minus
 *     that. */
#define TSQO_DIST_ONE ((int64_t)1 << 32)
#define TSQO_TREE_UPGMA 0
#define TSQO_TREE_NJ 1

typedef struct {
  int32_t left, right; /* node ids */
  int32_t size;        /* leaves under the join */
  int32_t pos;         /* position the join takes */
  int64_t dist;        /* D(left, right) when joined */
  int64_t height;      /* UPGMA height, 0 for NJ */
  int64_t left_length, right_length;
} tsqo_tree_node;

int64_t tsqo_identity_distance(int32_t n_ident, int32_t n_cols);

/* dist: n*n row-major, symmetric (the diagonal is ignored).  out: n-1
 * joins.  One leaf gives no joins. */
int tsqo_guide_tree(int32_t n, const int64_t *dist, int32_t method, tsqo_tree_node *out);

#ifdef __cplusplus
}
#endif

#endif /* TSQ_ORACLE_H_ */
