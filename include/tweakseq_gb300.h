/*
 * tweakseq_gb300.h -- C ABI of the GB300 pairwise-alignment library.
 *
 * The reference, groundstate/tweakseq, has no in-process pairwise alignment
 * call.  Its only seam for alignment is the AlignmentTool plugin
 * (tweakseq/Core/AlignmentTool.h:36-71): Project exports the selected
 * sequences as FASTA (tweakseq/Core/Project.cpp:870-894),
 * SeqEditMainWin::startAlignment runs the tool's command line through
 * QProcess (tweakseq/UI/SeqEditMainWin.cpp:1616-1663), and
 * Project::readNewAlignment reads back one gapped string per label
 * (tweakseq/Core/Project.cpp:908-1032).  The entry points below replace the
 * external process behind that seam: they take the residues the editor
 * would have written (Sequence::filter output, tweakseq/Core/Sequence.cpp:57-69:
 * uppercase ASCII, flag bits already stripped) and return the equal-length
 * gapped strings, with '-' as the gap character as the editor uses it
 * (tweakseq/Core/Sequences.cpp:266-287), that readNewAlignment consumes.
 *
 * Scoring: BLOSUM62 with the reference's letter map
 * (tweakseq/Core/Annotations/Consensus.cpp:34-69; J, O, U score as X), DNA
 * (+2 / -3 over IUPAC letters) or a caller-supplied 26x26 int8 matrix.  A gap
 * of length k costs gap_open + k * gap_extend.  Tie-breaks, identity and
 * coordinates follow the conventions stated in the library's documentation
 * and are bit-exact against the project's CPU oracle.
 *
 * Every function returns an int status: TSQ_OK (0) or a negative TSQ_E_*
 * code.  Nothing throws across the ABI.  There is no CPU fallback: without a
 * usable CUDA device the calls return TSQ_E_CUDA.
 */
#ifndef TWEAKSEQ_GB300_H_
#define TWEAKSEQ_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TSQ_ABI_VERSION 1

/* Status codes. */
#define TSQ_OK 0
#define TSQ_E_INVALID_ARG (-1)
#define TSQ_E_INVALID_RESIDUE (-2) /* byte outside 'A'..'Z' or not valid for the matrix */
#define TSQ_E_NOMEM (-3)           /* host or device allocation failed */
#define TSQ_E_CUDA (-4)            /* CUDA error or no device */
#define TSQ_E_TIMEOUT (-5)         /* a bounded device-side wait ran out */
#define TSQ_E_PENDING (-6)         /* server request not finished yet */
#define TSQ_E_REJECTED (-7)        /* request can never fit the server's HBM budget */
#define TSQ_E_NOT_FOUND (-8)       /* unknown server request id */
#define TSQ_E_CANCELLED (-9)       /* request cancelled before it ran */
#define TSQ_E_TOO_LARGE (-10)      /* input beyond a fixed capacity */

/* Scoring matrices. */
#define TSQ_MATRIX_BLOSUM62 0
#define TSQ_MATRIX_DNA 1
#define TSQ_MATRIX_CUSTOM 2

/* Alignment modes. */
#define TSQ_GLOBAL 0
#define TSQ_LOCAL 1

/* What to compute. */
#define TSQ_OUT_SCORE 0     /* score (local: plus end coordinates) */
#define TSQ_OUT_IDENTITY 1  /* score, n_ident and n_cols, no strings; a pair
                               with a_len + b_len > 65,535 gets
                               TSQ_E_TOO_LARGE (the two counts travel
                               together in 32 bits) -- use
                               TSQ_OUT_ALIGNMENT for longer pairs */
#define TSQ_OUT_ALIGNMENT 2 /* everything, gapped strings included */

/* DP lane width. */
#define TSQ_LANE_AUTO 0 /* int16x2 where it is exact, int32 otherwise */
#define TSQ_LANE_I16 1  /* int16x2 with overflow detection, int32 re-run on overflow */
#define TSQ_LANE_I32 2  /* int32 only */

typedef struct {
  int32_t matrix;              /* TSQ_MATRIX_* */
  int32_t gap_open;            /* >= 0 */
  int32_t gap_extend;          /* >= 0 */
  int32_t mode;                /* TSQ_GLOBAL or TSQ_LOCAL */
  int32_t output;              /* TSQ_OUT_* */
  int32_t lane;                /* TSQ_LANE_* */
  const int8_t *custom_score;  /* 26*26, [x][y] for 'A'+x vs 'A'+y (TSQ_MATRIX_CUSTOM) */
  const uint8_t *custom_valid; /* 26 flags (TSQ_MATRIX_CUSTOM) */
} tsq_params;

/* Result of one pair.  Coordinates are 0-based half-open: a[a_begin:a_end]
 * is aligned against b[b_begin:b_end].  Fields a mode does not compute are
 * -1 (begins for TSQ_OUT_SCORE local; n_ident/n_cols for TSQ_OUT_SCORE).
 * aln_a / aln_b are NUL-terminated, allocated by the library for
 * TSQ_OUT_ALIGNMENT and released by tsq_result_free; otherwise NULL. */
typedef struct {
  int32_t score;
  int32_t a_begin, a_end, b_begin, b_end;
  int32_t n_ident, n_cols;
  int32_t status; /* per-pair status (TSQ_OK or TSQ_E_INVALID_RESIDUE) */
  char *aln_a;
  char *aln_b;
} tsq_result;

/* One pair of a batch: offsets and lengths into the batch's residue buffer.
 * Per-pair limits (beyond them the pair gets TSQ_E_TOO_LARGE): each
 * sequence at most 1,048,575 residues; 3*gap_open + (a_len + b_len + 1) *
 * gap_extend below 2^28 (the int32 fill's range); identity output a_len +
 * b_len <= 65,535; local mode max_score * min(a_len, b_len) below 2^23. */
typedef struct {
  int64_t a_off, b_off;
  int32_t a_len, b_len;
} tsq_pair_desc;

typedef struct {
  int32_t device;       /* CUDA ordinal; -1 = current device */
  int32_t use_graph;    /* 1 = replay the launch sequence as a CUDA graph */
  int32_t autotune;     /* 1 = consult the tuned table (tsq_tune_load) */
  int32_t wait_polls;   /* polls a bounded device-side wait makes before it
                           gives up and its pair reports TSQ_E_TIMEOUT (the
                           long-pair fill's warps wait on one another);
                           0 = the default, 4,194,304 */
} tsq_batch_opts;

/* Counters of the last run of a batch. */
typedef struct {
  int64_t cells;           /* sum of m*n over the pairs */
  int64_t pairs;
  int64_t rerun_pairs;     /* pairs re-run in int32 after int16 overflow */
  int32_t launches;        /* kernel launches per run */
  int32_t buckets;         /* length buckets used */
  double device_ms;        /* device time of the last run (CUDA events) */
  double fill_ms;          /* of which the fill kernels */
} tsq_batch_stats;

/* ---- Version / device ---------------------------------------------------- */

/* ABI version and a static build description string. */
int tsq_version(int32_t *abi_version, const char **build);

/* ---- Plain form: one pair per call -------------------------------------- */

/* Aligns a (length la) with b (length lb) on the current CUDA device: one
 * launch sequence for this pair alone.  Fills *out; free it with
 * tsq_result_free. */
int tsq_align_pair(const uint8_t *a, int32_t la, const uint8_t *b, int32_t lb,
                   const tsq_params *p, tsq_result *out);

/* Releases the strings of one result (safe on results without strings). */
void tsq_result_free(tsq_result *r);
/* Releases the strings of n results. */
void tsq_results_free(tsq_result *r, int64_t n);
/* Copies the gapped strings of n results into one caller buffer, for
 * callers that take all of them at once (a binding that turns them into its
 * own string objects): for each result with strings, aln_a then aln_b,
 * n_cols bytes each, no terminators, back to back in result order; results
 * without strings contribute nothing.  Returns the bytes the strings take;
 * copies only when buf is not NULL and buf_len is at least that.  Negative
 * status on bad arguments.  Reads the results only (no device work). */
int64_t tsq_results_strings(const tsq_result *r, int64_t n, char *buf, int64_t buf_len);

/* ---- Batched form -------------------------------------------------------- */

/* Aligns n pairs over one host residue buffer in one planned launch
 * sequence (length buckets, persistent kernels, optional CUDA graph).
 * out[k] receives pair k.  Returns TSQ_E_INVALID_RESIDUE if any pair holds
 * an invalid residue (that pair's status says so; the others are valid). */
int tsq_align_batch(const uint8_t *seqs, int64_t seqs_len,
                    const tsq_pair_desc *pairs, int64_t n, const tsq_params *p,
                    const tsq_batch_opts *opts, tsq_result *out);

/* Device-resident batch: upload and plan once, run many times, read back. */
typedef struct tsq_batch tsq_batch;
int tsq_batch_create(const uint8_t *seqs, int64_t seqs_len,
                     const tsq_pair_desc *pairs, int64_t n, const tsq_params *p,
                     const tsq_batch_opts *opts, tsq_batch **out);
/* Enqueues one run on the batch's stream and waits for it. */
int tsq_batch_run(tsq_batch *b);
/* Enqueues one run without waiting (tsq_batch_sync waits). */
int tsq_batch_run_async(tsq_batch *b);
int tsq_batch_sync(tsq_batch *b);
/* Copies results of the last run to the host (strings allocated as above). */
int tsq_batch_results(tsq_batch *b, tsq_result *out);
int tsq_batch_get_stats(const tsq_batch *b, tsq_batch_stats *st);
/* The CUDA stream (cudaStream_t) the batch runs on, for event timing. */
int tsq_batch_stream(const tsq_batch *b, void **stream);
void tsq_batch_destroy(tsq_batch *b);

/* ---- Served form ----------------------------------------------------------- */

/* A continuous-batching server on one GPU.  Requests (1 to millions of
 * pairs, any parameters) are queued by tsq_server_submit from any thread; a
 * scheduler thread groups waiting requests with equal parameters into
 * ticks, admits a tick only while its device memory (residues, pair table,
 * results, band-boundary rows and, for alignments, traceback planes) fits
 * the HBM budget left by the ticks in flight, and runs up to `slots` ticks
 * at once on separate streams.  Each request's results equal those of
 * tsq_align_batch on that request alone.
 *
 * With opts.resident, score and identity requests whose pairs are at most
 * 2,048 residues long (and at most 65,536 pairs) go to a device-resident
 * request loop instead: a persistent kernel on half the SMs, one pair per
 * warp, takes the pairs of published requests from a task queue in device
 * memory; the request's residues, codes, pair table and results live in a
 * device arena until the request is polled, and completion is counted in
 * mapped host memory.  The kernel's waits are bounded: after
 * resident_idle_polls empty polls it ends, and the server relaunches it
 * when work arrives.  The loop holds SM resources while it runs, so ticks
 * running beside it get fewer blocks. */
typedef struct tsq_server tsq_server;

typedef struct {
  int32_t device;           /* CUDA ordinal; -1 = current device */
  int32_t slots;            /* ticks in flight at once (0 = 4) */
  int64_t hbm_budget_bytes; /* admission budget (0 = half the free HBM at creation) */
  int64_t max_tick_cells;   /* DP cells per tick before it closes (0 = 4e10) */
  int32_t autotune;         /* 1 = plan ticks with the tuned table */
  int32_t resident;         /* 1 = device-resident request loop for score and
                               identity requests of pairs up to 2,048 residues
                               (a persistent kernel fed from a device task
                               queue; see below) */
  int32_t resident_idle_polls; /* empty-queue polls (about a microsecond apart
                               at most) after which the loop's kernel ends;
                               the server relaunches it when work arrives
                               (0 = 1,048,576) */
  int32_t reserved;
} tsq_server_opts;

typedef struct {
  int64_t submitted, completed, rejected, cancelled;
  int64_t ticks;                /* launches planned so far */
  int64_t cells_completed;      /* DP cells of completed requests */
  int64_t peak_reserved_bytes;  /* largest HBM reservation of ticks in flight */
  int64_t admission_waits;      /* times the oldest request waited for memory */
  double p50_ms, p99_ms, max_ms; /* submit-to-completion latency */
  double span_s;                /* first submit to last completion */
  int64_t resident_requests;    /* requests served by the device-resident loop */
  int64_t resident_launches;    /* launches of the loop's kernel */
  int64_t resident_idle_exits;  /* times its kernel ended after idle_polls empty polls */
} tsq_server_stats;

int tsq_server_create(const tsq_server_opts *opts, tsq_server **out);
/* Queues a request (the inputs are copied); TSQ_E_REJECTED if it could never
 * fit the budget, TSQ_E_INVALID_ARG for a bad pair table. */
int tsq_server_submit(tsq_server *s, const uint8_t *seqs, int64_t seqs_len,
                      const tsq_pair_desc *pairs, int64_t n, const tsq_params *p,
                      uint64_t *request_id);
/* Waits up to wait_ms (0: no wait, <0: forever) for a request.  When it is
 * done, copies its n results to out (strings owned by the caller, release
 * with tsq_results_free), forgets the request and returns its status;
 * otherwise TSQ_E_PENDING.  TSQ_E_CANCELLED / TSQ_E_NOT_FOUND as named. */
int tsq_server_poll(tsq_server *s, uint64_t id, int32_t wait_ms, tsq_result *out, int64_t n);
/* Cancels a request that has not reached the device (TSQ_E_PENDING if it has). */
int tsq_server_cancel(tsq_server *s, uint64_t id);
int tsq_server_get_stats(tsq_server *s, tsq_server_stats *st);
/* Finishes the ticks in flight, cancels waiting requests, frees everything. */
int tsq_server_destroy(tsq_server *s);

/* ---- Autotuner ------------------------------------------------------------ */

/* Measures the compiled kernel shapes on the current device over seeded
 * synthetic pairs and writes the per-length-bucket choice as JSON. */
int tsq_tune_run(const char *json_path, int32_t quick);
/* Loads a tuned table written by tsq_tune_run (used when opts->autotune). */
int tsq_tune_load(const char *json_path);

/* ---- Allocation-free form --------------------------------------------------- */

/* Result of one pair written to device memory (same fields as tsq_result,
 * without strings). */
typedef struct {
  int32_t score;
  int32_t a_begin, a_end, b_begin, b_end;
  int32_t n_ident, n_cols;
  int32_t status;
} tsq_device_result;

/* Score-only batch for callers that cannot allocate device memory (their
 * memory is owned by another allocator, or allocation is not allowed on
 * their path).  This entry point has no counterpart in the reference.  The
 * caller passes device buffers it already owns -- residues d_seqs
 * (seqs_len bytes), the pair table d_pairs (n entries) and the results d_out
 * (n entries) -- and a CUDA stream (cudaStream_t, NULL for the legacy
 * stream); the call enqueues its kernels and returns without waiting.  All
 * intermediates live in one fixed 32 MiB device array inside the library
 * (held by every GPU that loads it until the process exits); nothing is
 * allocated.  Limits: seqs_len <= 8 MiB, n <= 1,048,576, max_len <= 2,048
 * (larger values return TSQ_E_TOO_LARGE); a pair longer than max_len or
 * outside the residue buffer gets status TSQ_E_TOO_LARGE / TSQ_E_INVALID_ARG
 * in d_out.  p->output must be TSQ_OUT_SCORE; p->lane is ignored (int32).
 * d_seqs must be 16-byte aligned (the residues are read 16 bytes at a
 * time), d_pairs 8-byte and d_out 4-byte aligned; a misaligned pointer is
 * refused with TSQ_E_INVALID_ARG before anything is launched.
 * The first call on a device sets up the device address of the array and
 * should come before any stream capture; that set-up lasts for the process
 * and is not redone after cudaDeviceReset.  Calls share the array: two calls
 * that overlap on the GPU race and corrupt each other's results. */
int tsq_align_score_noalloc(const uint8_t *d_seqs, int64_t seqs_len,
                            const tsq_pair_desc *d_pairs, int32_t n,
                            int32_t max_len, const tsq_params *p,
                            tsq_device_result *d_out, void *stream);

/* ---- Consensus line -------------------------------------------------------- */

/* Consensus of a gapped alignment; replaces Consensus::calculate
 * (tweakseq/Core/Annotations/Consensus.cpp:80-161, called from
 * Project::setAligned, tweakseq/Core/Project.cpp:112-121).  rows: nseq rows
 * of ncols bytes, row k at rows + k*stride (the low byte of each residue, as
 * the reference reads it).  For each column every row is scored against
 * every other row -- +1 when both bytes are outside 'A'..'Z' (a gap pair,
 * counted as a match), -4 when one is, else BLOSUM62 (a match when
 * positive; J, O, U share the X row) -- and the first row with the highest
 * sum wins.  consensus[c] is that row's byte when its match count is >=
 * plurality, else '?'.  plurality < 0 selects the reference's default,
 * nseq / 2 (Consensus::setSequences, Consensus.cpp:163-172).  best_score and
 * best_matches (either may be NULL) receive the winning row's figures.
 * Host buffers; the call copies in, computes and copies out. */
int tsq_consensus(const uint8_t *rows, int32_t nseq, int32_t ncols,
                  int64_t stride, double plurality, uint8_t *consensus,
                  int32_t *best_score, int32_t *best_matches);

/* Device-buffer form of tsq_consensus: everything already in device memory,
 * scratch of tsq_consensus_scratch_bytes(ncols) bytes supplied by the
 * caller, kernels enqueued on `stream` (cudaStream_t) without waiting.
 * Allocates nothing. */
size_t tsq_consensus_scratch_bytes(int32_t ncols);
int tsq_consensus_device(const uint8_t *d_rows, int32_t nseq, int32_t ncols,
                         int64_t stride, double plurality,
                         uint8_t *d_consensus, int32_t *d_best_score,
                         int32_t *d_best_matches, void *d_scratch,
                         size_t scratch_bytes, void *stream);

/* ---- Guide trees ------------------------------------------------------------- */

/* The tree step the external multiple aligners run after all-vs-all
 * (ClustalO is asked for tree order, tweakseq/Core/ClustalO.cpp:51); the
 * reference has no tree code of its own.  UPGMA or neighbour joining over
 * integer distances in units of 2^-32: d = floor((n_cols - n_ident) * 2^32
 * / n_cols), 2^32 when n_cols is 0.  Clusters hold positions 0..n-1; each
 * step joins the pair (i < j) with the smallest criterion (UPGMA: D(i,j);
 * NJ: (m-2) D(i,j) - r_i - r_j with r the row sums over the m active
 * clusters), ties to the smallest i then j; the join takes position i.
 * UPGMA: D(u,k) = floor((s_i D(i,k) + s_j D(j,k)) / (s_i + s_j)),
 * height floor(D(i,j)/2).  NJ: D(u,k) = floor((D(i,k) + D(j,k) - D(i,j))/2),
 * branch of i floor(((m-2) D(i,j) + r_i - r_j) / (2(m-2))) (floor(D(i,j)/2)
 * when m = 2), branch of j = D(i,j) minus that.  Join t is node n + t;
 * leaves are nodes 0..n-1.  n <= 65,535. */
#define TSQ_TREE_UPGMA 0
#define TSQ_TREE_NJ 1

typedef struct tsq_tree_node {
  int32_t left, right;   /* child node ids */
  int32_t size;          /* leaves under the join */
  int32_t pos;           /* position the join takes */
  int64_t dist;          /* D(left, right) when joined (2^-32 units) */
  int64_t height;        /* UPGMA height (2^-32 units); 0 for NJ */
  int64_t left_length;   /* branch lengths (2^-32 units) */
  int64_t right_length;
} tsq_tree_node;

/* From a symmetric n x n distance matrix (row-major, 2^-32 units; the
 * diagonal is ignored).  out: n - 1 joins. */
int tsq_guide_tree_dist(int32_t n, const int64_t *dist, int32_t method,
                        tsq_tree_node *out);

/* From identities of the n(n-1)/2 unordered pairs (i < j) in row-major
 * order: (0,1), (0,2), ..., (0,n-1), (1,2), ... */
int tsq_guide_tree(int32_t n, const int32_t *n_ident, const int32_t *n_cols,
                   int32_t method, tsq_tree_node *out);

/* From a batch that has run: its pairs must be the all-vs-all of n
 * sequences in the order above (pair (i,j) aligns sequence i as a against
 * sequence j as b) with TSQ_OUT_IDENTITY or TSQ_OUT_ALIGNMENT.  The
 * identities stay in device memory; only the joins come back. */
int tsq_batch_guide_tree(tsq_batch *b, int32_t n, int32_t method,
                         tsq_tree_node *out);

/* ---- Device probe ---------------------------------------------------------- */

/* Measured rate of the DP fill's DPX-class instructions (add-then-max and
 * three-way max) on the current device, in instructions per lane per second;
 * packed = 0 for the int32 forms, 1 for the int16x2 forms (two cells per
 * instruction).  This is the denominator of the fill's roofline. */
int tsq_probe_dpx(int32_t packed, double *instr_per_s);

#ifdef __cplusplus
}
#endif

#endif /* TWEAKSEQ_GB300_H_ */
