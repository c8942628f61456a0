"""GPU parity of the long-DNA traceback workload at its full size: all
1,000 pairs (reference lengths 10-50 kb, query with 10 % substitutions and
2 % indels, +2/-3, gap 5/2, global, full traceback) through
tsq_align_batch, which runs them in waves sized to the free device memory
on the CTA fill (bands striped over 8 warps, shared-memory rings, the
warp-7 to warp-0 wrap row) and the diagonal-run walker.  A seeded sample of
pairs, always including the longest pair of the workload (49,947 x 49,990,
2.5e9 cells, about 60,000 walk steps), is compared with the CPU oracle byte
for byte: score, coordinates, identity and both gapped strings.

The oracle keeps one direction byte per cell, so its threads are bounded by
the host's free memory."""
import numpy as np
import pytest

from oracle import oracle as O
from tweakseq_gb300 import aligner as A
from tweakseq_gb300 import build as B
from tweakseq_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FIELDS = ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols")


def sample_with_longest(ps, n_sample, seed):
    cells = ps.a_len.astype(np.int64) * ps.b_len.astype(np.int64)
    longest = int(np.argmax(cells))
    rest = np.random.default_rng(seed).choice(np.delete(np.arange(len(ps)), longest), n_sample - 1, replace=False)
    return np.concatenate([[longest], np.sort(rest)])


def test_long_dna_full_workload_strings_vs_oracle():
    B.build()
    O.build()
    ps = W.long_dna_pairs(1000)
    res = A.align_batch(ps, matrix="dna", gap_open=5, gap_extend=2, output="alignment")
    assert (res.table["status"] == 0).all()
    idx = sample_with_longest(ps, 8, seed=11)
    assert ps.a_len[idx[0]] == 49947 and ps.b_len[idx[0]] == 49990
    sub = ps.subset(idx)
    cells = sub.a_len.astype(np.int64) * sub.b_len.astype(np.int64)
    nthreads = O.threads_for_traceback(int(cells.max()), cap=4)
    want, sa, sb = O.batch(sub.seqs, sub.a_off, sub.a_len, sub.b_off, sub.b_len, O.DNA, 5, 2, False, O.MODE_ALIGN,
                           nthreads, True)
    for j, k in enumerate(idx):
        for f in FIELDS:
            assert res.table[f][k] == want[f][j], (int(k), f, int(res.table[f][k]), int(want[f][j]))
        assert res.aln_a[k] == sa[j], int(k)
        assert res.aln_b[k] == sb[j], int(k)
    # Every string of the 1,000 pairs: equal lengths, n_cols columns, the
    # inputs back when the gaps are removed.
    for k in range(len(ps)):
        a, b = ps.pair(k)
        assert len(res.aln_a[k]) == len(res.aln_b[k]) == res.table["n_cols"][k], k
        assert res.aln_a[k].replace("-", "").encode() == a and res.aln_b[k].replace("-", "").encode() == b, k
