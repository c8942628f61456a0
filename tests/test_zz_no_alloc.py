"""GPU test of the allocation-free entry point, tsq_align_score_noalloc.

It serves callers that cannot allocate device memory (another allocator
owns it, or allocation is not allowed on their path): they pass device
buffers they already own and a stream.  Here the test itself owns those
buffers (allocated with torch before the call); the entry point must
allocate nothing and must give the same scores as the ordinary batch entry
point tsq_align_batch, on two calls in a row (the second call runs over the
library's scratch array as the first one left it).  Integer scores: the
tolerance is exact equality.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

from tweakseq_gb300 import _native as N
from tweakseq_gb300 import aligner as A
from tweakseq_gb300 import build as B
from tweakseq_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _pairs(seed, n, lo, hi):
    rng = np.random.default_rng(seed)
    seqs, pairs = [], []
    for k in range(n):
        a = W.random_protein(rng, int(rng.integers(lo, hi + 1)))
        b, _ = W._mutate_proteins(rng, a, np.array([len(a)]), np.array([0.4]), 0.05)
        if len(b) == 0:
            b = a[:1]
        seqs += [a.tobytes(), b.tobytes()]
        pairs.append((2 * k, 2 * k + 1))
    return W._pairset_from_lists(seqs, pairs)


def _call(ps, mode, max_len, torch, stream):
    """Copies the pair set into device tensors owned by the test and calls
    the entry point; returns (status, results as a numpy structured array)."""
    L = N.lib()
    d_seqs = torch.from_numpy(ps.seqs.copy()).cuda()
    tab = A.pair_table(ps.a_off, ps.a_len, ps.b_off, ps.b_len)
    d_pairs = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
    d_out = torch.full((len(ps) * 8,), 7, dtype=torch.int32, device="cuda")
    p, keep = N.make_params(output="score", mode=mode)
    rc = L.tsq_align_score_noalloc(d_seqs.data_ptr(), len(ps.seqs), d_pairs.data_ptr(), len(ps), max_len,
                                   ctypes.byref(p), d_out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    stream.synchronize()
    out = d_out.cpu().numpy().view(np.dtype([(f, np.int32) for f in
                                             ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident",
                                              "n_cols", "status")]))
    del keep
    return rc, out


@pytest.mark.parametrize("mode", ["global", "local"])
def test_noalloc_matches_batch_entry_point_twice(mode):
    torch = pytest.importorskip("torch")
    B.build()
    stream = torch.cuda.Stream()
    ps = _pairs(77, 700, 1, 2048)
    want = A.align_batch(ps, mode=mode, output="score")
    fields = ("score", "a_end", "b_end") if mode == "local" else ("score",)
    for call in range(2):
        rc, got = _call(ps, mode, 2048, torch, stream)
        assert rc == N.TSQ_OK, call
        assert (got["status"] == 0).all(), call
        for f in fields:
            assert np.array_equal(got[f], want.table[f]), (call, f)
    # A smaller batch after a bigger one: stale scratch contents do not leak.
    small = ps.subset(np.arange(37))
    rc, got = _call(small, mode, 2048, torch, stream)
    assert rc == N.TSQ_OK and np.array_equal(got["score"], want.table["score"][:37])


def test_noalloc_rejects_sizes_beyond_its_limits():
    torch = pytest.importorskip("torch")
    B.build()
    stream = torch.cuda.Stream()
    ps = _pairs(5, 20, 100, 600)
    rc, _ = _call(ps, "global", 4096, torch, stream)  # max_len above 2,048
    assert rc == N.E_TOO_LARGE
    # Pairs longer than the caller's max_len are reported per pair.
    rc, got = _call(ps, "global", 300, torch, stream)
    assert rc == N.TSQ_OK
    too_long = (ps.a_len > 300) | (ps.b_len > 300)
    assert too_long.any() and (~too_long).any()
    assert (got["status"][too_long] == N.E_TOO_LARGE).all()
    want = A.align_batch(ps.subset(np.flatnonzero(~too_long)), output="score")
    assert np.array_equal(got["score"][~too_long], want.table["score"])
    # More residues than the array holds.
    L = N.lib()
    p, keep = N.make_params(output="score")
    rc = L.tsq_align_score_noalloc(None, (8 << 20) + 1, None, 0, 100, ctypes.byref(p), None, None)
    assert rc == N.E_TOO_LARGE
