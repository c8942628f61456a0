"""GPU test of the allocation-free entry point, tsq_align_score_noalloc.

It serves callers that cannot allocate device memory (another allocator
owns it, or allocation is not allowed on their path): they pass device
buffers they already own and a stream.  Here the test itself owns those
buffers (allocated with torch before the call).  The entry point must
allocate nothing -- the device's free memory stays the same across calls --
and must give the same scores as the CPU oracle and as the ordinary batch
entry point tsq_align_batch, on two calls in a row (the second call runs
over the library's scratch array as the first one left it).  Integer
scores: the tolerance is exact equality.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tweakseq_gb300 import _native as N
from tweakseq_gb300 import aligner as A
from tweakseq_gb300 import build as B
from tweakseq_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FIELDS = ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols", "status")


def _pairs(seed, n, lo, hi, edge_lengths=()):
    """Related protein pairs; the first pairs take the given lengths (a and b
    both), the rest uniform lengths in [lo, hi]."""
    rng = np.random.default_rng(seed)
    seqs, pairs = [], []
    for k in range(n):
        m = edge_lengths[k] if k < len(edge_lengths) else int(rng.integers(lo, hi + 1))
        a = W.random_protein(rng, m)
        b, _ = W._mutate_proteins(rng, a, np.array([len(a)]), np.array([0.4]), 0.05)
        b = b[:m] if len(b) >= m else np.concatenate([b, W.random_protein(rng, m - len(b))])
        if k >= len(edge_lengths) and len(b) == 0:
            b = a[:1]
        seqs += [a.tobytes(), b.tobytes()]
        pairs.append((2 * k, 2 * k + 1))
    return W._pairset_from_lists(seqs, pairs)


class _DeviceInputs:
    """The caller's own device buffers: residues, pair table, results."""

    def __init__(self, ps, torch):
        self.n = len(ps)
        self.seqs_len = len(ps.seqs)
        self.seqs = torch.from_numpy(ps.seqs.copy()).cuda()
        tab = A.pair_table(ps.a_off, ps.a_len, ps.b_off, ps.b_len)
        self.pairs = torch.from_numpy(tab.view(np.uint8).copy()).cuda()
        self.out = torch.full((self.n * 8,), 7, dtype=torch.int32, device="cuda")

    def call(self, mode, max_len, stream, seqs_ptr=None):
        L = N.lib()
        p, keep = N.make_params(output="score", mode=mode)
        self.out.fill_(7)
        rc = L.tsq_align_score_noalloc(self.seqs.data_ptr() if seqs_ptr is None else seqs_ptr, self.seqs_len,
                                       self.pairs.data_ptr(), self.n, max_len, ctypes.byref(p),
                                       self.out.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        stream.synchronize()
        del keep
        return rc

    def results(self):
        return self.out.cpu().numpy().view(np.dtype([(f, np.int32) for f in FIELDS]))


@pytest.mark.parametrize("mode", ["global", "local"])
def test_noalloc_matches_oracle_and_batch_twice(mode):
    torch = pytest.importorskip("torch")
    B.build()
    O.build()
    stream = torch.cuda.Stream()
    # Edge lengths first (1, a warp's width and its neighbours, the largest
    # lengths the entry point takes), then 700 uneven pairs.
    edges = (1, 2, 31, 32, 33, 63, 64, 65, 2047, 2048)
    ps = _pairs(77, 710, 1, 2048, edges)
    assert ps.a_len[8] == 2047 and ps.b_len[9] == 2048
    local = mode == "local"
    want = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, O.BLOSUM62, 11, 1, local, O.MODE_SCORE)
    batch = A.align_batch(ps, mode=mode, output="score")
    fields = ("score", "a_end", "b_end") if local else ("score",)
    dev = _DeviceInputs(ps, torch)
    free = []
    for call in range(3):
        rc = dev.call(mode, 2048, stream)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        got = dev.results()
        assert rc == N.TSQ_OK, call
        assert (got["status"] == 0).all(), call
        for f in fields:
            assert np.array_equal(got[f], want[f]), (call, f, np.flatnonzero(got[f] != want[f])[:10])
            assert np.array_equal(got[f], batch.table[f]), (call, f)
    # The first call sets the device up; later calls allocate nothing.
    assert free[1] == free[2], free
    # A smaller batch after a bigger one: stale scratch contents do not leak.
    small = _DeviceInputs(ps.subset(np.arange(37)), torch)
    assert small.call(mode, 2048, stream) == N.TSQ_OK
    assert np.array_equal(small.results()["score"], want["score"][:37])


def test_noalloc_rejects_misaligned_residues():
    """A residue pointer that is not 16-byte aligned (an offset into the
    caller's own buffer) is refused on the host before anything runs; the
    next aligned call works."""
    torch = pytest.importorskip("torch")
    B.build()
    stream = torch.cuda.Stream()
    ps = _pairs(6, 30, 20, 300)
    dev = _DeviceInputs(ps, torch)
    assert dev.seqs.data_ptr() % 16 == 0
    rc = dev.call("global", 2048, stream, seqs_ptr=dev.seqs.data_ptr() + 1)
    assert rc == N.E_INVALID_ARG
    assert (dev.results()["score"] == 7).all()  # nothing was written
    assert dev.call("global", 2048, stream) == N.TSQ_OK
    want = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, O.BLOSUM62, 11, 1, False, O.MODE_SCORE)
    assert np.array_equal(dev.results()["score"], want["score"])


def test_noalloc_rejects_sizes_beyond_its_limits():
    torch = pytest.importorskip("torch")
    B.build()
    stream = torch.cuda.Stream()
    ps = _pairs(5, 20, 100, 600)
    dev = _DeviceInputs(ps, torch)
    assert dev.call("global", 4096, stream) == N.E_TOO_LARGE  # max_len above 2,048
    # Pairs longer than the caller's max_len are reported per pair.
    assert dev.call("global", 300, stream) == N.TSQ_OK
    got = dev.results()
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
