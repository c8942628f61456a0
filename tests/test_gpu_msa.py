"""GPU tests of the consensus kernel and the guide-tree kernels against the
oracle: bit-exact consensus bytes and per-column figures, identical joins
(ids, positions, distances, heights, branch lengths)."""
import numpy as np
import pytest

from oracle import oracle as O
from tweakseq_gb300 import _native as N
from tweakseq_gb300 import aligner as A
from tweakseq_gb300 import build as B
from tweakseq_gb300 import msa
from tweakseq_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    B.build()
    O.build()


def _family_msa(rng, nseq, ncols, gap=0.15, conserve=0.6):
    """Rows sharing a column profile: each column has a favourite residue
    kept with probability `conserve`, gaps with probability `gap`."""
    fav = W.random_protein(rng, ncols)
    rows = np.empty((nseq, ncols), dtype=np.uint8)
    for k in range(nseq):
        r = W.random_protein(rng, ncols)
        keep = rng.random(ncols) < conserve
        r[keep] = fav[keep]
        r[rng.random(ncols) < gap] = ord("-")
        rows[k] = r
    return rows


def _check_consensus(rows, plurality=None):
    got = msa.consensus(rows, plurality)
    want = O.consensus(rows, -1.0 if plurality is None else plurality)
    assert got.sequence == want[0]
    assert np.array_equal(got.best_score, want[1]) and np.array_equal(got.best_matches, want[2])


@pytest.mark.parametrize("nseq,ncols", [(1, 5), (2, 1), (3, 33), (7, 64), (64, 500), (1000, 97), (3000, 200)])
def test_consensus_matches_oracle(nseq, ncols):
    rng = np.random.default_rng(nseq * 1000 + ncols)
    _check_consensus(_family_msa(rng, nseq, ncols))


def test_consensus_every_byte_class_and_plurality():
    rng = np.random.default_rng(11)
    alphabet = np.frombuffer(b"AAGGLLWWC-.-aJOUXBZ*\x00\x80\xff", dtype=np.uint8)
    for nseq in (2, 5, 40):
        rows = rng.choice(alphabet, size=(nseq, 300)).astype(np.uint8)
        for plur in (None, 0.0, 1.0, nseq / 3.0, float(nseq)):
            _check_consensus(rows, plur)


@pytest.mark.parametrize("first", [0, 31, 32, 33, 64, 99])
def test_consensus_winner_found_past_the_first_rows(first):
    """Gaps down to row `first`, then W: W wins every column and its first
    row is `first` (the warp scans 32 rows per step)."""
    rows = np.full((100, 40), ord("-"), dtype=np.uint8)
    rows[first:, :] = ord("W")
    rows[first:, 7] = ord("C")
    _check_consensus(rows)
    _check_consensus(rows, plurality=5.0)


def test_consensus_device_entry_point():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    rows = _family_msa(rng, 500, 300)
    stride = 320
    host = np.zeros((500, stride), dtype=np.uint8)
    host[:, :300] = rows
    d_rows = torch.from_numpy(host).cuda()
    d_out = torch.zeros(300, dtype=torch.uint8, device="cuda")
    d_sc = torch.zeros(300, dtype=torch.int32, device="cuda")
    d_mt = torch.zeros(300, dtype=torch.int32, device="cuda")
    nbytes = N.lib().tsq_consensus_scratch_bytes(300)
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    rc = N.lib().tsq_consensus_device(d_rows.data_ptr(), 500, 300, stride, -1.0, d_out.data_ptr(), d_sc.data_ptr(),
                                      d_mt.data_ptr(), scratch.data_ptr(), nbytes, stream.cuda_stream)
    assert rc == 0
    stream.synchronize()
    want = O.consensus(rows)
    assert d_out.cpu().numpy().tobytes() == want[0]
    assert np.array_equal(d_sc.cpu().numpy(), want[1]) and np.array_equal(d_mt.cpu().numpy(), want[2])
    # Too little scratch is refused before anything runs.
    assert N.lib().tsq_consensus_device(d_rows.data_ptr(), 500, 300, stride, -1.0, d_out.data_ptr(), None, None,
                                        scratch.data_ptr(), nbytes - 1, stream.cuda_stream) == N.E_INVALID_ARG


def test_consensus_bad_arguments():
    L = N.lib()
    buf = np.zeros(16, dtype=np.uint8)
    out = np.zeros(16, dtype=np.uint8)
    assert L.tsq_consensus(buf.ctypes.data, 0, 4, 4, -1.0, out.ctypes.data, None, None) == N.E_INVALID_ARG
    assert L.tsq_consensus(buf.ctypes.data, 2, 8, 4, -1.0, out.ctypes.data, None, None) == N.E_INVALID_ARG
    assert L.tsq_consensus(None, 2, 4, 4, -1.0, out.ctypes.data, None, None) == N.E_INVALID_ARG


def _same_tree(tree, want):
    got = tree.nodes
    assert len(got) == len(want)
    for f in N.TREE_NODE_DTYPE.names:
        assert np.array_equal(got[f], want[f]), f


def _tied_identities(rng, n, levels=5):
    """Identities on a coarse grid so that many pairs tie."""
    npairs = n * (n - 1) // 2
    cols = np.full(npairs, 100, dtype=np.int32)
    ident = (rng.integers(0, levels, npairs) * (100 // levels)).astype(np.int32)
    return ident, cols


@pytest.mark.parametrize("method", ["upgma", "nj"])
@pytest.mark.parametrize("n", [2, 3, 17, 200, 600])
def test_tree_matches_oracle(method, n):
    rng = np.random.default_rng(n)
    ident, cols = _tied_identities(rng, n)
    D = O.identity_distances(n, ident, cols)
    want = O.guide_tree(D, N.TREE[method])
    _same_tree(msa.guide_tree(n, ident, cols, method), want)
    _same_tree(msa.guide_tree_from_distances(D, method), want)


@pytest.mark.parametrize("method", ["upgma", "nj"])
def test_tree_from_continuous_identities(method):
    rng = np.random.default_rng(21)
    n = 400
    npairs = n * (n - 1) // 2
    cols = rng.integers(200, 700, npairs).astype(np.int32)
    ident = (cols * rng.uniform(0.1, 0.6, npairs)).astype(np.int32)
    want = O.guide_tree(O.identity_distances(n, ident, cols), N.TREE[method])
    _same_tree(msa.guide_tree(n, ident, cols, method), want)


@pytest.mark.parametrize("method", ["upgma", "nj"])
def test_tree_from_device_resident_all_vs_all(method):
    ps = W.guide_tree_families(n_families=3, per_family=40, seed=41)
    n = 120
    assert len(ps) == n * (n - 1) // 2
    with A.Batch(ps, output="identity") as b:
        b.run()
        tree = msa.guide_tree_from_batch(b, n, method)
        res = b.results()
    want = O.guide_tree(O.identity_distances(n, res.table["n_ident"], res.table["n_cols"]), N.TREE[method])
    _same_tree(tree, want)
    assert sorted(tree.leaf_order()) == list(range(n))
    assert tree.newick().count("(") == n - 1


def test_tree_bad_arguments():
    L = N.lib()
    D = np.array([[0, 1, 2], [1, 0, 3], [2, 4, 0]], dtype=np.int64)  # not symmetric
    out = np.zeros(2, dtype=N.TREE_NODE_DTYPE)
    assert L.tsq_guide_tree_dist(3, D.ctypes.data, 0, out.ctypes.data) == N.E_INVALID_ARG
    assert L.tsq_guide_tree_dist(3, D.ctypes.data, 7, out.ctypes.data) == N.E_INVALID_ARG
    ident = np.array([1, 2, 3], dtype=np.int32)
    cols = np.array([2, 1, 4], dtype=np.int32)  # n_ident > n_cols
    assert L.tsq_guide_tree(3, ident.ctypes.data, cols.ctypes.data, 0, out.ctypes.data) == N.E_INVALID_ARG
    # A batch that is not an all-vs-all, or holds scores only.
    ps = W.guide_tree_families(n_families=1, per_family=5, seed=3)
    with A.Batch(ps, output="identity") as b:
        b.run()
        assert L.tsq_batch_guide_tree(b._h, 4, 0, out.ctypes.data) == N.E_INVALID_ARG
    sub = ps.subset(np.array([1, 0, 2, 3, 4, 5, 6, 7, 8, 9]))
    with A.Batch(sub, output="identity") as b:
        b.run()
        assert L.tsq_batch_guide_tree(b._h, 5, 0, np.zeros(4, dtype=N.TREE_NODE_DTYPE).ctypes.data) == N.E_INVALID_ARG
    with A.Batch(ps, output="score") as b:
        b.run()
        assert L.tsq_batch_guide_tree(b._h, 5, 0, np.zeros(4, dtype=N.TREE_NODE_DTYPE).ctypes.data) == N.E_INVALID_ARG
