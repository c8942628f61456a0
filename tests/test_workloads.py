"""CPU tests of the seeded synthetic workloads the benchmark runs on: their
sizes, length ranges and the exact cell counts the bench reports (a change
to a generator would change every measured number, so the counts are
pinned here).  No GPU call."""
import numpy as np

from tweakseq_gb300 import workloads as W


def test_all_vs_all_of_64_proteins():
    ps = W.all_vs_all_proteins()
    assert len(ps) == 64 * 63 // 2 == 2016
    assert ps.cells == 177_528_662
    assert ps.a_len.min() >= 200 and ps.a_len.max() <= 400
    assert ps.matrix == W.BLOSUM62 and (ps.gap_open, ps.gap_extend) == (11, 1)


def test_uneven_pairs_100k():
    ps = W.uneven_pairs()
    assert len(ps) == 100_000
    assert ps.cells == 20_106_789_943
    assert ps.a_len.min() == 50 and ps.a_len.max() == 2000 and np.median(ps.a_len) == 350
    # Partners differ by point substitutions and single-residue indels (5 %).
    rel = ps.b_len.astype(np.float64) / ps.a_len
    assert 0.85 < rel.min() and rel.max() < 1.15 and abs(rel.mean() - 1.0) < 0.01
    letters = set(np.unique(ps.seqs).tobytes())
    assert letters <= set(b"ACDEFGHIKLMNPQRSTVWY")


def test_long_dna_pairs_1000():
    ps = W.long_dna_pairs(1000)
    assert len(ps) == 1000
    assert ps.cells == 1_034_831_748_406
    assert ps.a_len.min() >= 10_000 and ps.a_len.max() <= 50_000
    rel = ps.b_len.astype(np.float64) / ps.a_len
    assert 0.95 < rel.min() and rel.max() < 1.05
    assert set(np.unique(ps.seqs).tobytes()) == set(b"ACGT")
    assert ps.matrix == W.DNA and (ps.gap_open, ps.gap_extend) == (5, 2)


def test_guide_tree_families():
    ps = W.guide_tree_families()
    n = ps.meta["n_seqs"]
    assert n == 20 * 200 and len(ps) == n * (n - 1) // 2 == 7_998_000
    assert ps.cells == 1_728_690_192_088


def test_serving_stream():
    reqs = W.serving_stream(120, 1.0, seed=5)
    assert len(reqs) == 120
    assert sum(len(r.pairs) for r in reqs) == 33_707
    assert sum(r.pairs.cells for r in reqs) == 89_981_887_391
    assert sum(r.traceback for r in reqs) == 69 and sum(r.pairs.matrix == W.DNA for r in reqs) == 65
    sizes = [len(r.pairs) for r in reqs]
    assert min(sizes) >= 1 and max(sizes) <= 2000
    arrivals = [r.arrival_s for r in reqs]
    assert all(b > a for a, b in zip(arrivals, arrivals[1:]))
