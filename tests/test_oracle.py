"""CPU tests of the oracle itself: known answers, self-consistency, and the
scoring data pinned to the reference's BLOSUM62 (Consensus.cpp:34-69)."""
import itertools
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tweakseq_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rescore(aln_a: str, aln_b: str, mat, go: int, ge: int) -> int:
    """Score of a gapped pair under the affine model: each maximal run of
    '-' in one row costs go + len*ge."""
    s = 0
    for x, y in zip(aln_a, aln_b):
        assert not (x == "-" and y == "-")
        if x != "-" and y != "-":
            s += int(mat[ord(x) - 65][ord(y) - 65])
    for row in (aln_a, aln_b):
        k = 0
        while k < len(row):
            if row[k] == "-":
                j = k
                while j < len(row) and row[j] == "-":
                    j += 1
                s -= go + (j - k) * ge
                k = j
            else:
                k += 1
    return s


def test_blosum62_matches_reference_fixture():
    ref = json.load(open(os.path.join(GOLDEN, "blosum62_reference.json")))
    assert ref["order"] == "ARNDCQEGHILKMFPSTWYVBZX"
    mat, valid = O.scheme_arrays(O.BLOSUM62)
    assert valid.all()
    lm = ref["letter_map"]
    for x in range(26):
        for y in range(26):
            assert mat[x][y] == ref["matrix"][lm[x]][lm[y]], (chr(65 + x), chr(65 + y))


def test_dna_scheme():
    mat, valid = O.scheme_arrays(O.DNA)
    assert "".join(chr(65 + k) for k in range(26) if valid[k]) == "ABCDGHKMNRSTUVWY"
    for c in "ACGTU":
        assert mat[ord(c) - 65][ord(c) - 65] == 2
    assert mat[ord("N") - 65][ord("N") - 65] == -3
    assert mat[ord("T") - 65][ord("U") - 65] == -3


@pytest.mark.parametrize("local", [False, True])
def test_known_answers(local):
    # Hand-computed: BLOSUM62, open 11 / extend 1 (a single gap costs 12).
    r = O.align(b"", b"", local=local)
    assert (r.score, r.aln_a, r.aln_b, r.n_cols) == (0, "", "", 0)
    r = O.align(b"", b"ACD", local=local)
    assert r.score == (0 if local else -14)
    if not local:
        assert (r.aln_a, r.aln_b, r.n_cols, r.n_ident) == ("---", "ACD", 3, 0)
    r = O.align(b"W", b"W", local=local)
    assert (r.score, r.aln_a, r.aln_b, r.n_ident) == (11, "W", "W", 1)
    r = O.align(b"W", b"P", local=local)  # s(W,P) = -4
    assert r.score == (0 if local else -4)
    if local:
        assert (r.aln_a, r.n_cols, r.a_begin, r.a_end) == ("", 0, 0, 0)
    # One gap of two (-13) beats two gaps of one (-24): 8 - 13 = -5.
    r = O.align(b"AAAA", b"AA")
    assert r.score == -5 and r.aln_b.count("-") == 2 and "--" in r.aln_b
    # Diagonal wins ties at the end cell: the two A's pair at the right end.
    assert r.aln_a == "AAAA" and r.aln_b == "--AA"
    # HEAGAWGHEE / PAWHEAE: global 1 (gap of 3 = -14, then 15); local AWGHE-like core.
    assert O.align(b"HEAGAWGHEE", b"PAWHEAE").score == 1
    r = O.align(b"HEAGAWGHEE", b"PAWHEAE", local=True)
    assert r.score == 17 and rescore(r.aln_a, r.aln_b, O.scheme_arrays()[0], 11, 1) == 17
    # DNA +2/-3, gap 5/2: global 7 matches (14) and one gap (-7) = 7; local
    # keeps only the gap-free ACGT block (8).
    r = O.align(b"ACGTACGT", b"ACGACGT", O.DNA, 5, 2, local)
    assert r.score == (8 if local else 7)


def test_invalid_residues_rejected():
    for bad in (b"acgt", b"AC-GT", b"AC*", b"A1"):
        with pytest.raises(O.OracleError) as e:
            O.align(bad, b"ACGT")
        assert e.value.rc == -2
    with pytest.raises(O.OracleError):
        O.align(b"ACGE", b"ACGT", O.DNA, 5, 2)  # E is not a nucleotide code


def _all_alignments(a: str, b: str):
    """Every global alignment of a and b as (aln_a, aln_b)."""
    if not a and not b:
        yield "", ""
        return
    if a and b:
        for x, y in _all_alignments(a[:-1], b[:-1]):
            yield x + a[-1], y + b[-1]
    if a:
        for x, y in _all_alignments(a[:-1], b):
            yield x + a[-1], y + "-"
    if b:
        for x, y in _all_alignments(a, b[:-1]):
            yield x + "-", y + b[-1]


@pytest.mark.parametrize("seed", range(6))
def test_exhaustive_small(seed):
    """Brute force over every alignment (and every substring pair for local)
    agrees with the DP's score, for several gap settings."""
    rng = np.random.default_rng(seed)
    mat = O.scheme_arrays()[0]
    for _ in range(12):
        m, n = int(rng.integers(0, 5)), int(rng.integers(0, 5))
        a = W.random_protein(rng, m).tobytes().decode()
        b = W.random_protein(rng, n).tobytes().decode()
        go, ge = [(11, 1), (2, 1), (0, 1), (1, 3)][int(rng.integers(0, 4))]
        best_g = max(rescore(x, y, mat, go, ge) for x, y in _all_alignments(a, b))
        assert O.align(a, b, 0, go, ge).score == best_g
        best_l = 0
        for i0, i1 in itertools.combinations(range(m + 1), 2):
            for j0, j1 in itertools.combinations(range(n + 1), 2):
                for x, y in _all_alignments(a[i0:i1], b[j0:j1]):
                    best_l = max(best_l, rescore(x, y, mat, go, ge))
        assert O.align(a, b, 0, go, ge, True).score == best_l


@pytest.mark.parametrize("local", [False, True])
def test_self_consistency(local):
    rng = np.random.default_rng(7 + local)
    mat = O.scheme_arrays()[0]
    dmat = O.scheme_arrays(O.DNA)[0]
    for k in range(40):
        dna = k % 3 == 0
        m, n = int(rng.integers(0, 120)), int(rng.integers(0, 120))
        if dna:
            a = W.DNA_LETTERS[rng.integers(0, 4, m)].tobytes()
            b = W.DNA_LETTERS[rng.integers(0, 4, n)].tobytes()
            which, go, ge, M = O.DNA, 5, 2, dmat
        else:
            a = W.random_protein(rng, m).tobytes()
            b = W.random_protein(rng, n).tobytes()
            which, go, ge, M = O.BLOSUM62, 11, 1, mat
        r = O.align(a, b, which, go, ge, local)
        # The emitted strings are a valid alignment of the spans and rescore
        # to the reported score.
        assert len(r.aln_a) == len(r.aln_b) == r.n_cols
        assert r.aln_a.replace("-", "") == a[r.a_begin:r.a_end].decode()
        assert r.aln_b.replace("-", "") == b[r.b_begin:r.b_end].decode()
        assert rescore(r.aln_a, r.aln_b, M, go, ge) == r.score
        assert r.n_ident == sum(x == y and x != "-" for x, y in zip(r.aln_a, r.aln_b))
        if not local:
            assert (r.a_begin, r.a_end, r.b_begin, r.b_end) == (0, m, 0, n)
        # Swapping the inputs gives the same score (symmetric matrices).
        assert O.align(b, a, which, go, ge, local).score == r.score
        # Score-only and identity-carrying fills agree with the walk.
        s = O.score(a, b, which, go, ge, local)
        assert s.score == r.score
        si = O.score(a, b, which, go, ge, local, ident=True)
        assert (si.score, si.n_ident, si.n_cols) == (r.score, r.n_ident, r.n_cols)
        if local:
            assert (s.a_end, s.b_end) == (r.a_end, r.b_end)
        elif m >= 2:
            assert O.midpoint_score(a, b, which, go, ge) == r.score


def test_golden_cases_reproduce():
    cases = json.load(open(os.path.join(GOLDEN, "oracle_cases.json")))
    assert len(cases) >= 70
    for c in cases:
        r = O.align(c["a"].encode(), c["b"].encode(), c["matrix"], c["gap_open"], c["gap_extend"], c["local"])
        got = (r.score, r.a_begin, r.a_end, r.b_begin, r.b_end, r.n_ident, r.n_cols, r.aln_a, r.aln_b)
        want = tuple(c[k] for k in ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols", "aln_a",
                                    "aln_b"))
        assert got == want, c["name"]


def test_batch_matches_single_and_threads():
    ps = W.all_vs_all_proteins(n_seqs=12)
    out1 = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, mode=O.MODE_ALIGN, nthreads=1, strings=True)
    out4 = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, mode=O.MODE_ALIGN, nthreads=4, strings=True)
    assert (out1[0] == out4[0]).all() and out1[1] == out4[1] and out1[2] == out4[2]
    for k in range(len(ps)):
        a, b = ps.pair(k)
        r = O.align(a, b)
        assert (r.score, r.aln_a, r.aln_b) == (int(out1[0]["score"][k]), out1[1][k], out1[2][k])
    sc = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, mode=O.MODE_SCORE, nthreads=3)
    assert (sc["score"] == out1[0]["score"]).all()
    si = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, mode=O.MODE_IDENT, nthreads=3)
    assert (si["n_ident"] == out1[0]["n_ident"]).all() and (si["n_cols"] == out1[0]["n_cols"]).all()
