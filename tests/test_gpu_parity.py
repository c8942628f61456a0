"""GPU parity: the CUDA library, called through its C ABI, against the CPU
oracle on the same seeded inputs.  Integer work, so the bar is bit-exact:
scores, coordinates, identity counts and both gapped strings."""
import ctypes
import dataclasses
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tweakseq_gb300 import _native as N
from tweakseq_gb300 import aligner as A
from tweakseq_gb300 import build as B
from tweakseq_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols")


@pytest.fixture(scope="module", autouse=True)
def built():
    B.build()
    O.build()
    N.lib()


def oracle_batch(ps, local, mode, strings=False, nthreads=0):
    return O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, ps.matrix, ps.gap_open, ps.gap_extend, local,
                   mode, nthreads, strings)


def gpu_batch(ps, local, output, **kw):
    return A.align_batch(ps, matrix=ps.matrix, gap_open=ps.gap_open, gap_extend=ps.gap_extend,
                         mode="local" if local else "global", output=output, **kw)


def assert_same(got, want, fields, what):
    for f in fields:
        bad = np.flatnonzero(got.table[f] != want[f])
        assert len(bad) == 0, f"{what}: field {f} differs at pairs {bad[:10].tolist()} " \
                              f"(gpu {got.table[f][bad[:3]].tolist()} vs oracle {want[f][bad[:3]].tolist()})"


def score_fields(local):
    return ("score", "a_end", "b_end") if local else ("score",)


def ident_fields(local):
    return ("score", "a_end", "b_end", "n_ident", "n_cols") if local else ("score", "n_ident", "n_cols")


def test_golden_cases_plain_path():
    cases = json.load(open(os.path.join(GOLDEN, "oracle_cases.json")))
    for c in cases:
        r = A.align_pair(c["a"], c["b"], matrix=c["matrix"], gap_open=c["gap_open"], gap_extend=c["gap_extend"],
                         mode="local" if c["local"] else "global", output="alignment")
        got = (r.score, r.a_begin, r.a_end, r.b_begin, r.b_end, r.n_ident, r.n_cols, r.aln_a, r.aln_b)
        want = tuple(c[k] for k in FIELDS + ("aln_a", "aln_b"))
        assert got == want, c["name"]
        s = A.align_pair(c["a"], c["b"], matrix=c["matrix"], gap_open=c["gap_open"], gap_extend=c["gap_extend"],
                         mode="local" if c["local"] else "global", output="score")
        assert s.score == c["score"], c["name"]
        i = A.align_pair(c["a"], c["b"], matrix=c["matrix"], gap_open=c["gap_open"], gap_extend=c["gap_extend"],
                         mode="local" if c["local"] else "global", output="identity")
        assert (i.score, i.n_ident, i.n_cols) == (c["score"], c["n_ident"], c["n_cols"]), c["name"]


def random_pairs(seed, n, lo, hi, dna=False, related=0.5):
    rng = np.random.default_rng(seed)
    seqs, pairs = [], []
    for k in range(n):
        m = int(rng.integers(lo, hi + 1))
        if dna:
            a = W.DNA_LETTERS[rng.integers(0, 4, m)]
        else:
            a = W.random_protein(rng, m)
        if rng.random() < related and m > 0:
            if dna:
                b = W._mutate_dna(rng, a, 0.1, 0.02, 3.0)
            else:
                b, _ = W._mutate_proteins(rng, a, np.array([m]), np.array([0.5]), 0.05)
        else:
            nn = int(rng.integers(lo, hi + 1))
            b = W.DNA_LETTERS[rng.integers(0, 4, nn)] if dna else W.random_protein(rng, nn)
        seqs += [a.tobytes(), b.tobytes()]
        pairs.append((2 * k, 2 * k + 1))
    kw = dict(matrix=W.DNA, gap_open=5, gap_extend=2) if dna else {}
    return W._pairset_from_lists(seqs, pairs, **kw)


@pytest.mark.parametrize("local", [False, True])
@pytest.mark.parametrize("output", ["score", "identity", "alignment"])
def test_random_uneven_protein(local, output):
    ps = random_pairs(100 + local, 600, 0, 700)
    got = gpu_batch(ps, local, output)
    if output == "alignment":
        want, sa, sb = oracle_batch(ps, local, O.MODE_ALIGN, strings=True)
        assert_same(got, want, FIELDS, "alignment")
        assert got.aln_a == sa and got.aln_b == sb
    elif output == "identity":
        want = oracle_batch(ps, local, O.MODE_IDENT)
        assert_same(got, want, ident_fields(local), "identity")
    else:
        want = oracle_batch(ps, local, O.MODE_SCORE)
        assert_same(got, want, score_fields(local), "score")


@pytest.mark.parametrize("local", [False, True])
def test_low_complexity_ties(local):
    """Homopolymers and short repeats create many equal-score paths: the
    tie-breaks decide every traceback."""
    seqs, pairs = [], []
    motifs = [b"A", b"AG", b"GGA", b"W", b"KR", b"ACGT"]
    rng = np.random.default_rng(9)
    for k in range(120):
        ma, mb = motifs[k % len(motifs)], motifs[(k // 3) % len(motifs)]
        a = (ma * 400)[: int(rng.integers(1, 300))]
        b = (mb * 400)[: int(rng.integers(1, 300))]
        seqs += [a, b]
        pairs.append((2 * k, 2 * k + 1))
    for gaps in ((11, 1), (0, 1), (3, 0)):
        ps = W._pairset_from_lists(seqs, pairs, gap_open=gaps[0], gap_extend=gaps[1])
        got = gpu_batch(ps, local, "alignment")
        want, sa, sb = oracle_batch(ps, local, O.MODE_ALIGN, strings=True)
        assert_same(got, want, FIELDS, f"ties {gaps}")
        assert got.aln_a == sa and got.aln_b == sb


def test_all_vs_all_64_proteins_alignment():
    """64 proteins (lengths 200-400, seed 1), all 2,016 global pairs with
    full traceback: scores, strings and identity bit-exact."""
    ps = W.all_vs_all_proteins()
    got = gpu_batch(ps, False, "alignment")
    want, sa, sb = oracle_batch(ps, False, O.MODE_ALIGN, strings=True)
    assert_same(got, want, FIELDS, "c1")
    assert got.aln_a == sa and got.aln_b == sb


def test_uneven_pairs_score_full():
    """All 100,000 uneven pairs (log-normal lengths 50-2,000), score only."""
    ps = W.uneven_pairs()
    got = gpu_batch(ps, False, "score")
    want = oracle_batch(ps, False, O.MODE_SCORE)
    assert_same(got, want, ("score",), "c2")


def test_dna_long_traceback():
    ps = random_pairs(7, 6, 1500, 4000, dna=True, related=1.0)
    for local in (False, True):
        got = gpu_batch(ps, local, "alignment")
        want, sa, sb = oracle_batch(ps, local, O.MODE_ALIGN, strings=True)
        assert_same(got, want, FIELDS, "dna")
        assert got.aln_a == sa and got.aln_b == sb


def test_guide_tree_identity_sample():
    ps = W.guide_tree_families(n_families=3, per_family=30)
    got = gpu_batch(ps, False, "identity")
    want = oracle_batch(ps, False, O.MODE_IDENT)
    assert_same(got, want, ("score", "n_ident", "n_cols"), "c4 sample")


def test_invalid_residues_reported_per_pair():
    seqs = [b"ACDEFG", b"ACDXFG", b"acdefg", b"ACD", b"AC-DE", b"", b"A1"]
    pairs = [(0, 1), (0, 2), (3, 0), (4, 3), (5, 6), (5, 0)]
    ps = W._pairset_from_lists(seqs, pairs)
    with pytest.raises(N.TsqError) as e:
        gpu_batch(ps, False, "alignment")
    assert e.value.rc == N.E_INVALID_RESIDUE
    got = gpu_batch(ps, False, "alignment", check=False)
    assert got.table["status"].tolist() == [0, -2, 0, -2, -2, 0]
    ok = [0, 2, 5]
    want, sa, sb = oracle_batch(ps.subset(ok), False, O.MODE_ALIGN, strings=True)
    for j, k in enumerate(ok):
        assert got.table["score"][k] == want["score"][j] and got.aln_a[k] == sa[j] and got.aln_b[k] == sb[j]
    with pytest.raises(N.TsqError) as e:
        A.align_pair(b"ACGE", b"ACGT", matrix="dna", gap_open=5, gap_extend=2)
    assert e.value.rc == N.E_INVALID_RESIDUE


@pytest.mark.parametrize("local,lane", [(False, "auto"), (True, "auto"), (False, "i16")])
def test_invalid_residues_in_score_batches(local, lane):
    """Score batches (the int16x2 fill) with invalid bytes planted in some
    pairs (lowercase, '*', '-', digits, bytes >= 0x80, NUL): exactly those
    pairs report TSQ_E_INVALID_RESIDUE, every other score equals the
    oracle's, including pairs whose neighbours in the residue buffer are
    invalid."""
    ps = W.uneven_pairs(n_pairs=3000, seed=21)
    seqs = ps.seqs.copy()
    rng = np.random.default_rng(22)
    planted = rng.choice(len(ps), 300, replace=False)
    junk = np.frombuffer(b"ac*-0\x80\xff\x00z", dtype=np.uint8)
    for k in planted:
        off, ln = (ps.a_off[k], ps.a_len[k]) if k % 2 else (ps.b_off[k], ps.b_len[k])
        seqs[off + rng.integers(ln)] = junk[k % len(junk)]
    bad = dataclasses.replace(ps, seqs=seqs)
    got = gpu_batch(bad, local, "score", lane=lane, check=False)
    is_bad = np.zeros(len(ps), dtype=bool)
    is_bad[planted] = True
    assert np.array_equal(got.table["status"] == N.E_INVALID_RESIDUE, is_bad)
    ok = np.flatnonzero(~is_bad)
    want = oracle_batch(bad.subset(ok), local, O.MODE_SCORE)
    assert np.array_equal(got.table["score"][ok], want["score"])
    # DNA: protein letters are invalid there.
    dna = W.long_dna_pairs(6, lo=300, hi=600)
    dseqs = dna.seqs.copy()
    dseqs[dna.a_off[2] + 5] = ord("E")
    dbad = dataclasses.replace(dna, seqs=dseqs)
    got = gpu_batch(dbad, local, "score", lane=lane, check=False)
    assert got.table["status"].tolist() == [0, 0, N.E_INVALID_RESIDUE, 0, 0, 0]
    keep = np.array([0, 1, 3, 4, 5])
    want = oracle_batch(dbad.subset(keep), local, O.MODE_SCORE)
    assert np.array_equal(got.table["score"][keep], want["score"])


def test_bad_arguments_rejected():
    with pytest.raises(N.TsqError) as e:
        A.align_pair(b"ACD", b"ACD", gap_open=-1)
    assert e.value.rc == N.E_INVALID_ARG
    ps = W._pairset_from_lists([b"ACD", b"ACD"], [(0, 1)])
    ps.a_off = ps.a_off + 5  # out of the residue buffer
    with pytest.raises(N.TsqError) as e:
        gpu_batch(ps, False, "score")
    assert e.value.rc == N.E_INVALID_ARG


def test_custom_matrix_asymmetric():
    rng = np.random.default_rng(3)
    mat = rng.integers(-6, 9, size=(26, 26)).astype(np.int8)
    valid = np.ones(26, np.uint8)
    valid[ord("Z") - 65] = 0
    ps = random_pairs(11, 80, 1, 200)
    for local in (False, True):
        got = A.align_batch(ps, custom=(mat, valid), gap_open=4, gap_extend=2,
                            mode="local" if local else "global", output="alignment")
        want, sa, sb = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, (mat, valid), 4, 2, local,
                               O.MODE_ALIGN, 0, True)
        assert_same(got, want, FIELDS, "custom")
        assert got.aln_a == sa and got.aln_b == sb
    # Long pairs over all 25 valid letters: 25 score classes, whose profile
    # takes the 8-warp variant of the int16x2 CTA fill.
    letters = np.frombuffer(bytes(c for c in range(65, 91) if c != ord("Z")), dtype=np.uint8)
    seqs = [letters[rng.integers(0, len(letters), L)].tobytes() for L in (9000, 8000, 12000, 700)]
    ps = W._pairset_from_lists(seqs, [(0, 1), (2, 3)])
    for output, omode in (("score", O.MODE_SCORE), ("alignment", O.MODE_ALIGN)):
        got = A.align_batch(ps, custom=(mat, valid), gap_open=4, gap_extend=2, output=output)
        want = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, (mat, valid), 4, 2, False, omode, 0,
                       omode == O.MODE_ALIGN)
        if omode == O.MODE_ALIGN:
            want, sa, sb = want
            assert got.aln_a == sa and got.aln_b == sb
        assert_same(got, want, FIELDS if omode == O.MODE_ALIGN else ("score",), f"custom long {output}")


def test_graph_replay_and_device_resident_batch():
    ps = random_pairs(5, 3000, 20, 500)
    want = oracle_batch(ps, False, O.MODE_SCORE)
    with A.Batch(ps, output="score", use_graph=True) as b:
        for _ in range(3):
            b.run()
            got = b.results()
            assert_same(got, want, ("score",), "graph replay")
        st = b.stats()
        assert st["cells"] == ps.cells and st["pairs"] == len(ps) and st["device_ms"] > 0


def test_plain_equals_batch():
    ps = random_pairs(21, 40, 0, 900)
    bat = gpu_batch(ps, True, "alignment")
    for k in range(len(ps)):
        a, b = ps.pair(k)
        r = A.align_pair(a, b, mode="local", output="alignment")
        assert (r.score, r.aln_a, r.aln_b, r.a_begin, r.b_begin) == (
            int(bat.table["score"][k]), bat.aln_a[k], bat.aln_b[k], int(bat.table["a_begin"][k]),
            int(bat.table["b_begin"][k]))


@pytest.mark.parametrize("output", ["score", "identity", "alignment"])
def test_one_pair_path_every_kind(output):
    """tsq_align_pair's one-pair path against the oracle, on every kind of
    pair it runs: empty sequences, int16x2 warp tasks, int32 warp tasks, the
    CTA fill (long int32 pairs, among them W:W pairs past the proven int16
    range, which it runs in int32 at once) and, with lane 'i16', the calls it
    leaves to the batch engine.  Calls in a row reuse its buffers: sizes go
    up and down."""
    rng = np.random.default_rng(41)

    def prot(n):
        return W.random_protein(rng, n).tobytes()

    cases = [(b"", prot(30)), (prot(25), b""), (b"", b""), (prot(1), prot(1)), (prot(300), prot(500)),
             (prot(900), prot(40)), (b"W" * 2900, b"W" * 2900), (b"W" * 3100, b"W" * 3100),
             (prot(3000), prot(2600)), (prot(64), prot(70)), (prot(600), prot(500)), (prot(1100), prot(900))]
    seqs, pairs = [], []
    for a, b in cases:
        seqs += [a, b]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    ps = W._pairset_from_lists(seqs, pairs)
    omode = {"score": O.MODE_SCORE, "identity": O.MODE_IDENT, "alignment": O.MODE_ALIGN}[output]
    for local in (False, True):
        mode = "local" if local else "global"
        if output == "alignment":
            want, sa, sb = oracle_batch(ps, local, omode, strings=True)
            fields = FIELDS
        else:
            want = oracle_batch(ps, local, omode)
            fields = score_fields(local) if output == "score" else ident_fields(local)
        for lane in ("auto", "i32", "i16"):
            for k, (a, b) in enumerate(cases):
                r = A.align_pair(a, b, mode=mode, output=output, lane=lane)
                got = tuple(getattr(r, f) for f in fields)
                exp = tuple(int(want[f][k]) for f in fields)
                assert got == exp, (output, mode, lane, k, len(a), len(b))
                if output == "alignment":
                    assert (r.aln_a, r.aln_b) == (sa[k], sb[k]), (mode, lane, k)


@pytest.mark.parametrize("local", [False, True])
def test_int16_overflow_rerun_and_lane_choices(local):
    """Scores beyond int16: the checked int16x2 fill flags them and the int32
    re-run makes them exact; pairs at the edge of the proven range stay in
    int16x2; lane='i16' forces the checked kernel on every pair and
    lane='i32' the int32 kernel."""
    rng = np.random.default_rng(31)
    seqs, pairs = [], []
    for L in (2900, 2978, 2979, 3100, 3500):  # W:W scores 11 per residue
        seqs += [b"W" * L, b"W" * L]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    for k in range(40):  # ordinary pairs mixed in
        a = W.random_protein(rng, int(rng.integers(20, 900))).tobytes()
        b = W.random_protein(rng, int(rng.integers(20, 900))).tobytes()
        seqs += [a, b]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    ps = W._pairset_from_lists(seqs, pairs)
    want = oracle_batch(ps, local, O.MODE_SCORE)
    mode = "local" if local else "global"
    for lane in ("auto", "i16", "i32"):
        got = A.align_batch(ps, mode=mode, output="score", lane=lane)
        assert_same(got, want, score_fields(local), f"lane {lane}")
    # (Lane auto sends the 3,100 and 3,500-residue pairs to the CTA fill in
    # int32; lane i16 keeps them on the checked int16x2 kernel.)
    with A.Batch(ps, mode=mode, output="score", lane="i16") as b:
        b.run()
        assert_same(b.results(), want, score_fields(local), "batch")
        assert b.stats()["rerun_pairs"] >= 3  # 2979, 3100 and 3500 overflow (2978 is flagged too)


def _overflow_edge_pairs(seed, n_random, hi):
    """W:W homopolymers around the int16 edge (W scores 11 per residue, so
    2978 residues is the longest proven pair) plus ordinary random pairs."""
    rng = np.random.default_rng(seed)
    seqs, pairs = [], []
    for L in (2900, 2978, 2979, 3100):
        seqs += [b"W" * L, b"W" * L]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    for k in range(n_random):
        a = W.random_protein(rng, int(rng.integers(1, hi))).tobytes()
        b = W.random_protein(rng, int(rng.integers(1, hi))).tobytes()
        seqs += [a, b]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    return W._pairset_from_lists(seqs, pairs)


@pytest.mark.parametrize("output,local", [("alignment", False), ("alignment", True), ("identity", False)])
def test_int16_traceback_and_identity_fills_at_the_overflow_edge(output, local):
    """The int16x2 traceback and identity fills: pairs past the proven int16
    range are flagged by the checked kernel and re-run in int32 (planes and
    counts rewritten), pairs at the edge stay in int16x2; every lane choice
    gives the oracle's scores, counts and strings."""
    ps = _overflow_edge_pairs(37, 40, 900)
    mode = "local" if local else "global"
    if output == "alignment":
        want, sa, sb = oracle_batch(ps, local, O.MODE_ALIGN, strings=True)
        fields = FIELDS
    else:
        want, sa, sb = oracle_batch(ps, local, O.MODE_IDENT), None, None
        fields = ident_fields(local)
    for lane in ("auto", "i16", "i32"):
        got = A.align_batch(ps, mode=mode, output=output, lane=lane)
        assert_same(got, want, fields, f"{output} lane {lane}")
        if sa is not None:
            assert got.aln_a == sa and got.aln_b == sb, f"strings, lane {lane}"
    with A.Batch(ps, mode=mode, output=output, lane="i16") as b:
        b.run()
        assert_same(b.results(), want, fields, "batch")
        assert b.stats()["rerun_pairs"] >= 2  # 2979 and 3100 overflow


@pytest.mark.parametrize("dna", [False, True])
def test_int16_and_int32_lanes_agree_all_outputs(dna):
    """Uneven pairs (proteins, or DNA at +2/-3) through the int16x2 fills
    (lane auto) and the int32 fills (lane i32): both equal the oracle for
    every output, global and local, including open 0 and extend 0 gaps."""
    ps = random_pairs(53 + dna, 300, 0, 1200 if dna else 700, dna=dna)
    gap_sets = ((ps.gap_open, ps.gap_extend), (0, 2), (4, 0))
    for go, ge in gap_sets:
        q = dataclasses.replace(ps, gap_open=go, gap_extend=ge)
        for local in (False, True):
            want, sa, sb = oracle_batch(q, local, O.MODE_ALIGN, strings=True)
            wid = oracle_batch(q, local, O.MODE_IDENT)
            for lane in ("auto", "i32"):
                got = gpu_batch(q, local, "alignment", lane=lane)
                assert_same(got, want, FIELDS, f"alignment gaps {go}/{ge} local {local} lane {lane}")
                assert got.aln_a == sa and got.aln_b == sb, f"strings gaps {go}/{ge} local {local} lane {lane}"
                gi = gpu_batch(q, local, "identity", lane=lane)
                assert_same(gi, wid, ident_fields(local), f"identity gaps {go}/{ge} local {local} lane {lane}")


def test_identity_counts_letters_sharing_a_score_class():
    """J, O, U and X score alike under BLOSUM62 (one score class) but are
    different letters: the identity fill counts only equal letters."""
    rng = np.random.default_rng(77)
    alpha = np.frombuffer(b"JOUXBZ" + b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
    seqs, pairs = [], []
    for k in range(200):
        a = alpha[rng.integers(0, 8 if k % 2 else len(alpha), int(rng.integers(1, 400)))]
        b = a.copy()
        flip = rng.random(len(b)) < 0.3
        b[flip] = alpha[rng.integers(0, 6, int(flip.sum()))]
        seqs += [a.tobytes(), b.tobytes()]
        pairs.append((2 * k, 2 * k + 1))
    ps = W._pairset_from_lists(seqs, pairs)
    want = oracle_batch(ps, False, O.MODE_IDENT)
    for lane in ("auto", "i16", "i32"):
        got = gpu_batch(ps, False, "identity", lane=lane)
        assert_same(got, want, ident_fields(False), f"identity lane {lane}")
    want_a, sa, sb = oracle_batch(ps, False, O.MODE_ALIGN, strings=True)
    got = gpu_batch(ps, False, "alignment")
    assert_same(got, want_a, FIELDS, "alignment")
    assert got.aln_a == sa and got.aln_b == sb


def test_mixed_lane_types_one_batch():
    """One batch whose pairs split over int16x2, checked int16x2 and int32:
    with extend 60 the lower bound only fits int16 for short pairs."""
    ps = random_pairs(41, 300, 5, 700)
    for local in (False, True):
        got = A.align_batch(ps, gap_open=20, gap_extend=60, mode="local" if local else "global", output="score")
        want = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, O.BLOSUM62, 20, 60, local, O.MODE_SCORE)
        assert_same(got, want, score_fields(local), "mixed")


@pytest.mark.parametrize("local", [False, True])
def test_long_pairs_on_the_cta_fill_all_outputs(local):
    """Pairs long enough for the CTA fill (bands striped over the warps of
    a CTA): 79, 12 and 3 bands (fewer bands than warps), long rows and long
    columns, score / identity / alignment, against the oracle."""
    rng = np.random.default_rng(17 + local)
    seqs, pairs = [], []
    for m, n in ((20000, 3000), (3000, 20000), (2900, 2700), (700, 9000)):
        a = W.DNA_LETTERS[rng.integers(0, 4, m)]
        b = W._mutate_dna(rng, a, 0.1, 0.02, 3.0)[:n] if n <= m else W.DNA_LETTERS[rng.integers(0, 4, n)]
        if n > m:
            b[: m // 2] = a[: m // 2]  # related prefix so the alignment is not trivial
        seqs += [a.tobytes(), b.tobytes()]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    ps = W._pairset_from_lists(seqs, pairs, matrix=W.DNA, gap_open=5, gap_extend=2)
    want, sa, sb = oracle_batch(ps, local, O.MODE_ALIGN, strings=True)
    # lane auto: the 20 kb pairs (past the int16 range) on the CTA fill,
    # the others on int16x2 lanes; lane i32: all four on the CTA fill.
    for lane in ("auto", "i32"):
        got = gpu_batch(ps, local, "score", lane=lane)
        assert_same(got, oracle_batch(ps, local, O.MODE_SCORE), score_fields(local), f"cta score {lane}")
        got = gpu_batch(ps, local, "identity", lane=lane)
        assert_same(got, oracle_batch(ps, local, O.MODE_IDENT), ident_fields(local), f"cta identity {lane}")
        got = gpu_batch(ps, local, "alignment", lane=lane)
        assert_same(got, want, FIELDS, f"cta alignment {lane}")
        assert got.aln_a == sa and got.aln_b == sb
    # The plain form of a long pair takes the same path.
    a, b = ps.pair(2)
    r = A.align_pair(a, b, matrix="dna", gap_open=5, gap_extend=2, mode="local" if local else "global")
    assert (r.score, r.aln_a, r.aln_b) == (int(want["score"][2]), sa[2], sb[2])


@pytest.mark.parametrize("local", [False, True])
@pytest.mark.parametrize("output", ["score", "alignment"])
def test_int16_cta_fill_rebased_values(output, local):
    """Long pairs on the CTA fill in int16x2 lanes, whose values are kept
    relative to a moving base: scores far past the int16 range upwards
    (W:W, 176,000) and downwards, a 4,000-residue gap, a 40-column pair (no
    interior steps), 513 rows (a one-row second pass), 17 passes (the
    wrap-around row), BLOSUM62 (23 classes, 16 warps global, 8 local) and
    DNA, against the oracle; gap costs at the bound (open + ext + max score
    = 40) and past it (the int32 CTA fill).  Local mode: a 5,000-residue
    identical block followed by 12,000 unrelated residues (the maximum far
    behind the base when the fill ends).  The plain form of a long pair
    takes the same kernel."""
    rng = np.random.default_rng(61)

    def prot(n):
        return W.random_protein(rng, n).tobytes()

    big = prot(20000)
    block = prot(5000)
    prot_cases = [(b"W" * 16000, b"W" * 16000), (prot(16000), prot(15000)), (big, big[:8000] + big[12000:]),
                  (block + prot(12000), block + prot(12000)),
                  (prot(80000), prot(40)), (prot(200000), prot(1)), (prot(1), prot(30000)), (prot(512), prot(45000)),
                  (prot(513), prot(40000)), (prot(8193), prot(23000))]
    d = W.DNA_LETTERS[rng.integers(0, 4, 30000)]
    dna_cases = [(d.tobytes(), W._mutate_dna(rng, d, 0.05, 0.01, 3.0)[:29000].tobytes()),
                 (W.DNA_LETTERS[rng.integers(0, 4, 20000)].tobytes(),
                  W.DNA_LETTERS[rng.integers(0, 4, 20000)].tobytes())]
    omode = O.MODE_ALIGN if output == "alignment" else O.MODE_SCORE
    fields = FIELDS if output == "alignment" else score_fields(local)
    mode = "local" if local else "global"
    for cases, matrix, gaps in ((prot_cases, "blosum62", ((11, 1), (25, 4), (27, 4))),
                                (dna_cases, "dna", ((5, 2),))):
        seqs, pairs = [], []
        for a, b in cases:
            seqs += [a, b]
            pairs.append((len(seqs) - 2, len(seqs) - 1))
        ps = W._pairset_from_lists(seqs, pairs)
        which = O.DNA if matrix == "dna" else O.BLOSUM62
        for go, ge in gaps:
            want = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, which, go, ge, local, omode, 0,
                           output == "alignment")
            if output == "alignment":
                want, sa, sb = want
            got = A.align_batch(ps, matrix=matrix, gap_open=go, gap_extend=ge, mode=mode, output=output)
            assert_same(got, want, fields, f"{matrix} {go}/{ge} {mode}")
            if output == "alignment":
                assert got.aln_a == sa and got.aln_b == sb, f"{matrix} {go}/{ge} {mode}"
            r = A.align_pair(*ps.pair(len(ps) - 1), matrix=matrix, gap_open=go, gap_extend=ge, mode=mode,
                             output=output)
            assert r.score == int(want["score"][len(ps) - 1])
            if output == "alignment":
                assert (r.aln_a, r.aln_b) == (sa[-1], sb[-1])
    # An invalid residue in a long pair: that pair reports it, the others
    # of the launch are unaffected.
    bad = bytearray(big)
    bad[12345] = ord("*")
    ps = W._pairset_from_lists([bytes(bad), big[:15000], big, big[:15000]], [(0, 1), (2, 3)])
    got = A.align_batch(ps, mode=mode, output=output, check=False)
    assert got.table["status"].tolist() == [N.E_INVALID_RESIDUE, 0]
    want = O.batch(ps.seqs, ps.a_off[1:], ps.a_len[1:], ps.b_off[1:], ps.b_len[1:], O.BLOSUM62, 11, 1, local,
                   O.MODE_SCORE, 0, False)
    assert int(got.table["score"][1]) == int(want["score"][0])


def test_alignment_batch_in_waves(monkeypatch):
    """An alignment batch whose traceback planes exceed the memory budget
    runs in waves (largest pairs first); every result matches the
    single-wave run and the oracle."""
    rng = np.random.default_rng(31)
    seqs, pairs = [], []
    for k in range(24):
        a = W.DNA_LETTERS[rng.integers(0, 4, int(rng.integers(200, 3000)))]
        seqs += [a.tobytes(), W._mutate_dna(rng, a, 0.1, 0.02, 3.0).tobytes()]
        pairs.append((2 * k, 2 * k + 1))
    ps = W._pairset_from_lists(seqs, pairs, matrix=W.DNA, gap_open=5, gap_extend=2)
    kw = dict(matrix="dna", gap_open=5, gap_extend=2, output="alignment")
    whole = A.align_batch(ps, **kw)
    monkeypatch.setenv("TSQ_WAVE_BUDGET_BYTES", str(12 << 20))  # a few pairs per wave
    waved = A.align_batch(ps, **kw)
    for f in ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols", "status"):
        assert np.array_equal(whole.table[f], waved.table[f]), f
    assert whole.aln_a == waved.aln_a and whole.aln_b == waved.aln_b
    want, sa, sb = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, O.DNA, 5, 2, False, O.MODE_ALIGN, 0, True)
    assert waved.aln_a == sa and waved.aln_b == sb
    assert np.array_equal(waved.table["score"], want["score"])
    # A pair larger than the budget on its own is refused, the rest align.
    monkeypatch.setenv("TSQ_WAVE_BUDGET_BYTES", str(1 << 20))
    raw = np.zeros(len(ps), dtype=N.RESULT_DTYPE)
    seqs_arr, tab = A._as_inputs(ps)
    p, keep = N.make_params(**kw)
    rc = N.lib().tsq_align_batch(seqs_arr.ctypes.data, len(seqs_arr), tab.ctypes.data, len(tab), ctypes.byref(p),
                                 ctypes.byref(A._opts()), raw.ctypes.data)
    assert rc == N.E_TOO_LARGE
    a_len, b_len = ps.a_len.astype(np.int64), ps.b_len.astype(np.int64)
    big = (a_len + 255) * (b_len + 31) // 2 + 2 * (a_len + b_len) + 512 > (1 << 20)
    assert big.any() and (~big).any()
    assert np.all(raw["status"][big] == N.E_TOO_LARGE) and np.all(raw["status"][~big] == 0)
    N.lib().tsq_results_free(raw.ctypes.data, len(raw))


@pytest.mark.parametrize("output,local", [("score", False), ("identity", False), ("score", True)])
def test_chunked_call_equals_single_plan(output, local):
    """A large score or identity call through tsq_align_batch runs in chunks
    planned while earlier chunks run; every result equals the single-plan
    device-resident batch's, and a sample equals the oracle's."""
    ps = W.uneven_pairs(n_pairs=40000, seed=12)
    mode = "local" if local else "global"
    got = A.align_batch(ps, output=output, mode=mode)
    with A.Batch(ps, output=output, mode=mode, use_graph=False) as b:
        b.run()
        want = b.results()
    for f in ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols", "status"):
        assert np.array_equal(got.table[f], want.table[f]), f
    idx = np.random.default_rng(5).choice(len(ps), 300, replace=False)
    sub = ps.subset(idx)
    o = O.batch(sub.seqs, sub.a_off, sub.a_len, sub.b_off, sub.b_len, O.BLOSUM62, 11, 1, local,
                O.MODE_IDENT if output == "identity" else O.MODE_SCORE)
    assert np.array_equal(got.table["score"][idx], o["score"])
    if output == "identity":
        assert np.array_equal(got.table["n_ident"][idx], o["n_ident"])
        assert np.array_equal(got.table["n_cols"][idx], o["n_cols"])
    if local:
        assert np.array_equal(got.table["a_end"][idx], o["a_end"])
        assert np.array_equal(got.table["b_end"][idx], o["b_end"])


def _call_batch(seqs_ptr, seqs_len, tab, output="score", mode="global"):
    raw = np.zeros(len(tab), dtype=N.RESULT_DTYPE)
    p, keep = N.make_params(output=output, mode=mode)
    rc = N.lib().tsq_align_batch(seqs_ptr, seqs_len, tab.ctypes.data, len(tab), ctypes.byref(p),
                                 ctypes.byref(A._opts()), raw.ctypes.data)
    return rc, raw


@pytest.mark.parametrize("output,mode", [("score", "global"), ("identity", "global"), ("score", "local")])
def test_chunked_call_page_locked_input(output, mode):
    """Page-locked residues are encoded in place and the chunks are cut by
    cost; the results equal those of the same call on pageable memory
    (chunks of consecutive pairs), including empty pairs and a pair with an
    invalid residue, and a sample equals the oracle."""
    torch = pytest.importorskip("torch")
    ps = W.uneven_pairs(n_pairs=40000, seed=14)
    seqs, tab = A._as_inputs(ps)
    seqs, tab = seqs.copy(), tab.copy()
    seqs[int(tab["a_off"][35000]) + 3] = ord("#")
    tab["a_len"][100] = 0
    tab["b_len"][20000] = 0
    pinned = torch.from_numpy(seqs).pin_memory()
    rc_p, got = _call_batch(pinned.data_ptr(), len(seqs), tab, output, mode)
    rc_h, want = _call_batch(seqs.ctypes.data, len(seqs), tab, output, mode)
    assert rc_p == rc_h == N.E_INVALID_RESIDUE
    assert got["status"][35000] == N.E_INVALID_RESIDUE
    for f in ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols", "status"):
        assert np.array_equal(got[f], want[f]), f
    idx = np.random.default_rng(7).choice(len(tab), 200, replace=False)
    idx = idx[idx != 35000]
    o = O.batch(seqs, tab["a_off"][idx], tab["a_len"][idx], tab["b_off"][idx], tab["b_len"][idx], O.BLOSUM62, 11, 1,
                mode == "local", O.MODE_IDENT if output == "identity" else O.MODE_SCORE)
    assert np.array_equal(got["score"][idx], o["score"])
    bad = tab.copy()
    bad["b_len"][39000] = -1
    rc, _ = _call_batch(pinned.data_ptr(), len(seqs), bad, output, mode)
    assert rc == N.E_INVALID_ARG
    rc, again = _call_batch(pinned.data_ptr(), len(seqs), tab, output, mode)
    assert rc == N.E_INVALID_RESIDUE and np.array_equal(again["score"], want["score"])


def test_chunked_call_reports_the_first_bad_pair():
    ps = W.uneven_pairs(n_pairs=40000, seed=13)
    seqs, tab = A._as_inputs(ps)
    tab = tab.copy()
    tab["a_len"][30000] = -1  # in the third chunk
    raw = np.zeros(len(tab), dtype=N.RESULT_DTYPE)
    p, keep = N.make_params(output="score")
    rc = N.lib().tsq_align_batch(seqs.ctypes.data, len(seqs), tab.ctypes.data, len(tab), ctypes.byref(p),
                                 ctypes.byref(A._opts()), raw.ctypes.data)
    assert rc == N.E_INVALID_ARG
    # The engines are usable again afterwards.
    ok = A.align_batch(ps.subset(np.arange(40000)), output="score")
    assert (ok.table["status"] == 0).all()


@pytest.mark.parametrize("output", ["alignment", "score"])
def test_cta_wait_runs_out_then_engine_recovers(output):
    """The long-pair fill's warps wait on one another with bounded polls.
    With the limit set to a single poll the waits run out: the kernel still
    returns, the long pair reports TSQ_E_TIMEOUT, the short pairs of the
    same call (warp-per-pair fills) are unaffected, and the next call on the
    same cached engine, with the default limit, is bit-exact."""
    rng = np.random.default_rng(57)
    seqs, pairs = [], []
    a = W.DNA_LETTERS[rng.integers(0, 4, 20000)]
    seqs += [a.tobytes(), W._mutate_dna(rng, a, 0.1, 0.02, 3.0)[:3000].tobytes()]
    pairs.append((0, 1))
    for k in range(30):
        x = W.DNA_LETTERS[rng.integers(0, 4, int(rng.integers(50, 400)))]
        seqs += [x.tobytes(), W._mutate_dna(rng, x, 0.1, 0.02, 3.0).tobytes()]
        pairs.append((len(seqs) - 2, len(seqs) - 1))
    ps = W._pairset_from_lists(seqs, pairs, matrix=W.DNA, gap_open=5, gap_extend=2)
    kw = dict(matrix="dna", gap_open=5, gap_extend=2, output=output)
    mode = O.MODE_ALIGN if output == "alignment" else O.MODE_SCORE
    want = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, O.DNA, 5, 2, False, mode, 0, mode == O.MODE_ALIGN)
    if mode == O.MODE_ALIGN:
        want, sa, sb = want
    with pytest.raises(N.TsqError) as e:
        A.align_batch(ps, wait_polls=1, **kw)
    assert e.value.rc == N.E_TIMEOUT
    got = A.align_batch(ps, wait_polls=1, check=False, **kw)
    assert got.table["status"][0] == N.E_TIMEOUT
    assert (got.table["status"][1:] == 0).all()
    assert np.array_equal(got.table["score"][1:], want["score"][1:])
    # The same engine, default limit: every pair bit-exact.
    got = A.align_batch(ps, **kw)
    assert (got.table["status"] == 0).all()
    assert np.array_equal(got.table["score"], want["score"])
    if mode == O.MODE_ALIGN:
        assert got.aln_a == sa and got.aln_b == sb
    # A device-resident batch with a short limit times out on every run and
    # keeps running.
    with A.Batch(ps, use_graph=False, wait_polls=1, **kw) as b:
        for _ in range(2):
            b.run()
            r = b.results(check=False)
            assert r.table["status"][0] == N.E_TIMEOUT and (r.table["status"][1:] == 0).all()
