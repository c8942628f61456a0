"""GPU tests of the tsq_align command (the drop-in for the editor's external
aligner): gapped FASTA out for two sequences, identity table for
all-vs-all, both checked against the oracle."""
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tweakseq_gb300 import build as B
from tweakseq_gb300 import fasta as F
from tweakseq_gb300 import tool as T
from tweakseq_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    B.build()
    O.build()


def test_pairwise_fasta_round_trip(tmp_path):
    rng = np.random.default_rng(12)
    a = W.random_protein(rng, 230).tobytes().decode()
    b, _ = W._mutate_proteins(rng, np.frombuffer(a.encode(), np.uint8), np.array([230]), np.array([0.4]), 0.05)
    b = b.tobytes().decode()
    # The editor's export: existing insertions and lower case are allowed.
    exported = [F.Record(">seqA some description", "seqA", a[:50].lower() + "--" + a[50:]),
                F.Record(">seqB", "seqB", b[:30] + "..." + b[30:])]
    fin, fout = tmp_path / "in.fa", tmp_path / "out.fa"
    F.write(str(fin), exported)
    tool = T.GpuAlignmentTool()
    r = tool.align_files(str(fin), str(fout))
    assert r.returncode == 0, r.stderr
    recs = F.read(str(fout))
    assert [x.header for x in recs] == [">seqA some description", ">seqB"]
    want = O.align(a.encode(), b.encode())
    assert (recs[0].sequence, recs[1].sequence) == (want.aln_a, want.aln_b)
    assert all(len(line) <= 80 for line in fout.read_text().splitlines())
    # Local mode and DNA scoring through the same command.
    dna = [F.Record(">x", "x", "ACGTACGTTTGACCAACGT"), F.Record(">y", "y", "TTACGACGTTAGACNCA")]
    F.write(str(fin), dna)
    assert tool.align_files(str(fin), str(fout), local=True, dna=True).returncode == 0
    got = F.read(str(fout))
    want = O.align(b"ACGTACGTTTGACCAACGT", b"TTACGACGTTAGACNCA", O.DNA, 5, 2, True)
    _check_full_local_rows(got, "ACGTACGTTTGACCAACGT", "TTACGACGTTAGACNCA", want)


def _check_full_local_rows(recs, a, b, want):
    """Full-length local rows: equal length, each row without its gaps is
    its whole input sequence, and the columns between the flanks are the
    oracle's local alignment."""
    ra, rb = recs[0].sequence, recs[1].sequence
    assert len(ra) == len(rb)
    assert ra.replace("-", "") == a and rb.replace("-", "") == b
    lead = want.a_begin + want.b_begin
    assert ra[:lead] == a[:want.a_begin] + "-" * want.b_begin
    assert rb[:lead] == "-" * want.a_begin + b[:want.b_begin]
    assert ra[lead:lead + want.n_cols] == want.aln_a and rb[lead:lead + want.n_cols] == want.aln_b
    tail_a, tail_b = len(a) - want.a_end, len(b) - want.b_end
    assert ra[lead + want.n_cols:] == a[want.a_end:] + "-" * tail_b
    assert rb[lead + want.n_cols:] == "-" * tail_a + b[want.b_end:]
    assert len(ra) == lead + want.n_cols + tail_a + tail_b


def test_local_mode_keeps_whole_sequences(tmp_path):
    """The editor replaces each sequence with the row it reads back
    (Project::readNewAlignment), so local output must keep the unaligned
    flanks: protein pairs with a shared core inside unrelated flanks, a pair
    with no positive cell (empty local alignment) and a pair aligned from
    its first residues."""
    rng = np.random.default_rng(41)
    tool = T.GpuAlignmentTool()
    fin, fout = tmp_path / "in.fa", tmp_path / "out.fa"
    cases = []
    for k in range(6):
        core = W.random_protein(rng, int(rng.integers(40, 160)))
        mut, _ = W._mutate_proteins(rng, core, np.array([len(core)]), np.array([0.3]), 0.05)
        fa = W.random_protein(rng, int(rng.integers(0, 90))).tobytes().decode()
        fb = W.random_protein(rng, int(rng.integers(0, 90))).tobytes().decode()
        ta = W.random_protein(rng, int(rng.integers(0, 90))).tobytes().decode()
        tb = W.random_protein(rng, int(rng.integers(0, 90))).tobytes().decode()
        cases.append((fa + core.tobytes().decode() + ta, fb + mut.tobytes().decode() + tb))
    cases.append(("PPPPPPPP", "WWWWW"))  # every cell scores below zero: empty local alignment
    cases.append(("HEAGAWGHEE", "HEAGAWGHEEPAWHEAE"))
    for a, b in cases:
        F.write(str(fin), [F.Record(">a", "a", a), F.Record(">b", "b", b)])
        r = tool.align_files(str(fin), str(fout), local=True)
        assert r.returncode == 0, r.stderr
        want = O.align(a.encode(), b.encode(), local=True)
        _check_full_local_rows(F.read(str(fout)), a, b, want)


def test_all_vs_all_identity_table(tmp_path):
    rng = np.random.default_rng(3)
    recs = []
    for k in range(9):
        s = W.random_protein(rng, int(rng.integers(80, 300))).tobytes().decode()
        recs.append(F.Record(f">p{k} protein {k}", f"p{k}", s))
    fin, fout = tmp_path / "in.fa", tmp_path / "out.tsv"
    F.write(str(fin), recs)
    r = subprocess.run([B.CLI, "-i", str(fin), "-o", str(fout), "--all-vs-all"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rows = [line.split("\t") for line in fout.read_text().splitlines()]
    assert rows[0] == ["label_a", "label_b", "score", "n_ident", "n_cols", "identity_pct"]
    k = 1
    for x in range(9):
        for y in range(x + 1, 9):
            want = O.score(recs[x].sequence.encode(), recs[y].sequence.encode(), ident=True)
            assert rows[k][:5] == [f"p{x}", f"p{y}", str(want.score), str(want.n_ident), str(want.n_cols)]
            k += 1
    assert k == len(rows)


def _parse_newick(text):
    """Leaf-set splits and leaf order of a Newick string (no quoting)."""
    import re
    order = re.findall(r"[(,]([A-Za-z0-9_]+):", text)
    return order


def test_guide_tree_newick(tmp_path):
    from tweakseq_gb300 import msa

    rng = np.random.default_rng(4)
    recs = []
    for k in range(12):
        s = W.random_protein(rng, int(rng.integers(80, 200))).tobytes().decode()
        recs.append(F.Record(f">s{k}", f"s{k}", s))
    fin, fout = tmp_path / "in.fa", tmp_path / "tree.dnd"
    F.write(str(fin), recs)
    for method in ("upgma", "nj"):
        r = subprocess.run([B.CLI, "-i", str(fin), "-o", str(fout), "--tree", method], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        text = fout.read_text().strip()
        # The same tree as the library's from the oracle's identities.
        ps = W._pairset_from_lists([x.sequence.encode() for x in recs],
                                   np.stack(np.triu_indices(12, 1), 1))
        want = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, mode=O.MODE_IDENT)
        joins = O.guide_tree(O.identity_distances(12, want["n_ident"], want["n_cols"]), N_TREE[method])
        tree = msa.Tree(12, joins, method)
        assert text == tree.newick([x.label for x in recs])
        assert sorted(_parse_newick(text)) == sorted(x.label for x in recs)


N_TREE = {"upgma": 0, "nj": 1}


def test_consensus_line(tmp_path):
    rows = ["AAA-IWW", "A-AaVWW", "A-A.IW-"]
    recs = [F.Record(f">r{k}", f"r{k}", r) for k, r in enumerate(rows)]
    fin, fout = tmp_path / "aln.fa", tmp_path / "cons.fa"
    F.write(str(fin), recs)
    r = subprocess.run([B.CLI, "-i", str(fin), "-o", str(fout), "--consensus"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = F.read(str(fout))
    assert out[0].label == "consensus" and out[0].sequence == "A?A-IW?"
    # Rows of different lengths are refused.
    F.write(str(fin), recs + [F.Record(">short", "short", "AAA")])
    r = subprocess.run([B.CLI, "-i", str(fin), "-o", str(fout), "--consensus"], capture_output=True, text=True)
    assert r.returncode == 1 and "equal length" in r.stderr


def test_in_process_cpp_tool(tmp_path):
    """The C++ tool of include/tweakseq_gb300_tool.hpp aligns in process
    what the command does: gapped FASTA with the input's header lines, the
    oracle's global alignment; in local mode whole rows around the oracle's
    local core."""
    from test_tool_cpp import build_tool_check
    exe = build_tool_check(tmp_path)
    rng = np.random.default_rng(43)
    a = W.random_protein(rng, 310).tobytes().decode()
    b, _ = W._mutate_proteins(rng, np.frombuffer(a.encode(), np.uint8), np.array([310]), np.array([0.5]), 0.05)
    b = b.tobytes().decode()
    fin, fout = tmp_path / "in.fa", tmp_path / "out.fa"
    F.write(str(fin), [F.Record(">first one", "first", a[:40].lower() + "-" + a[40:]), F.Record(">second", "second", b)])
    r = subprocess.run([exe, str(fin), str(fout)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr
    recs = F.read(str(fout))
    assert [x.header for x in recs] == [">first one", ">second"]
    want = O.align(a.encode(), b.encode())
    assert (recs[0].sequence, recs[1].sequence) == (want.aln_a, want.aln_b)
    r = subprocess.run([exe, str(fin), str(fout), "--local"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _check_full_local_rows(F.read(str(fout)), a, b, O.align(a.encode(), b.encode(), O.BLOSUM62, 11, 1, True))
    # An invalid residue is reported, not aligned.
    F.write(str(fin), [F.Record(">x", "x", "ACD1E"), F.Record(">y", "y", "ACDE")])
    r = subprocess.run([exe, str(fin), str(fout)], capture_output=True, text=True)
    assert r.returncode != 0 and "invalid residue" in r.stdout
