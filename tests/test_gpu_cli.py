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
    assert (got[0].sequence, got[1].sequence) == (want.aln_a, want.aln_b)


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
