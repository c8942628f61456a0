"""CPU tests of the FASTA conventions (tweakseq/Core/FASTAFile.cpp) and of
the AlignmentTool-shaped builtin tool; no GPU call."""
import os
import subprocess
import xml.etree.ElementTree as ET

from tweakseq_gb300 import build as B
from tweakseq_gb300 import fasta as F
from tweakseq_gb300 import tool as T


def test_parse_follows_the_editor_reader():
    text = "\n".join([
        "random preamble is skipped",
        ">seq1 first protein, with a comment",
        "; a comment line right after the header",
        "MKTAY",
        "  IAKQR  ",
        "",
        ";seq2",
        "AC-DE.",
        ">seq3",
    ])
    recs = F.parse(text)
    assert [r.label for r in recs] == ["seq1", "seq2", "seq3"]
    assert recs[0].header == ">seq1 first protein, with a comment"
    assert recs[0].sequence == "MKTAYIAKQR"
    assert recs[1].sequence == "AC-DE."
    assert recs[2].sequence == ""
    assert F.residues("ac-De. f") == "ACDEF"


def test_write_wraps_at_80_columns(tmp_path):
    recs = [F.Record(">a x", "a", "A" * 170), F.Record(">b", "b", "C" * 80)]
    p = tmp_path / "o.fa"
    F.write(str(p), recs)
    lines = p.read_text().splitlines()
    assert lines == [">a x", "A" * 80, "A" * 80, "A" * 10, ">b", "C" * 80]
    assert [(r.label, r.sequence) for r in F.read(str(p))] == [("a", "A" * 170), ("b", "C" * 80)]


def test_tool_interface_and_settings():
    t = T.GpuAlignmentTool()
    assert t.name() == "tweakseq-gb300" and not t.usesStdOut() and not t.preferred()
    exe, args = t.makeCommand("/tmp/in.fa", "/tmp/out.fa")
    assert exe == B.CLI and args == ["-in", "/tmp/in.fa", "-out", "/tmp/out.fa"]
    t.setPreferred(True)
    t.setExecutable("/opt/tsq_align")
    root = ET.Element("settings")
    t.writeSettings(root)
    u = T.GpuAlignmentTool()
    u.readSettings(root)
    assert u.preferred() and u.executable() == "/opt/tsq_align"
    other = ET.fromstring("<s><alignment_tool><name>MUSCLE</name><path>/x</path>"
                          "<preferred>yes</preferred></alignment_tool></s>")
    v = T.GpuAlignmentTool()
    v.readSettings(other)  # another tool's entry is ignored
    assert not v.preferred() and v.executable() == B.CLI


def test_cli_builds_and_prints_usage_without_a_gpu():
    B.build()
    assert os.path.exists(B.CLI)
    r = subprocess.run([B.CLI, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "usage: tsq_align" in r.stderr
    r = subprocess.run([B.CLI, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2
