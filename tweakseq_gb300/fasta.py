"""FASTA reading and writing with the editor's conventions.

Reading follows tweakseq/Core/FASTAFile.cpp:71-147: a record starts at a line
beginning with '>' or ';', its label is the header text up to the first
space (FASTAFile.cpp:177-187), ';' lines right after a header are comments,
and sequence lines are concatenated.  Writing follows FASTAFile.cpp:149-171:
the header line, then the sequence in lines of 80 characters.
"""
from __future__ import annotations

from dataclasses import dataclass


@dataclass
class Record:
    header: str  # the whole header line, '>' included
    label: str
    sequence: str


def label_of(header: str) -> str:
    sp = header.find(" ", 1)
    return header[1:] if sp == -1 else header[1:sp]


def parse(text: str) -> list[Record]:
    recs: list[Record] = []
    state = "seek"
    for raw in text.splitlines():
        line = raw.strip()
        if not line:
            continue
        c = line[0]
        if c in ">;":
            if state == "comment" and c == ";":
                continue
            recs.append(Record(line, label_of(line), ""))
            state = "comment"
            continue
        if state == "seek":
            continue
        recs[-1].sequence += line
        state = "sequence"
    return recs


def read(path: str) -> list[Record]:
    with open(path) as f:
        return parse(f.read())


def format_records(recs: list[Record], width: int = 80) -> str:
    out = []
    for r in recs:
        out.append(r.header)
        for k in range(0, len(r.sequence), width):
            out.append(r.sequence[k:k + width])
    return "\n".join(out) + ("\n" if out else "")


def write(path: str, recs: list[Record]) -> None:
    with open(path, "w") as f:
        f.write(format_records(recs))


def residues(seq: str) -> str:
    """What the aligner is given: gap characters dropped, letters upper-cased
    (as the external aligners treat the editor's exported FASTA)."""
    return "".join(ch for ch in seq.upper() if ch not in "-. \t")
