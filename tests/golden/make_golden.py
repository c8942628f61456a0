"""Regenerates the committed golden fixtures.  Run explicitly:

    python tests/golden/make_golden.py --reference-root DIR

1. ``blosum62_reference.json`` -- the BLOSUM62 table and its 'A'..'Z' index
   map, parsed from the reference's own source text,
   tweakseq/Core/Annotations/Consensus.cpp:34-69 (the only integer
   substitution data in groundstate/tweakseq).  The oracle and the CUDA
   library both carry the table; tests check both against this fixture, so
   the scoring data is pinned to the reference even though the DP itself has
   no reference implementation to pin against.
2. ``oracle_cases.json`` -- seeded and hand-picked alignment cases with the
   oracle's outputs (score, coordinates, identity, gapped strings).  Tests
   re-run the oracle on them to catch drift, and the GPU tests compare the
   CUDA path against the same records.

The reference tree is read only when (1) is regenerated; nothing at test time
reads it.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def parse_consensus_cpp(path: str) -> dict:
    text = open(path, encoding="utf-8", errors="replace").read()
    m = re.search(r"static\s+int\s+BLOSUM62\s*\[23\]\s*\[23\]\s*=\s*\{(.*?)\};", text, re.S)
    if not m:
        raise SystemExit("BLOSUM62 table not found")
    body = m.group(1)
    rows, order = [], []
    for line in body.splitlines():
        if "{" not in line:
            continue
        nums = line[line.index("{") + 1:line.index("}")]
        rows.append([int(v) for v in nums.replace(" ", "").split(",")])
        tail = line[line.index("}") + 1:]
        lm = re.search(r"//\s*\d+\s+([A-Z])", tail)
        order.append(lm.group(1) if lm else "?")
    mm = re.search(r"static\s+int\s+BLOSUM62map\s*\[26\]\s*=\s*\{(.*?)\};", text, re.S)
    if not mm:
        raise SystemExit("BLOSUM62map not found")
    amap = [int(v) for v in re.findall(r"-?\d+", mm.group(1))]
    assert len(rows) == 23 and all(len(r) == 23 for r in rows) and len(amap) == 26
    return {
        "source": "tweakseq/Core/Annotations/Consensus.cpp:34-69",
        "order": "".join(order),
        "matrix": rows,
        "letter_map": amap,
    }


def oracle_cases() -> list[dict]:
    from oracle import oracle as O
    from tweakseq_gb300 import workloads as W

    cases = []

    def add(name, a, b, matrix=0, go=11, ge=1, local=False):
        r = O.align(a, b, matrix, go, ge, local)
        cases.append({
            "name": name, "a": a.decode() if isinstance(a, bytes) else a, "b": b.decode() if isinstance(b, bytes) else b,
            "matrix": matrix, "gap_open": go, "gap_extend": ge, "local": local,
            "score": r.score, "a_begin": r.a_begin, "a_end": r.a_end, "b_begin": r.b_begin, "b_end": r.b_end,
            "n_ident": r.n_ident, "n_cols": r.n_cols, "aln_a": r.aln_a, "aln_b": r.aln_b,
        })

    # Hand-checkable edge cases.
    for local in (False, True):
        tag = "local" if local else "global"
        add(f"empty_empty_{tag}", b"", b"", local=local)
        add(f"empty_vs_three_{tag}", b"", b"ACD", local=local)
        add(f"one_vs_empty_{tag}", b"W", b"", local=local)
        add(f"single_match_{tag}", b"W", b"W", local=local)
        add(f"single_mismatch_{tag}", b"W", b"P", local=local)
        add(f"gap_run_{tag}", b"AAAA", b"AA", local=local)
        add(f"textbook_{tag}", b"HEAGAWGHEE", b"PAWHEAE", local=local)
        add(f"ambiguity_letters_{tag}", b"BJZXOU", b"DNEQXX", local=local)
        add(f"identical_{tag}", b"MKTAYIAKQRQISFVKSHFSRQ", b"MKTAYIAKQRQISFVKSHFSRQ", local=local)
        add(f"dna_{tag}", b"ACGTACGTTTGACCA", b"ACGACGTTAGACNCA", matrix=1, go=5, ge=2, local=local)
        add(f"dna_iupac_{tag}", b"NNNRYACGT", b"NNNRYACGU", matrix=1, go=5, ge=2, local=local)
    # Seeded random cases across shapes and gap settings.
    rng = np.random.default_rng(20261203)
    for k in range(48):
        m, n = int(rng.integers(0, 70)), int(rng.integers(0, 70))
        local = bool(k % 2)
        if k % 3 == 2:
            a = W.DNA_LETTERS[rng.integers(0, 4, m)].tobytes()
            b = W.DNA_LETTERS[rng.integers(0, 4, n)].tobytes()
            add(f"random_dna_{k}", a, b, 1, 5, 2, local)
        else:
            a = W.random_protein(rng, m).tobytes()
            b = W.random_protein(rng, n).tobytes()
            go, ge = [(11, 1), (10, 1), (5, 2), (0, 1), (3, 0)][k % 5]
            add(f"random_protein_{k}", a, b, 0, go, ge, local)
    # Related pairs (long enough to cross several GPU tiles).
    for k in range(6):
        L = int(rng.integers(150, 400))
        a = W.random_protein(rng, L)
        b, _ = W._mutate_proteins(rng, a, np.array([L]), np.array([0.4]), 0.05)
        add(f"related_protein_{k}", a.tobytes(), b.tobytes(), 0, 11, 1, bool(k % 2))
    return cases


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", required=True,
                    help="root of the groundstate/tweakseq source tree (holds tweakseq/Core/...)")
    args = ap.parse_args()
    cpp = os.path.join(args.reference_root, "tweakseq/Core/Annotations/Consensus.cpp")
    if not os.path.exists(cpp):
        raise SystemExit(f"{cpp} not found: --reference-root must name the reference source tree")
    with open(os.path.join(HERE, "blosum62_reference.json"), "w") as f:
        json.dump(parse_consensus_cpp(cpp), f, indent=1)
    print("wrote blosum62_reference.json")
    with open(os.path.join(HERE, "oracle_cases.json"), "w") as f:
        json.dump(oracle_cases(), f, indent=1)
    print("wrote oracle_cases.json")


if __name__ == "__main__":
    main()
