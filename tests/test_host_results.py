"""CPU tests of the Python layer's result collection: the gapped strings of
a result array come back through one tsq_results_strings copy and are
sliced per pair.  The library's own tsq_results_strings runs (it only reads
host results); freeing is stubbed, because the strings here belong to
Python buffers.  No GPU call."""
import ctypes

import numpy as np
import pytest

from tweakseq_gb300 import _native as N
from tweakseq_gb300 import aligner as A
from tweakseq_gb300 import build as B


class _Lib:
    """The real library, with tsq_results_free replaced by a recorder."""

    def __init__(self, real):
        self.real = real
        self.freed = []

    def __getattr__(self, name):
        return getattr(self.real, name)

    def tsq_results_free(self, ptr, n):
        self.freed.append(n)


@pytest.fixture
def fake_lib(monkeypatch):
    B.build()
    lib = _Lib(N.lib())
    monkeypatch.setattr(N, "lib", lambda: lib)
    return lib


def _results(texts):
    keep = []
    raw = np.zeros(len(texts), dtype=N.RESULT_DTYPE)
    for k, t in enumerate(texts):
        raw["score"][k] = 10 * k - 7
        raw["status"][k] = 0 if t is not None else N.E_INVALID_RESIDUE
        if t is None:
            continue
        a, b = ctypes.create_string_buffer(t[0].encode() + b"\0"), ctypes.create_string_buffer(t[1].encode() + b"\0")
        keep += [a, b]
        raw["aln_a"][k], raw["aln_b"][k] = ctypes.addressof(a), ctypes.addressof(b)
        raw["n_cols"][k] = len(t[0])
        raw["n_ident"][k] = sum(x == y for x, y in zip(*t))
    return raw, keep


def test_collect_slices_every_pair(fake_lib):
    texts = [("AC-GT", "ACTG-"), None, ("", ""), ("W" * 300, "-" * 300), None, ("K", "K")]
    raw, keep = _results(texts)
    res = A._collect(raw, True)
    assert res.aln_a == [None if t is None else t[0] for t in texts]
    assert res.aln_b == [None if t is None else t[1] for t in texts]
    for f in ("score", "n_ident", "n_cols", "status"):
        assert np.array_equal(res.table[f], raw[f]), f
    assert fake_lib.freed == [len(texts)]
    assert res[3].aln_a == "W" * 300 and res[5].n_ident == 1


def test_collect_without_strings_and_empty(fake_lib):
    raw, keep = _results([("A", "A")])
    res = A._collect(raw, False)
    assert res.aln_a is None and res.aln_b is None and fake_lib.freed == []
    empty = A._collect(np.zeros(0, dtype=N.RESULT_DTYPE), True)
    assert empty.aln_a == [] and empty.aln_b == [] and len(empty) == 0
