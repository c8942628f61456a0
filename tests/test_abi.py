"""CPU tests of the C ABI boundary: the library builds for sm_103a, loads,
and exports every function include/tweakseq_gb300.h declares.  No compute
call is made here (there is no GPU in this container)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from tweakseq_gb300 import _native as N
from tweakseq_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "tweakseq_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"^\s*(?:int|void|size_t|int64_t)\s+\*?\s*(tsq_\w+)\s*\(", text, flags=re.M))


@pytest.fixture(scope="module")
def lib():
    B.build()
    return N.lib()


def test_header_declares_bound_functions():
    declared = header_functions()
    assert declared, "no functions parsed from the header"
    assert declared == N.declared_functions()


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", B.LIB], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (tsq_\w+)", out))
    missing = header_functions() - exported
    assert not missing, missing
    for name in header_functions():
        assert hasattr(lib, name)


def test_build_targets_sm_103a_only():
    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_version_and_struct_layouts(lib):
    v = ctypes.c_int32()
    s = ctypes.c_char_p()
    assert lib.tsq_version(ctypes.byref(v), ctypes.byref(s)) == 0
    assert v.value == 1 and b"sm_103a" in s.value
    assert ctypes.sizeof(N.Params) == 40
    assert ctypes.sizeof(N.Result) == 48
    assert ctypes.sizeof(N.PairDesc) == 24
    assert N.TREE_NODE_DTYPE.itemsize == 48


def test_results_strings_packs_every_string(lib):
    """tsq_results_strings reads host results only: aln_a then aln_b of each
    result with strings, n_cols bytes each, back to back."""
    texts = [(b"AC-GT", b"ACTG-"), None, (b"", b""), (b"W", b"-")]
    keep = []
    raw = np.zeros(len(texts), dtype=N.RESULT_DTYPE)
    for k, t in enumerate(texts):
        if t is None:
            continue
        a, b = ctypes.create_string_buffer(t[0] + b"\0"), ctypes.create_string_buffer(t[1] + b"\0")
        keep += [a, b]
        raw["aln_a"][k], raw["aln_b"][k] = ctypes.addressof(a), ctypes.addressof(b)
        raw["n_cols"][k] = len(t[0])
    want = b"AC-GTACTG-" + b"W-"
    assert lib.tsq_results_strings(raw.ctypes.data, len(raw), None, 0) == len(want)
    small = ctypes.create_string_buffer(b"x" * 4)
    assert lib.tsq_results_strings(raw.ctypes.data, len(raw), small, 4) == len(want)
    assert small.raw[:4] == b"xxxx"  # too small: nothing copied
    buf = ctypes.create_string_buffer(len(want))
    assert lib.tsq_results_strings(raw.ctypes.data, len(raw), buf, len(want)) == len(want)
    assert buf.raw == want
    assert lib.tsq_results_strings(None, 0, None, 0) == 0
    assert lib.tsq_results_strings(None, 2, None, 0) == N.E_INVALID_ARG
    assert lib.tsq_results_strings(raw.ctypes.data, -1, None, 0) == N.E_INVALID_ARG
    raw["n_cols"][0] = -1
    assert lib.tsq_results_strings(raw.ctypes.data, len(raw), None, 0) == N.E_INVALID_ARG
