"""CPU tests of the C ABI boundary: the library builds for sm_103a, loads,
and exports every function include/tweakseq_gb300.h declares.  No compute
call is made here (there is no GPU in this container)."""
import ctypes
import os
import re
import subprocess

import pytest

from tweakseq_gb300 import _native as N
from tweakseq_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "tweakseq_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"^\s*(?:int|void|size_t)\s+\*?\s*(tsq_\w+)\s*\(", text, flags=re.M))


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
