"""The in-process C++ tool (include/tweakseq_gb300_tool.hpp), without a GPU:
a small program compiled against the header and the library runs the
FASTA reader and writer, the settings XML and makeCommand."""
import os
import shutil
import subprocess

import pytest

from tweakseq_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))


def build_tool_check(out_dir):
    """Compiles tests/cpp/tool_check.cpp against the in-tree library."""
    B.build()
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = os.path.join(str(out_dir), "tool_check")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-I", os.path.join(B.ROOT, "include"),
                        os.path.join(HERE, "cpp", "tool_check.cpp"), "-o", exe, "-L", B.LIBDIR, "-ltsq_gb300",
                        "-Wl,-rpath," + B.LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_tool_header_host_parts(tmp_path):
    exe = build_tool_check(tmp_path)
    r = subprocess.run([exe, "--host"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "host ok", r.stderr
