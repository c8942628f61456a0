"""ctypes front end of the CPU oracle (oracle/tsq_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
as the checker, and by bench.py's CPU-baseline / reference leg.  The product
(tweakseq_gb300/) never imports this module.

Parity is unpinned: the reference (groundstate/tweakseq) has no pairwise DP of
its own (its alignment runs in external programs launched from
tweakseq/UI/SeqEditMainWin.cpp:1616-1663), so this oracle restates Gotoh
(1982) with the conventions written in oracle/tsq_oracle.h.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libtsq_oracle.so")

BLOSUM62 = 0
DNA = 1


class Scheme(ctypes.Structure):
    _fields_ = [("score", (ctypes.c_int8 * 26) * 26), ("valid", ctypes.c_uint8 * 26)]


class Result(ctypes.Structure):
    _fields_ = [
        ("score", ctypes.c_int32),
        ("a_begin", ctypes.c_int32),
        ("a_end", ctypes.c_int32),
        ("b_begin", ctypes.c_int32),
        ("b_end", ctypes.c_int32),
        ("n_ident", ctypes.c_int32),
        ("n_cols", ctypes.c_int32),
    ]


RESULT_DTYPE = np.dtype(
    [(name, np.int32) for name in ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols")]
)

_lib = None


def build(force: bool = False) -> str:
    """Compiles the oracle with its Makefile (gcc, no GPU needed)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("tsq_oracle.c", "tsq_oracle.h")
    ):
        subprocess.run(["make", "-s", "-B", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        i32 = ctypes.c_int32
        L.tsqo_builtin_scheme.argtypes = [ctypes.c_int, ctypes.POINTER(Scheme)]
        common = [u8p, i32, u8p, i32, ctypes.POINTER(Scheme), i32, i32, i32]
        L.tsqo_align.argtypes = common + [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(Result)]
        L.tsqo_score.argtypes = common + [ctypes.POINTER(Result)]
        L.tsqo_score_ident.argtypes = common + [ctypes.POINTER(Result)]
        L.tsqo_score_global_midpoint.argtypes = [u8p, i32, u8p, i32, ctypes.POINTER(Scheme), i32, i32,
                                                 ctypes.POINTER(i32)]
        vp = ctypes.c_void_p
        L.tsqo_batch.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int64, ctypes.POINTER(Scheme), i32, i32, i32,
                                 i32, i32, vp, vp, vp, vp]
        L.tsqo_num_cores.restype = ctypes.c_int
        L.tsqo_consensus.argtypes = [vp, i32, i32, ctypes.c_int64, ctypes.c_double, i32, vp, vp, vp]
        L.tsqo_identity_distance.argtypes = [i32, i32]
        L.tsqo_identity_distance.restype = ctypes.c_int64
        L.tsqo_guide_tree.argtypes = [i32, vp, i32, vp]
        _lib = L
    return _lib


def scheme(which=BLOSUM62) -> Scheme:
    """A builtin scheme (BLOSUM62 or DNA) or a (26x26 matrix, 26 valid) pair."""
    s = Scheme()
    if isinstance(which, int):
        rc = lib().tsqo_builtin_scheme(which, ctypes.byref(s))
        if rc:
            raise ValueError(f"unknown scheme {which}")
        return s
    mat, valid = which
    mat = np.ascontiguousarray(mat, dtype=np.int8).reshape(26, 26)
    valid = np.ascontiguousarray(valid, dtype=np.uint8).reshape(26)
    ctypes.memmove(s.score, mat.ctypes.data, 676)
    ctypes.memmove(s.valid, valid.ctypes.data, 26)
    return s


def scheme_arrays(which=BLOSUM62):
    s = scheme(which)
    mat = np.frombuffer(bytes(s.score), dtype=np.int8).reshape(26, 26).copy()
    valid = np.frombuffer(bytes(s.valid), dtype=np.uint8).copy()
    return mat, valid


class OracleError(RuntimeError):
    def __init__(self, rc):
        super().__init__(f"oracle status {rc}")
        self.rc = rc


def _buf(s: bytes):
    arr = (ctypes.c_uint8 * max(1, len(s))).from_buffer_copy(s if s else b"\0")
    return arr


@dataclass
class Alignment:
    score: int
    a_begin: int
    a_end: int
    b_begin: int
    b_end: int
    n_ident: int
    n_cols: int
    aln_a: str | None = None
    aln_b: str | None = None


def _res(r: Result, aa=None, ab=None) -> Alignment:
    return Alignment(r.score, r.a_begin, r.a_end, r.b_begin, r.b_end, r.n_ident, r.n_cols, aa, ab)


def align(a: bytes, b: bytes, which=BLOSUM62, gap_open=11, gap_extend=1, local=False) -> Alignment:
    if isinstance(a, str):
        a = a.encode()
    if isinstance(b, str):
        b = b.encode()
    sc = scheme(which)
    cap = len(a) + len(b) + 1
    sa, sb = ctypes.create_string_buffer(cap), ctypes.create_string_buffer(cap)
    r = Result()
    rc = lib().tsqo_align(_buf(a), len(a), _buf(b), len(b), ctypes.byref(sc), gap_open, gap_extend, int(local), sa,
                          sb, ctypes.byref(r))
    if rc:
        raise OracleError(rc)
    return _res(r, sa.value.decode(), sb.value.decode())


def score(a: bytes, b: bytes, which=BLOSUM62, gap_open=11, gap_extend=1, local=False, ident=False) -> Alignment:
    if isinstance(a, str):
        a = a.encode()
    if isinstance(b, str):
        b = b.encode()
    sc = scheme(which)
    r = Result()
    fn = lib().tsqo_score_ident if ident else lib().tsqo_score
    rc = fn(_buf(a), len(a), _buf(b), len(b), ctypes.byref(sc), gap_open, gap_extend, int(local), ctypes.byref(r))
    if rc:
        raise OracleError(rc)
    return _res(r)


def midpoint_score(a: bytes, b: bytes, which=BLOSUM62, gap_open=11, gap_extend=1) -> int:
    sc = scheme(which)
    out = ctypes.c_int32()
    rc = lib().tsqo_score_global_midpoint(_buf(a), len(a), _buf(b), len(b), ctypes.byref(sc), gap_open, gap_extend,
                                          ctypes.byref(out))
    if rc:
        raise OracleError(rc)
    return out.value


def num_cores() -> int:
    return lib().tsqo_num_cores()


MODE_SCORE, MODE_IDENT, MODE_ALIGN = 0, 1, 2


def batch(seqs: np.ndarray, a_off, a_len, b_off, b_len, which=BLOSUM62, gap_open=11, gap_extend=1, local=False,
          mode=MODE_SCORE, nthreads=0, strings=False):
    """Runs the oracle over many pairs on nthreads host threads.

    Returns a structured numpy array (RESULT_DTYPE) and, when strings=True
    (mode 2), lists of gapped strings."""
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    a_off = np.ascontiguousarray(a_off, dtype=np.int64)
    b_off = np.ascontiguousarray(b_off, dtype=np.int64)
    a_len = np.ascontiguousarray(a_len, dtype=np.int32)
    b_len = np.ascontiguousarray(b_len, dtype=np.int32)
    n = len(a_off)
    out = np.zeros(n, dtype=RESULT_DTYPE)
    sc = scheme(which)
    aln_a = aln_b = aln_off = None
    if strings:
        caps = a_len.astype(np.int64) + b_len + 1
        aln_off = np.zeros(n, dtype=np.int64)
        aln_off[1:] = np.cumsum(caps)[:-1]
        total = int(caps.sum()) if n else 1
        aln_a = np.zeros(total, dtype=np.uint8)
        aln_b = np.zeros(total, dtype=np.uint8)
    p = lambda x: None if x is None else x.ctypes.data
    rc = lib().tsqo_batch(p(seqs), p(a_off), p(a_len), p(b_off), p(b_len), n, ctypes.byref(sc), gap_open,
                          gap_extend, int(local), mode, nthreads, p(aln_a), p(aln_b), p(aln_off), p(out))
    if rc:
        raise OracleError(rc)
    if not strings:
        return out
    sa, sb = [], []
    for k in range(n):
        o = int(aln_off[k])
        L = int(out["n_cols"][k])
        sa.append(aln_a[o:o + L].tobytes().decode())
        sb.append(aln_b[o:o + L].tobytes().decode())
    return out, sa, sb


def consensus(rows: np.ndarray, plurality: float = -1.0, nthreads: int = 0):
    """Consensus::calculate restated (tsqo_consensus) over a 2-D uint8 array
    (one row per sequence).  Returns (consensus bytes, best_score,
    best_matches)."""
    rows = np.ascontiguousarray(rows, dtype=np.uint8)
    nseq, ncols = rows.shape
    out = np.zeros(max(ncols, 1), dtype=np.uint8)
    sc = np.zeros(max(ncols, 1), dtype=np.int32)
    mt = np.zeros(max(ncols, 1), dtype=np.int32)
    rc = lib().tsqo_consensus(rows.ctypes.data, nseq, ncols, ncols, plurality, nthreads, out.ctypes.data,
                              sc.ctypes.data, mt.ctypes.data)
    if rc:
        raise OracleError(rc)
    return out[:ncols].tobytes(), sc[:ncols], mt[:ncols]


TREE_UPGMA, TREE_NJ = 0, 1
DIST_ONE = 1 << 32
TREE_NODE_DTYPE = np.dtype([("left", np.int32), ("right", np.int32), ("size", np.int32), ("pos", np.int32),
                            ("dist", np.int64), ("height", np.int64), ("left_length", np.int64),
                            ("right_length", np.int64)])


def identity_distances(n: int, n_ident, n_cols) -> np.ndarray:
    """Full n x n int64 distance matrix (2^-32 units) from the identities of
    the unordered pairs (i < j) in row-major order."""
    n_ident = np.asarray(n_ident, dtype=np.int64)
    n_cols = np.asarray(n_cols, dtype=np.int64)
    num = (n_cols - n_ident).astype(np.uint64) << np.uint64(32)
    d = np.where(n_cols > 0, num // np.maximum(n_cols, 1).astype(np.uint64), np.uint64(DIST_ONE)).astype(np.int64)
    D = np.zeros((n, n), dtype=np.int64)
    iu = np.triu_indices(n, 1)
    D[iu] = d
    D.T[iu] = d
    return D


def guide_tree(dist: np.ndarray, method: int = TREE_UPGMA) -> np.ndarray:
    """tsqo_guide_tree over a full symmetric int64 matrix; n-1 joins."""
    dist = np.ascontiguousarray(dist, dtype=np.int64)
    n = dist.shape[0]
    out = np.zeros(max(n - 1, 1), dtype=TREE_NODE_DTYPE)
    rc = lib().tsqo_guide_tree(n, dist.ctypes.data, method, out.ctypes.data)
    if rc:
        raise OracleError(rc)
    return out[:max(n - 1, 0)]


def threads_for_traceback(max_cells: int, cap: int = 0) -> int:
    """Host threads for a traceback batch whose largest pair has max_cells
    cells: the oracle's direction matrix takes one byte per cell per thread,
    so the count is bounded by the memory available now (with a 1.5x margin)
    as well as by the host cores (and by cap when it is set)."""
    try:
        avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except (ValueError, OSError, AttributeError):
        avail = 8 << 30
    by_ram = int(avail // max(1, int(1.5 * max_cells)))
    n = max(1, min(num_cores(), by_ram))
    return min(n, cap) if cap > 0 else n
