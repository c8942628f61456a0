"""ctypes binding of the C ABI in include/tweakseq_gb300.h.

The shared library is built in-tree by ``tweakseq_gb300.build`` (nvcc,
sm_103a).  Loading fails loudly when it is missing: there is no CPU path.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

TSQ_OK = 0
ERRORS = {
    -1: "TSQ_E_INVALID_ARG",
    -2: "TSQ_E_INVALID_RESIDUE",
    -3: "TSQ_E_NOMEM",
    -4: "TSQ_E_CUDA",
    -5: "TSQ_E_TIMEOUT",
    -6: "TSQ_E_PENDING",
    -7: "TSQ_E_REJECTED",
    -8: "TSQ_E_NOT_FOUND",
    -9: "TSQ_E_CANCELLED",
    -10: "TSQ_E_TOO_LARGE",
}
E_INVALID_ARG, E_INVALID_RESIDUE, E_NOMEM, E_CUDA, E_TIMEOUT, E_PENDING = -1, -2, -3, -4, -5, -6
E_REJECTED, E_NOT_FOUND, E_CANCELLED, E_TOO_LARGE = -7, -8, -9, -10

MATRIX = {"blosum62": 0, "dna": 1, "custom": 2}
MODE = {"global": 0, "local": 1}
OUTPUT = {"score": 0, "identity": 1, "alignment": 2}
LANE = {"auto": 0, "i16": 1, "i32": 2}


class TsqError(RuntimeError):
    def __init__(self, rc: int, what: str = ""):
        super().__init__(f"{what}: {ERRORS.get(rc, rc)}" if what else ERRORS.get(rc, str(rc)))
        self.rc = rc


class Params(ctypes.Structure):
    _fields_ = [
        ("matrix", ctypes.c_int32),
        ("gap_open", ctypes.c_int32),
        ("gap_extend", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("output", ctypes.c_int32),
        ("lane", ctypes.c_int32),
        ("custom_score", ctypes.POINTER(ctypes.c_int8)),
        ("custom_valid", ctypes.POINTER(ctypes.c_uint8)),
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("score", ctypes.c_int32),
        ("a_begin", ctypes.c_int32),
        ("a_end", ctypes.c_int32),
        ("b_begin", ctypes.c_int32),
        ("b_end", ctypes.c_int32),
        ("n_ident", ctypes.c_int32),
        ("n_cols", ctypes.c_int32),
        ("status", ctypes.c_int32),
        ("aln_a", ctypes.c_void_p),
        ("aln_b", ctypes.c_void_p),
    ]


class PairDesc(ctypes.Structure):
    _fields_ = [("a_off", ctypes.c_int64), ("b_off", ctypes.c_int64), ("a_len", ctypes.c_int32),
                ("b_len", ctypes.c_int32)]


class BatchOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("use_graph", ctypes.c_int32), ("autotune", ctypes.c_int32),
                ("wait_polls", ctypes.c_int32)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("slots", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_int64),
                ("max_tick_cells", ctypes.c_int64), ("autotune", ctypes.c_int32), ("resident", ctypes.c_int32),
                ("resident_idle_polls", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("rejected", ctypes.c_int64),
                ("cancelled", ctypes.c_int64), ("ticks", ctypes.c_int64), ("cells_completed", ctypes.c_int64),
                ("peak_reserved_bytes", ctypes.c_int64), ("admission_waits", ctypes.c_int64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("span_s", ctypes.c_double), ("resident_requests", ctypes.c_int64),
                ("resident_launches", ctypes.c_int64), ("resident_idle_exits", ctypes.c_int64)]


class BatchStats(ctypes.Structure):
    _fields_ = [
        ("cells", ctypes.c_int64),
        ("pairs", ctypes.c_int64),
        ("rerun_pairs", ctypes.c_int64),
        ("launches", ctypes.c_int32),
        ("buckets", ctypes.c_int32),
        ("device_ms", ctypes.c_double),
        ("fill_ms", ctypes.c_double),
    ]


# numpy views of the same layouts (for whole-batch conversions).
RESULT_DTYPE = np.dtype([
    ("score", np.int32), ("a_begin", np.int32), ("a_end", np.int32), ("b_begin", np.int32), ("b_end", np.int32),
    ("n_ident", np.int32), ("n_cols", np.int32), ("status", np.int32), ("aln_a", np.uint64), ("aln_b", np.uint64),
])
PAIR_DTYPE = np.dtype([("a_off", np.int64), ("b_off", np.int64), ("a_len", np.int32), ("b_len", np.int32)])
assert RESULT_DTYPE.itemsize == ctypes.sizeof(Result) and PAIR_DTYPE.itemsize == ctypes.sizeof(PairDesc)

_lib = None

# Every function the header declares, with its ctypes signature.
TREE_NODE_DTYPE = np.dtype([("left", np.int32), ("right", np.int32), ("size", np.int32), ("pos", np.int32),
                            ("dist", np.int64), ("height", np.int64), ("left_length", np.int64),
                            ("right_length", np.int64)])
TREE = {"upgma": 0, "nj": 1}
DIST_ONE = 1 << 32  # distances and branch lengths are in units of 2^-32

_VP = ctypes.c_void_p
_SIGS = {
    "tsq_version": ([ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_char_p)], ctypes.c_int),
    "tsq_align_pair": ([_VP, ctypes.c_int32, _VP, ctypes.c_int32, ctypes.POINTER(Params), _VP], ctypes.c_int),
    "tsq_result_free": ([_VP], None),
    "tsq_results_free": ([_VP, ctypes.c_int64], None),
    "tsq_results_strings": ([_VP, ctypes.c_int64, _VP, ctypes.c_int64], ctypes.c_int64),
    "tsq_align_batch": ([_VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.POINTER(Params), ctypes.POINTER(BatchOpts),
                         _VP], ctypes.c_int),
    "tsq_batch_create": ([_VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.POINTER(Params),
                          ctypes.POINTER(BatchOpts), ctypes.POINTER(_VP)], ctypes.c_int),
    "tsq_batch_run": ([_VP], ctypes.c_int),
    "tsq_batch_run_async": ([_VP], ctypes.c_int),
    "tsq_batch_sync": ([_VP], ctypes.c_int),
    "tsq_batch_results": ([_VP, _VP], ctypes.c_int),
    "tsq_batch_get_stats": ([_VP, ctypes.POINTER(BatchStats)], ctypes.c_int),
    "tsq_batch_stream": ([_VP, ctypes.POINTER(_VP)], ctypes.c_int),
    "tsq_batch_destroy": ([_VP], None),
    "tsq_server_create": ([ctypes.POINTER(ServerOpts), ctypes.POINTER(_VP)], ctypes.c_int),
    "tsq_server_submit": ([_VP, _VP, ctypes.c_int64, _VP, ctypes.c_int64, ctypes.POINTER(Params),
                           ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "tsq_server_poll": ([_VP, ctypes.c_uint64, ctypes.c_int32, _VP, ctypes.c_int64], ctypes.c_int),
    "tsq_server_cancel": ([_VP, ctypes.c_uint64], ctypes.c_int),
    "tsq_server_get_stats": ([_VP, ctypes.POINTER(ServerStats)], ctypes.c_int),
    "tsq_server_destroy": ([_VP], ctypes.c_int),
    "tsq_tune_run": ([ctypes.c_char_p, ctypes.c_int32], ctypes.c_int),
    "tsq_tune_load": ([ctypes.c_char_p], ctypes.c_int),
    "tsq_probe_dpx": ([ctypes.c_int32, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "tsq_align_score_noalloc": ([_VP, ctypes.c_int64, _VP, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(Params),
                                 _VP, _VP], ctypes.c_int),
    "tsq_consensus": ([_VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_double, _VP, _VP, _VP],
                      ctypes.c_int),
    "tsq_consensus_scratch_bytes": ([ctypes.c_int32], ctypes.c_size_t),
    "tsq_consensus_device": ([_VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, ctypes.c_double, _VP, _VP, _VP,
                              _VP, ctypes.c_size_t, _VP], ctypes.c_int),
    "tsq_guide_tree_dist": ([ctypes.c_int32, _VP, ctypes.c_int32, _VP], ctypes.c_int),
    "tsq_guide_tree": ([ctypes.c_int32, _VP, _VP, ctypes.c_int32, _VP], ctypes.c_int),
    "tsq_batch_guide_tree": ([_VP, ctypes.c_int32, ctypes.c_int32, _VP], ctypes.c_int),
}


def declared_functions() -> set[str]:
    return set(_SIGS)


def lib(build_if_missing: bool = False) -> ctypes.CDLL:
    """Loads libtsq_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise RuntimeError(f"{LIB_PATH} is missing: build it with tweakseq_gb300.build.build() "
                                   "(there is no CPU fallback)")
            _build.build()
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(rc: int, what: str = "") -> None:
    if rc != TSQ_OK:
        raise TsqError(rc, what)


def make_params(matrix="blosum62", gap_open=11, gap_extend=1, mode="global", output="alignment", lane="auto",
                custom=None) -> tuple[Params, tuple]:
    """Builds a Params struct; ``custom`` is (26x26 int8, 26 uint8) for a
    custom matrix.  Returns (params, keepalive)."""
    p = Params()
    p.matrix = MATRIX[matrix] if isinstance(matrix, str) else int(matrix)
    p.gap_open, p.gap_extend = int(gap_open), int(gap_extend)
    p.mode = MODE[mode] if isinstance(mode, str) else int(mode)
    p.output = OUTPUT[output] if isinstance(output, str) else int(output)
    p.lane = LANE[lane] if isinstance(lane, str) else int(lane)
    keep = ()
    if custom is not None:
        mat = np.ascontiguousarray(custom[0], dtype=np.int8).reshape(26, 26)
        val = np.ascontiguousarray(custom[1], dtype=np.uint8).reshape(26)
        p.matrix = MATRIX["custom"]
        p.custom_score = mat.ctypes.data_as(ctypes.POINTER(ctypes.c_int8))
        p.custom_valid = val.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        keep = (mat, val)
    return p, keep
