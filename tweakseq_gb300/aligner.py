"""Python host API over the C ABI: plain, batched and device-resident forms.

The reference (groundstate/tweakseq) aligns through an AlignmentTool plugin
that the editor drives with FASTA files (tweakseq/Core/AlignmentTool.h:36-71,
tweakseq/UI/SeqEditMainWin.cpp:1616-1663).  This module is the in-process
call that replaces the external program; ``tweakseq_gb300.tool`` wraps it in
the same plugin shape.  Every call goes through libtsq_gb300.so; nothing
here computes an alignment.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N


@dataclass
class Alignment:
    score: int
    a_begin: int
    a_end: int
    b_begin: int
    b_end: int
    n_ident: int
    n_cols: int
    status: int = 0
    aln_a: str | None = None
    aln_b: str | None = None

    @property
    def identity(self) -> float:
        """Percent identity: identical columns / alignment columns * 100."""
        return 100.0 * self.n_ident / self.n_cols if self.n_cols > 0 else 0.0


def _bytes(s) -> bytes:
    if isinstance(s, str):
        return s.encode("ascii")
    if isinstance(s, np.ndarray):
        return s.astype(np.uint8, copy=False).tobytes()
    return bytes(s)


def align_pair(a, b, matrix="blosum62", gap_open=11, gap_extend=1, mode="global", output="alignment", lane="auto",
               custom=None) -> Alignment:
    """Plain form: one pair, one launch sequence on the current GPU."""
    L = N.lib()
    a, b = _bytes(a), _bytes(b)
    p, keep = N.make_params(matrix, gap_open, gap_extend, mode, output, lane, custom)
    r = N.Result()
    ba = (ctypes.c_uint8 * max(1, len(a))).from_buffer_copy(a or b"\0")
    bb = (ctypes.c_uint8 * max(1, len(b))).from_buffer_copy(b or b"\0")
    rc = L.tsq_align_pair(ctypes.cast(ba, ctypes.c_void_p), len(a), ctypes.cast(bb, ctypes.c_void_p), len(b),
                          ctypes.byref(p), ctypes.byref(r))
    try:
        N.check(rc, "tsq_align_pair")
        out = Alignment(r.score, r.a_begin, r.a_end, r.b_begin, r.b_end, r.n_ident, r.n_cols, r.status)
        if r.aln_a:
            out.aln_a = ctypes.string_at(r.aln_a, r.n_cols).decode("ascii")
            out.aln_b = ctypes.string_at(r.aln_b, r.n_cols).decode("ascii")
        return out
    finally:
        L.tsq_result_free(ctypes.byref(r))
        del keep


@dataclass
class BatchResult:
    """Per-pair results of a batch: numpy columns plus optional strings."""

    table: np.ndarray  # structured, fields score .. status
    aln_a: list | None = None
    aln_b: list | None = None

    def __len__(self):
        return len(self.table)

    def __getitem__(self, k) -> Alignment:
        t = self.table[k]
        return Alignment(int(t["score"]), int(t["a_begin"]), int(t["a_end"]), int(t["b_begin"]), int(t["b_end"]),
                         int(t["n_ident"]), int(t["n_cols"]), int(t["status"]),
                         self.aln_a[k] if self.aln_a is not None else None,
                         self.aln_b[k] if self.aln_b is not None else None)


def pair_table(a_off, a_len, b_off, b_len) -> np.ndarray:
    t = np.zeros(len(a_off), dtype=N.PAIR_DTYPE)
    t["a_off"], t["a_len"], t["b_off"], t["b_len"] = a_off, a_len, b_off, b_len
    return t


def _per_pair_status(rc: int, raw: np.ndarray) -> bool:
    """True when a batch call's status is OK or one that pairs of the batch
    report in their own status field (an invalid residue, a device-side
    wait that ran out, a pair too large for memory): the results of the
    other pairs are valid then."""
    if rc == N.TSQ_OK:
        return True
    return rc in (N.E_INVALID_RESIDUE, N.E_TIMEOUT, N.E_TOO_LARGE) and bool((raw["status"] == rc).any())


def _collect(raw: np.ndarray, strings: bool) -> BatchResult:
    L = N.lib()
    table = np.empty(len(raw), dtype=[(k, np.int32) for k in
                                      ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols",
                                       "status")])
    for k in table.dtype.names:
        table[k] = raw[k]
    sa = sb = None
    if strings:
        # All strings in one copy (tsq_results_strings), then slices of one
        # decoded text: a string_at per string costs more than the alignment.
        ptr = raw.ctypes.data if len(raw) else None
        total = L.tsq_results_strings(ptr, len(raw), None, 0)
        N.check(min(total, 0), "tsq_results_strings")
        buf = np.empty(max(total, 1), dtype=np.uint8)
        got = L.tsq_results_strings(ptr, len(raw), buf.ctypes.data, total)
        N.check(min(got, 0), "tsq_results_strings")
        text = buf[:total].tobytes().decode("ascii")
        has = ((raw["aln_a"] != 0) & (raw["aln_b"] != 0)).tolist()
        lens = np.where(has, raw["n_cols"], 0).astype(np.int64)
        ends = np.cumsum(2 * lens).tolist()
        sa, sb = [], []
        for h, c, e in zip(has, lens.tolist(), ends):
            if h:
                sa.append(text[e - 2 * c:e - c])
                sb.append(text[e - c:e])
            else:
                sa.append(None)
                sb.append(None)
        L.tsq_results_free(raw.ctypes.data, len(raw))
    return BatchResult(table, sa, sb)


def _as_inputs(pairs):
    """Accepts a workloads.PairSet or a (seqs, a_off, a_len, b_off, b_len) tuple."""
    if hasattr(pairs, "seqs"):
        seqs, a_off, a_len, b_off, b_len = pairs.seqs, pairs.a_off, pairs.a_len, pairs.b_off, pairs.b_len
    else:
        seqs, a_off, a_len, b_off, b_len = pairs
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    return seqs, pair_table(a_off, a_len, b_off, b_len)


def _opts(use_graph=False, autotune=False, device=-1, wait_polls=0) -> N.BatchOpts:
    o = N.BatchOpts()
    o.device, o.use_graph, o.autotune = int(device), int(bool(use_graph)), int(bool(autotune))
    o.wait_polls = int(wait_polls)
    return o


def align_batch(pairs, matrix="blosum62", gap_open=11, gap_extend=1, mode="global", output="alignment",
                lane="auto", custom=None, use_graph=False, autotune=False, check=True, wait_polls=0) -> BatchResult:
    """Batched form: all pairs in one planned launch sequence.  Host buffers
    in, host results out (the copies are part of the call)."""
    L = N.lib()
    seqs, tab = _as_inputs(pairs)
    p, keep = N.make_params(matrix, gap_open, gap_extend, mode, output, lane, custom)
    raw = np.zeros(len(tab), dtype=N.RESULT_DTYPE)
    o = _opts(use_graph, autotune, wait_polls=wait_polls)
    rc = L.tsq_align_batch(seqs.ctypes.data if len(seqs) else None, len(seqs), tab.ctypes.data if len(tab) else None,
                           len(tab), ctypes.byref(p), ctypes.byref(o), raw.ctypes.data if len(raw) else None)
    if not _per_pair_status(rc, raw):
        N.check(rc, "tsq_align_batch")
    res = _collect(raw, output == "alignment" or output == 2)
    del keep
    if check and rc != N.TSQ_OK:
        N.check(rc, "tsq_align_batch")
    return res


class Batch:
    """Device-resident batch: inputs uploaded and planned once, then any
    number of runs; results stay in HBM until ``results()``."""

    def __init__(self, pairs, matrix="blosum62", gap_open=11, gap_extend=1, mode="global", output="score",
                 lane="auto", custom=None, use_graph=True, autotune=False, wait_polls=0):
        L = N.lib()
        seqs, tab = _as_inputs(pairs)
        p, keep = N.make_params(matrix, gap_open, gap_extend, mode, output, lane, custom)
        o = _opts(use_graph, autotune, wait_polls=wait_polls)
        h = ctypes.c_void_p()
        rc = L.tsq_batch_create(seqs.ctypes.data if len(seqs) else None, len(seqs),
                                tab.ctypes.data if len(tab) else None, len(tab), ctypes.byref(p), ctypes.byref(o),
                                ctypes.byref(h))
        del keep
        N.check(rc, "tsq_batch_create")
        self._h = h
        self.n = len(tab)
        self.output = output
        self.cells = int(np.dot(tab["a_len"].astype(np.int64), tab["b_len"].astype(np.int64)))

    def run(self):
        N.check(N.lib().tsq_batch_run(self._h), "tsq_batch_run")

    def run_async(self):
        N.check(N.lib().tsq_batch_run_async(self._h), "tsq_batch_run_async")

    def sync(self):
        N.check(N.lib().tsq_batch_sync(self._h), "tsq_batch_sync")

    def results(self, check=True) -> BatchResult:
        raw = np.zeros(self.n, dtype=N.RESULT_DTYPE)
        rc = N.lib().tsq_batch_results(self._h, raw.ctypes.data if self.n else None)
        if not _per_pair_status(rc, raw):
            N.check(rc, "tsq_batch_results")
        res = _collect(raw, self.output in ("alignment", 2))
        if check and rc != N.TSQ_OK:
            N.check(rc, "tsq_batch_results")
        return res

    def stats(self) -> dict:
        s = N.BatchStats()
        N.check(N.lib().tsq_batch_get_stats(self._h, ctypes.byref(s)), "tsq_batch_get_stats")
        return {k: getattr(s, k) for k, _ in s._fields_}

    @property
    def stream(self) -> int:
        v = ctypes.c_void_p()
        N.check(N.lib().tsq_batch_stream(self._h, ctypes.byref(v)), "tsq_batch_stream")
        return v.value or 0

    def close(self):
        if getattr(self, "_h", None):
            N.lib().tsq_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def version() -> tuple[int, str]:
    v = ctypes.c_int32()
    s = ctypes.c_char_p()
    N.check(N.lib().tsq_version(ctypes.byref(v), ctypes.byref(s)))
    return v.value, s.value.decode()


def tune(path: str, quick: bool = True) -> None:
    N.check(N.lib().tsq_tune_run(path.encode(), int(quick)), "tsq_tune_run")


def load_tuning(path: str) -> None:
    N.check(N.lib().tsq_tune_load(path.encode()), "tsq_tune_load")


def probe_dpx(packed: bool = False) -> float:
    """Measured DPX-class instructions per lane per second on this GPU."""
    v = ctypes.c_double()
    N.check(N.lib().tsq_probe_dpx(int(packed), ctypes.byref(v)), "tsq_probe_dpx")
    return v.value


class Server:
    """Continuous-batching server (tsq_server_*): submit requests of any
    size from any thread, poll their results; the library's scheduler thread
    groups, admits (by HBM budget) and overlaps them on the GPU.  With
    resident=True, score and identity requests of pairs up to 2,048 residues
    go to the device-resident request loop (a persistent kernel fed from a
    device task queue) instead of ticks."""

    def __init__(self, slots=4, hbm_budget_bytes=0, max_tick_cells=0, autotune=False, device=-1, resident=False,
                 resident_idle_polls=0):
        o = N.ServerOpts()
        o.device, o.slots, o.hbm_budget_bytes, o.max_tick_cells = device, slots, hbm_budget_bytes, max_tick_cells
        o.autotune = int(bool(autotune))
        o.resident = int(bool(resident))
        o.resident_idle_polls = int(resident_idle_polls)
        h = ctypes.c_void_p()
        N.check(N.lib().tsq_server_create(ctypes.byref(o), ctypes.byref(h)), "tsq_server_create")
        self._h = h
        self._meta = {}

    def submit(self, pairs, matrix="blosum62", gap_open=11, gap_extend=1, mode="global", output="alignment",
               lane="auto", custom=None) -> int:
        seqs, tab = _as_inputs(pairs)
        p, keep = N.make_params(matrix, gap_open, gap_extend, mode, output, lane, custom)
        rid = ctypes.c_uint64()
        rc = N.lib().tsq_server_submit(self._h, seqs.ctypes.data if len(seqs) else None, len(seqs),
                                       tab.ctypes.data if len(tab) else None, len(tab), ctypes.byref(p),
                                       ctypes.byref(rid))
        del keep
        N.check(rc, "tsq_server_submit")
        self._meta[rid.value] = (len(tab), output)
        return rid.value

    def poll(self, rid: int, wait_ms: int = -1, check=True):
        """Returns the request's BatchResult, or None while it is pending."""
        n, output = self._meta[rid]
        raw = np.zeros(n, dtype=N.RESULT_DTYPE)
        rc = N.lib().tsq_server_poll(self._h, rid, int(wait_ms), raw.ctypes.data if n else None, n)
        if rc == N.E_PENDING:
            return None
        if rc not in (N.TSQ_OK, N.E_INVALID_RESIDUE):
            self._meta.pop(rid, None)
            N.check(rc, "tsq_server_poll")
        self._meta.pop(rid, None)
        res = _collect(raw, output in ("alignment", 2))
        if check and rc != N.TSQ_OK:
            N.check(rc, "tsq_server_poll")
        return res

    def cancel(self, rid: int) -> int:
        return N.lib().tsq_server_cancel(self._h, rid)

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(N.lib().tsq_server_get_stats(self._h, ctypes.byref(st)), "tsq_server_get_stats")
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "_h", None):
            N.lib().tsq_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
