"""Host API for the two steps either side of the pairwise path: the
consensus line of an alignment and guide trees from all-vs-all identities.

``consensus`` replaces Consensus::calculate
(tweakseq/Core/Annotations/Consensus.cpp:80-161, run by Project::setAligned,
tweakseq/Core/Project.cpp:112-121).  ``guide_tree`` is the step the external
multiple aligners run after all-vs-all (the editor asks ClustalO for tree
order, tweakseq/Core/ClustalO.cpp:51).  Both run in libtsq_gb300.so.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _native as N


@dataclass
class Consensus:
    sequence: bytes           # one byte per column ('?' where no plurality)
    best_score: np.ndarray    # int32 per column: the winning row's sum
    best_matches: np.ndarray  # int32 per column: the winning row's matches

    def text(self) -> str:
        return self.sequence.decode("latin-1")


def _rows(rows) -> np.ndarray:
    if isinstance(rows, np.ndarray):
        arr = np.ascontiguousarray(rows, dtype=np.uint8)
        if arr.ndim != 2:
            raise ValueError("rows must be 2-D (one row per sequence)")
        return arr
    seqs = [r.encode("latin-1") if isinstance(r, str) else bytes(r) for r in rows]
    if not seqs:
        raise ValueError("no rows")
    if len({len(s) for s in seqs}) != 1:
        raise ValueError("aligned rows must all have the same length")
    return np.frombuffer(b"".join(seqs), dtype=np.uint8).reshape(len(seqs), len(seqs[0]))


def consensus(rows, plurality: float | None = None) -> Consensus:
    """Consensus of equal-length gapped rows (strings, bytes or a 2-D uint8
    array).  ``plurality`` defaults to half the number of rows, as the
    reference's does."""
    arr = _rows(rows)
    nseq, ncols = arr.shape
    out = np.zeros(max(ncols, 1), dtype=np.uint8)
    sc = np.zeros(max(ncols, 1), dtype=np.int32)
    mt = np.zeros(max(ncols, 1), dtype=np.int32)
    rc = N.lib().tsq_consensus(arr.ctypes.data, nseq, ncols, ncols, -1.0 if plurality is None else float(plurality),
                               out.ctypes.data, sc.ctypes.data, mt.ctypes.data)
    N.check(rc, "tsq_consensus")
    return Consensus(out[:ncols].tobytes(), sc[:ncols], mt[:ncols])


@dataclass
class Tree:
    """n - 1 joins (structured array, fields of tsq_tree_node) over n leaves.
    Distances and branch lengths are integers in units of 2^-32."""
    n: int
    nodes: np.ndarray
    method: str

    def newick(self, labels=None) -> str:
        """Newick text; branch lengths as decimals (length / 2^32)."""
        labels = [str(k) for k in range(self.n)] if labels is None else [str(x) for x in labels]
        if self.n == 1:
            return labels[0] + ";"
        text = {k: labels[k] for k in range(self.n)}
        for t, nd in enumerate(self.nodes):
            a, b = int(nd["left"]), int(nd["right"])
            la = int(nd["left_length"]) / N.DIST_ONE
            lb = int(nd["right_length"]) / N.DIST_ONE
            text[self.n + t] = f"({text.pop(a)}:{la:.6f},{text.pop(b)}:{lb:.6f})"
        return text[2 * self.n - 2] + ";"

    def leaf_order(self) -> list[int]:
        """Leaves in tree order (left to right), as an aligner's tree-ordered
        output lists them."""
        if self.n == 1:
            return [0]
        order: list[int] = []
        stack = [2 * self.n - 2]
        while stack:
            v = stack.pop()
            if v < self.n:
                order.append(v)
            else:
                nd = self.nodes[v - self.n]
                stack.append(int(nd["right"]))
                stack.append(int(nd["left"]))
        return order


def _method(method) -> int:
    return N.TREE[method] if isinstance(method, str) else int(method)


def _nodes(n: int) -> np.ndarray:
    return np.zeros(max(n - 1, 1), dtype=N.TREE_NODE_DTYPE)


def guide_tree(n: int, n_ident, n_cols, method="upgma") -> Tree:
    """Tree from the identities of the n(n-1)/2 pairs (i < j) in row-major
    order, as an all-vs-all batch lists them."""
    ident = np.ascontiguousarray(n_ident, dtype=np.int32)
    cols = np.ascontiguousarray(n_cols, dtype=np.int32)
    if len(ident) != n * (n - 1) // 2 or len(cols) != len(ident):
        raise ValueError("need n(n-1)/2 identities")
    out = _nodes(n)
    rc = N.lib().tsq_guide_tree(n, ident.ctypes.data if len(ident) else None,
                                cols.ctypes.data if len(cols) else None, _method(method), out.ctypes.data)
    N.check(rc, "tsq_guide_tree")
    return Tree(n, out[:n - 1], str(method))


def guide_tree_from_distances(dist: np.ndarray, method="upgma") -> Tree:
    """Tree from a symmetric n x n int64 matrix in units of 2^-32."""
    D = np.ascontiguousarray(dist, dtype=np.int64)
    n = D.shape[0]
    out = _nodes(n)
    N.check(N.lib().tsq_guide_tree_dist(n, D.ctypes.data, _method(method), out.ctypes.data), "tsq_guide_tree_dist")
    return Tree(n, out[:n - 1], str(method))


def guide_tree_from_batch(batch, n: int, method="upgma") -> Tree:
    """Tree from a device-resident all-vs-all Batch (identity or alignment
    output) that has run; the identities never leave the GPU."""
    out = _nodes(n)
    N.check(N.lib().tsq_batch_guide_tree(batch._h, n, _method(method), out.ctypes.data), "tsq_batch_guide_tree")
    return Tree(n, out[:n - 1], str(method))


def all_vs_all_table(lengths) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
    """Pair table (a_off, a_len, b_off, b_len) of every pair (i < j) in
    row-major order over sequences stored back to back."""
    lengths = np.asarray(lengths, dtype=np.int64)
    off = np.zeros(len(lengths), dtype=np.int64)
    off[1:] = np.cumsum(lengths)[:-1]
    i, j = np.triu_indices(len(lengths), 1)
    return off[i], lengths[i].astype(np.int32), off[j], lengths[j].astype(np.int32)


__all__ = ["Consensus", "consensus", "Tree", "guide_tree", "guide_tree_from_distances", "guide_tree_from_batch",
           "all_vs_all_table"]
