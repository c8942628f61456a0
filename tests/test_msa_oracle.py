"""CPU tests of the oracle's consensus and guide-tree restatements:
hand-worked known answers, an independent pure-Python restatement on small
random inputs, and the textbook properties (NJ recovers an additive tree,
UPGMA an ultrametric one).  The reference has no tests of its own for
either step."""
import itertools

import numpy as np
import pytest

from oracle import oracle as O

B62_ORDER = "ARNDCQEGHILKMFPSTWYVBZX"


def _b62():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    fx = json.load(open(os.path.join(here, "golden", "blosum62_reference.json")))
    return np.array(fx["matrix"], dtype=np.int64), fx["letter_map"]


def consensus_literal(rows, plurality=None):
    """Consensus::calculate (Consensus.cpp:80-161) line by line in Python."""
    mat, letter_map = _b62()
    nseq, ncols = len(rows), len(rows[0])
    plur = nseq / 2.0 if plurality is None else plurality
    idx = [[(letter_map[b - 65] if 0 <= b - 65 <= 25 else 99) for b in r] for r in rows]
    out, scores, matches = bytearray(), [], []
    for c in range(ncols):
        hi, ri_hi, ri_m = 0.0, 0, 0.0
        for ri in range(nseq):
            s = m = 0.0
            for rj in range(nseq):
                if ri == rj:
                    continue
                a, b = idx[ri][c], idx[rj][c]
                if a == 99 and b == 99:
                    s += 1.0
                    m += 1.0
                elif a == 99 or b == 99:
                    s += -4.0
                else:
                    s += float(mat[a][b])
                    if mat[a][b] > 0:
                        m += 1.0
            if ri == 0 or s > hi:
                hi, ri_hi, ri_m = s, ri, m
        out.append(rows[ri_hi][c] if ri_m >= plur else ord("?"))
        scores.append(int(hi))
        matches.append(int(ri_m))
    return bytes(out), scores, matches


def _msa(rng, nseq, ncols, alphabet):
    return [bytes(rng.choice(alphabet, ncols)) for _ in range(nseq)]


def test_consensus_known_answers():
    rows = [b"AAA-IWW", b"A-AaVWW", b"A-A.IW-"]
    arr = np.frombuffer(b"".join(rows), dtype=np.uint8).reshape(3, 7)
    cons, score, match = O.consensus(arr)
    # A,A,A: 4+4 each; A,-,-: gap rows score +1-4 = -3 with 1 match < 1.5;
    # three gap-class bytes: +2, 2 matches; I,V,I: I scores 4+3 and is first;
    # W,W,W: 22; W,W,-: 11-4 = 7 with 1 match < 1.5.
    assert cons == b"A?A-IW?"
    assert score.tolist() == [8, -3, 8, 2, 7, 22, 7]
    assert match.tolist() == [2, 1, 2, 2, 2, 2, 1]
    # One row: no pairs, 0 matches < 0.5.
    assert O.consensus(np.frombuffer(b"ACD", dtype=np.uint8).reshape(1, 3))[0] == b"???"
    # J, O, U score as X; all tie at -2 and the first row wins (0 matches).
    col = np.frombuffer(b"JXB", dtype=np.uint8).reshape(3, 1)
    c, s, m = O.consensus(col, plurality=0.0)
    assert c == b"J" and s.tolist() == [-2]
    # A custom plurality lets the weaker columns through (column 1 shows its
    # best row, a gap).
    assert O.consensus(arr, plurality=1.0)[0] == b"A-A-IWW"


@pytest.mark.parametrize("seed", range(6))
def test_consensus_matches_literal_restatement(seed):
    rng = np.random.default_rng(seed)
    alphabet = np.frombuffer(b"AAAAGGGLLWC-.-aJOUXBZ*\x80\xff", dtype=np.uint8)
    nseq = int(rng.integers(1, 10))
    ncols = int(rng.integers(1, 25))
    rows = _msa(rng, nseq, ncols, alphabet)
    plur = None if seed % 2 == 0 else float(rng.integers(0, nseq + 1)) / 2
    want = consensus_literal(rows, plur)
    got = O.consensus(np.frombuffer(b"".join(rows), dtype=np.uint8).reshape(nseq, ncols),
                      -1.0 if plur is None else plur)
    assert got[0] == want[0]
    assert got[1].tolist() == want[1] and got[2].tolist() == want[2]


def tree_literal(D, method):
    """The guide-tree definition in Python: scan positions, join, repeat."""
    D = [list(map(int, r)) for r in D]
    n = len(D)
    active = list(range(n))
    node = list(range(n))
    size = [1] * n
    height = [0] * n
    out = []
    for t in range(n - 1):
        m = len(active)
        r = {k: sum(D[k][l] for l in active if l != k) for k in active}
        best = None
        for i, j in itertools.combinations(active, 2):
            c = D[i][j] if method == 0 else (m - 2) * D[i][j] - r[i] - r[j]
            if best is None or c < best[0]:
                best = (c, i, j)
        _, i, j = best
        dij = D[i][j]
        if method == 0:
            h = dij // 2
            ll, rl = h - height[i], h - height[j]
        else:
            h = 0
            ll = ((m - 2) * dij + r[i] - r[j]) // (2 * (m - 2)) if m > 2 else dij // 2
            rl = dij - ll
        out.append((node[i], node[j], size[i] + size[j], i, dij, h, ll, rl))
        for k in active:
            if k in (i, j):
                continue
            if method == 0:
                du = (size[i] * D[i][k] + size[j] * D[j][k]) // (size[i] + size[j])
            else:
                du = (D[i][k] + D[j][k] - dij) // 2
            D[i][k] = D[k][i] = du
        if method == 0:
            height[i] = h
        node[i] = n + t
        size[i] += size[j]
        active.remove(j)
    return out


def test_tree_known_answers():
    D = np.array([[0, 2, 6, 10], [2, 0, 6, 10], [6, 6, 0, 10], [10, 10, 10, 0]])
    up = O.guide_tree(D, O.TREE_UPGMA)
    assert [tuple(int(v) for v in x) for x in up] == [(0, 1, 2, 0, 2, 1, 1, 1), (4, 2, 3, 0, 6, 3, 2, 3),
                                                      (5, 3, 4, 0, 10, 5, 2, 5)]
    # Saitou & Nei's five-taxon example: a,b join with 2 and 3; then (ab),c
    # with 3 and 4 (a tie with d,e broken by position); then d with 2 and 2;
    # e last with 1.
    W = np.zeros((5, 5), dtype=np.int64)
    for a, b, v in [(0, 1, 5), (0, 2, 9), (0, 3, 9), (0, 4, 8), (1, 2, 10), (1, 3, 10), (1, 4, 9), (2, 3, 8),
                    (2, 4, 7), (3, 4, 3)]:
        W[a, b] = W[b, a] = v
    nj = O.guide_tree(W, O.TREE_NJ)
    assert [(int(x["left"]), int(x["right"]), int(x["left_length"]), int(x["right_length"])) for x in nj] == [
        (0, 1, 2, 3), (5, 2, 3, 4), (6, 3, 2, 2), (7, 4, 0, 1)]


@pytest.mark.parametrize("seed", range(8))
@pytest.mark.parametrize("method", [O.TREE_UPGMA, O.TREE_NJ])
def test_tree_matches_literal_restatement(seed, method):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(2, 12))
    # Few distinct values, so ties are everywhere.
    D = rng.integers(0, 4, size=(n, n)) * (1 << 30)
    D = np.triu(D, 1)
    D = D + D.T
    got = [tuple(int(v) for v in x) for x in O.guide_tree(D, method)]
    assert got == tree_literal(D, method)


def _random_tree(rng, n):
    """Random rooted binary tree: parent links and even integer branch lengths."""
    parent, length = {}, {}
    nodes = list(range(n))
    nxt = n
    while len(nodes) > 1:
        a, b = rng.choice(len(nodes), 2, replace=False)
        x, y = nodes[a], nodes[b]
        for v in (x, y):
            parent[v] = nxt
            length[v] = 2 * int(rng.integers(1, 50)) << 20
        nodes = [v for k, v in enumerate(nodes) if k not in (a, b)] + [nxt]
        nxt += 1
    return parent, length


def _splits(n, joins):
    """Leaf sets below each join."""
    below = {k: frozenset([k]) for k in range(n)}
    out = set()
    for t, x in enumerate(joins):
        s = below[int(x["left"])] | below[int(x["right"])]
        below[n + t] = s
        if len(s) < n:
            out.add(min(s, frozenset(range(n)) - s, key=sorted))
    return out


def test_nj_recovers_an_additive_tree():
    rng = np.random.default_rng(7)
    n = 12
    parent, length = _random_tree(rng, n)

    def path(v):
        p = [v]
        while p[-1] in parent:
            p.append(parent[p[-1]])
        return p

    D = np.zeros((n, n), dtype=np.int64)
    for i in range(n):
        for j in range(i + 1, n):
            pi, pj = path(i), path(j)
            lca = next(v for v in pi if v in pj)
            d = sum(length[v] for v in pi[:pi.index(lca)]) + sum(length[v] for v in pj[:pj.index(lca)])
            D[i, j] = D[j, i] = d
    joins = O.guide_tree(D, O.TREE_NJ)
    # Unrooted splits of the true tree.
    true = set()
    for v in set(parent.values()):
        leaves = frozenset(k for k in range(n) if v in path(k))
        if 1 < len(leaves) < n - 1:
            true.add(min(leaves, frozenset(range(n)) - leaves, key=sorted))
    got = {s for s in _splits(n, joins) if 1 < len(s) < n - 1}
    assert got == true
    # Leaf branch lengths come back exactly.
    leaf_len = {}
    for x in joins:
        for side in ("left", "right"):
            if int(x[side]) < n:
                leaf_len[int(x[side])] = int(x[side + "_length"])
    root_kids = [v for v in parent if parent[v] == max(parent.values())]
    for k in range(n):
        if k not in root_kids:
            assert leaf_len[k] == length[k]


def test_upgma_recovers_an_ultrametric_tree():
    rng = np.random.default_rng(8)
    n = 16
    # Leaves under joins of strictly increasing heights.
    clusters = [[k] for k in range(n)]
    D = np.zeros((n, n), dtype=np.int64)
    h = 0
    while len(clusters) > 1:
        a, b = sorted(rng.choice(len(clusters), 2, replace=False))
        h += 2 * int(rng.integers(1, 20)) << 20
        for x in clusters[a]:
            for y in clusters[b]:
                D[x, y] = D[y, x] = 2 * h
        clusters[a] = clusters[a] + clusters[b]
        del clusters[b]
    joins = O.guide_tree(D, O.TREE_UPGMA)
    assert np.all(np.diff(joins["height"]) > 0)
    assert sorted(int(x) for x in joins["height"]) == sorted(set(int(v) // 2 for v in D[np.triu_indices(n, 1)]))


def test_identity_distance():
    assert O.lib().tsqo_identity_distance(0, 0) == 1 << 32
    assert O.lib().tsqo_identity_distance(3, 4) == (1 << 32) // 4
    assert O.lib().tsqo_identity_distance(1, 3) == ((2 << 32) // 3)
    D = O.identity_distances(3, [1, 2, 3], [2, 2, 4])
    assert D[0, 1] == 1 << 31 and D[0, 2] == 0 and D[1, 2] == (1 << 32) // 4 and D[2, 1] == D[1, 2]


@pytest.mark.parametrize("method", [O.TREE_UPGMA, O.TREE_NJ])
def test_tree_text_and_leaf_order(method):
    """msa.Tree's Newick text and leaf order (host logic over the join list)
    on trees the oracle builds: every leaf once, one pair of parentheses per
    join, branch lengths as length / 2^32, and leaf order matching the
    Newick leaves read left to right."""
    import re

    from tweakseq_gb300 import msa

    rng = np.random.default_rng(41 + method)
    n = 23
    x = rng.random((n, 3))
    d = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
    D = np.round(d * (1 << 32)).astype(np.int64)
    nodes = O.guide_tree(D, method)
    tree = msa.Tree(n, nodes, "upgma" if method == O.TREE_UPGMA else "nj")
    labels = [f"s{k}" for k in range(n)]
    text = tree.newick(labels)
    assert text.endswith(";") and text.count("(") == text.count(")") == n - 1
    leaves = re.findall(r"[(,](s\d+):", text)
    assert sorted(leaves) == sorted(labels)
    assert [labels[k] for k in tree.leaf_order()] == leaves
    lengths = [float(v) for v in re.findall(r":(-?\d+\.\d+)", text)]
    want = sorted(float(f"{v / (1 << 32):.6f}") for v in np.concatenate([nodes["left_length"], nodes["right_length"]]))
    assert sorted(lengths) == want
    one = msa.Tree(1, np.zeros(0, dtype=O.TREE_NODE_DTYPE), "upgma")
    assert one.newick(["only"]) == "only;" and one.leaf_order() == [0]
