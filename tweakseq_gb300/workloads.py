"""Seeded synthetic workloads for the five alignment configurations.

No public benchmark set is named for this path, so every workload is
synthetic, generated here from a fixed seed with the shapes, sizes and
residue distributions of the configurations:

* ``all_vs_all_proteins`` -- 64 proteins, lengths uniform 200..400, residues
  i.i.d. from the amino-acid background; all 2,016 unordered pairs.
* ``uneven_pairs`` -- 100,000 protein pairs, lengths log-normal (median 350,
  sigma 0.5) clipped to 50..2,000; the second sequence is derived from the
  first at a per-pair identity drawn uniformly from 30..90 % with 5 % single
  residue indels.
* ``long_dna_pairs`` -- DNA pairs, reference length uniform 10..50 kb over
  uniform ACGT; the query carries 10 % substitutions and 2 % indel events of
  geometric length (mean 3).
* ``guide_tree_families`` -- 4,000 proteins in 20 families (root length
  uniform 250..600) evolved down random binary trees, all-vs-all pairs.
* ``serving_stream`` -- Poisson arrivals of requests of 1..2,000 pairs
  (log-uniform), protein or DNA, lengths 50..5,000, traceback on half.

The amino-acid background is the table of Robinson & Robinson (1991), PNAS
88:8880-8884 (the frequencies BLAST uses for its composition statistics).

A workload is a ``PairSet``: one concatenated uint8 residue buffer plus, per
pair, the offset and length of each sequence in it.  That is the layout the
C ABI's batch entry point takes.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# Robinson & Robinson (1991) background frequencies, in percent.
AA_LETTERS = np.frombuffer(b"ARNDCQEGHILKMFPSTWYV", dtype=np.uint8)
AA_FREQ = np.array(
    [7.805, 5.129, 4.487, 5.364, 1.925, 4.264, 6.295, 7.377, 2.199, 5.142,
     9.019, 5.744, 2.243, 3.856, 5.203, 7.120, 5.841, 1.330, 3.216, 6.441])
AA_FREQ = AA_FREQ / AA_FREQ.sum()
DNA_LETTERS = np.frombuffer(b"ACGT", dtype=np.uint8)

BLOSUM62, DNA = 0, 1


@dataclass
class PairSet:
    """Pairs over one residue buffer (the batch layout of the C ABI)."""

    seqs: np.ndarray  # uint8, concatenated residues
    a_off: np.ndarray  # int64
    a_len: np.ndarray  # int32
    b_off: np.ndarray  # int64
    b_len: np.ndarray  # int32
    matrix: int = BLOSUM62
    gap_open: int = 11
    gap_extend: int = 1
    local: bool = False
    name: str = ""
    meta: dict = field(default_factory=dict)

    def __len__(self) -> int:
        return len(self.a_off)

    @property
    def cells(self) -> int:
        return int(np.dot(self.a_len.astype(np.int64), self.b_len.astype(np.int64)))

    def pair(self, k: int) -> tuple[bytes, bytes]:
        a = self.seqs[self.a_off[k]:self.a_off[k] + self.a_len[k]].tobytes()
        b = self.seqs[self.b_off[k]:self.b_off[k] + self.b_len[k]].tobytes()
        return a, b

    def subset(self, idx) -> "PairSet":
        idx = np.asarray(idx)
        return PairSet(self.seqs, self.a_off[idx], self.a_len[idx], self.b_off[idx], self.b_len[idx], self.matrix,
                       self.gap_open, self.gap_extend, self.local, self.name + "[subset]", dict(self.meta))


def _pairset_from_lists(seqs_list, pairs, **kw) -> PairSet:
    """Builds a PairSet from a list of byte strings and (i, j) index pairs."""
    lens = np.array([len(s) for s in seqs_list], dtype=np.int64)
    offs = np.zeros(len(seqs_list), dtype=np.int64)
    if len(seqs_list):
        offs[1:] = np.cumsum(lens)[:-1]
    buf = np.frombuffer(b"".join(seqs_list), dtype=np.uint8).copy() if seqs_list else np.zeros(0, np.uint8)
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    return PairSet(buf, offs[pairs[:, 0]], lens[pairs[:, 0]].astype(np.int32), offs[pairs[:, 1]],
                   lens[pairs[:, 1]].astype(np.int32), **kw)


_AA_CDF = np.cumsum(AA_FREQ)
_AA_CDF[-1] = 1.0


def random_protein(rng: np.random.Generator, n: int) -> np.ndarray:
    """n residues drawn i.i.d. from the background (inverse-CDF sampling)."""
    return AA_LETTERS[np.searchsorted(_AA_CDF, rng.random(n), side="right").clip(0, 19)]


def all_vs_all_proteins(n_seqs: int = 64, lo: int = 200, hi: int = 400, seed: int = 1) -> PairSet:
    """64 proteins, lengths U[200,400], all unordered pairs, global 11/1."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(lo, hi + 1, size=n_seqs)
    seqs = [random_protein(rng, int(L)).tobytes() for L in lens]
    iu, ju = np.triu_indices(n_seqs, k=1)
    return _pairset_from_lists(seqs, np.stack([iu, ju], 1), name=f"all_vs_all_{n_seqs}_proteins",
                               meta={"seed": seed, "n_seqs": n_seqs, "len_range": [lo, hi]})


def _mutate_proteins(rng, parents: np.ndarray, seg_len: np.ndarray, sub_rate: np.ndarray, indel_rate: float):
    """Vectorised point substitutions plus single-residue indels.

    parents: concatenated residues; seg_len: per-sequence lengths; sub_rate:
    per-sequence substitution probability.  Returns (children, child_lens)."""
    total = len(parents)
    seg_id = np.repeat(np.arange(len(seg_len)), seg_len)
    p_sub = sub_rate[seg_id]
    child = parents.copy()
    sub = rng.random(total) < p_sub
    child[sub] = random_protein(rng, int(sub.sum()))
    ev = rng.random(total)
    counts = np.ones(total, dtype=np.int64)
    counts[ev < indel_rate / 2] = 0  # deletion of this residue
    counts[(ev >= indel_rate / 2) & (ev < indel_rate)] = 2  # insertion after it
    out = np.repeat(child, counts)
    # The second copy of an inserted residue becomes a fresh random residue.
    ins_pos = np.cumsum(counts)[counts == 2] - 1
    out[ins_pos] = random_protein(rng, len(ins_pos))
    child_lens = np.add.reduceat(counts, np.concatenate([[0], np.cumsum(seg_len)[:-1]])) if total else seg_len * 0
    # Guard against a sequence deleted to nothing.
    return out, child_lens.astype(np.int64)


def uneven_pairs(n_pairs: int = 100_000, median: float = 350.0, sigma: float = 0.5, lo: int = 50, hi: int = 2000,
                 ident_lo: float = 0.30, ident_hi: float = 0.90, indel: float = 0.05, seed: int = 2) -> PairSet:
    """Protein pairs of log-normal length; partner at 30-90 % identity."""
    rng = np.random.default_rng(seed)
    lens = np.clip(np.rint(rng.lognormal(np.log(median), sigma, size=n_pairs)), lo, hi).astype(np.int64)
    first = random_protein(rng, int(lens.sum()))
    ident = rng.uniform(ident_lo, ident_hi, size=n_pairs)
    # A substituted residue is redrawn from the background, so it stays the
    # same letter with probability sum(f^2); correct for that.
    same = float(np.sum(AA_FREQ ** 2))
    sub_rate = np.clip((1.0 - ident) / (1.0 - same), 0.0, 1.0)
    second, lens2 = _mutate_proteins(rng, first, lens, sub_rate, indel)
    a_off = np.zeros(n_pairs, dtype=np.int64)
    a_off[1:] = np.cumsum(lens)[:-1]
    b_off = np.zeros(n_pairs, dtype=np.int64)
    b_off[1:] = np.cumsum(lens2)[:-1]
    b_off += len(first)
    seqs = np.concatenate([first, second])
    return PairSet(seqs, a_off, lens.astype(np.int32), b_off, lens2.astype(np.int32), name=f"uneven_pairs_{n_pairs}",
                   meta={"seed": seed, "median": median, "sigma": sigma, "clip": [lo, hi],
                         "identity": [ident_lo, ident_hi], "indel": indel})


def _mutate_dna(rng, ref: np.ndarray, sub: float, indel: float, mean_len: float) -> np.ndarray:
    """Substitutions (to one of the three other bases) at rate sub, and indel
    events at rate indel per position with geometric lengths (mean
    mean_len), half deletions and half insertions of random bases."""
    L = len(ref)
    q = ref.copy()
    m = rng.random(L) < sub
    shift = rng.integers(1, 4, size=int(m.sum()))
    idx = np.searchsorted(DNA_LETTERS, q[m])
    q[m] = DNA_LETTERS[(idx + shift) % 4]
    events = np.flatnonzero(rng.random(L) < indel)
    lens = rng.geometric(1.0 / mean_len, size=len(events))
    is_del = rng.random(len(events)) < 0.5
    # Deletions: mark [p, p + len) through a difference array.
    diff = np.zeros(L + 1, dtype=np.int64)
    np.add.at(diff, events[is_del], 1)
    np.add.at(diff, np.minimum(events[is_del] + lens[is_del], L), -1)
    keep = (np.cumsum(diff[:L]) == 0).astype(np.int64)
    # Insertions: repeat the base at p 1 + len times, then randomise the copies.
    counts = keep.copy()
    ins_at = events[~is_del]
    ins_len = lens[~is_del]
    ok = keep[ins_at] > 0
    np.add.at(counts, ins_at[ok], ins_len[ok])
    out = np.repeat(q, counts)
    ends = np.cumsum(counts)
    starts = ends - counts
    fresh = np.zeros(len(out), dtype=bool)
    for p, ln in zip(ins_at[ok], ins_len[ok]):
        fresh[starts[p] + 1:starts[p] + 1 + ln] = True
    out[fresh] = DNA_LETTERS[rng.integers(0, 4, size=int(fresh.sum()))]
    return out


def long_dna_pairs(n_pairs: int = 1000, lo: int = 10_000, hi: int = 50_000, sub: float = 0.10, indel: float = 0.02,
                   mean_indel: float = 3.0, seed: int = 3) -> PairSet:
    """DNA pairs, +2/-3, gap 5/2; query = mutated reference."""
    rng = np.random.default_rng(seed)
    seqs = []
    for _ in range(n_pairs):
        L = int(rng.integers(lo, hi + 1))
        ref = DNA_LETTERS[rng.integers(0, 4, size=L)]
        seqs.append(ref.tobytes())
        seqs.append(_mutate_dna(rng, ref, sub, indel, mean_indel).tobytes())
    pairs = np.arange(2 * n_pairs).reshape(-1, 2)
    return _pairset_from_lists(seqs, pairs, matrix=DNA, gap_open=5, gap_extend=2, name=f"long_dna_{n_pairs}",
                               meta={"seed": seed, "len_range": [lo, hi], "sub": sub, "indel": indel,
                                     "mean_indel": mean_indel})


def guide_tree_families(n_families: int = 20, per_family: int = 200, lo: int = 250, hi: int = 600,
                        indel: float = 0.03, seed: int = 4, all_pairs: bool = True) -> PairSet:
    """Protein families evolved down random binary trees; all-vs-all.

    Each family is an ultrametric random binary tree: the root sits at
    divergence 0.8 (expected substitutions per site from any leaf), every
    internal node somewhere between its parent and 0.26, leaves at 0.  A
    branch of length L replaces each residue with probability 1 - exp(-L)
    and carries indels in proportion to L (3 % over a root-to-leaf path).
    Two leaves differ by twice the height of their last common ancestor, so
    leaf pairs of a family fall between about 20 % identity (ancestor at the
    root) and 60 % (ancestor at 0.26); pairs from different families are
    unrelated."""
    rng = np.random.default_rng(seed)
    leaves = []
    same = float(np.sum(AA_FREQ ** 2))
    h_root, h_floor = 0.8, 0.26

    def branch(seq, length):
        p_sub = (1.0 - np.exp(-length)) / (1.0 - same)
        child, _ = _mutate_proteins(rng, seq, np.array([len(seq)]), np.array([min(1.0, p_sub)]),
                                    indel * length / h_root)
        return child if len(child) else random_protein(rng, 1)

    def grow(seq, k, h):
        if k == 1:
            leaves.append(seq.tobytes())
            return
        k1 = int(rng.integers(1, k))
        for kk in (k1, k - k1):
            h_child = 0.0 if kk == 1 else h - rng.uniform(0.0, 0.5) * (h - h_floor)
            grow(branch(seq, h - h_child), kk, h_child)

    for _ in range(n_families):
        grow(random_protein(rng, int(rng.integers(lo, hi + 1))), per_family, h_root)
    n = len(leaves)
    if all_pairs:
        iu, ju = np.triu_indices(n, k=1)
        pairs = np.stack([iu, ju], 1)
    else:
        pairs = np.zeros((0, 2), dtype=np.int64)
    ps = _pairset_from_lists(leaves, pairs, name=f"guide_tree_{n}",
                             meta={"seed": seed, "families": n_families, "per_family": per_family})
    ps.meta["n_seqs"] = n
    return ps


@dataclass
class Request:
    arrival_s: float
    pairs: PairSet
    traceback: bool


def serving_stream(n_requests: int, rate_per_s: float, max_pairs: int = 2000, lo: int = 50, hi: int = 5000,
                   seed: int = 5) -> list[Request]:
    """Poisson arrivals; each request is 1..max_pairs pairs (log-uniform),
    protein (BLOSUM62 11/1) or DNA (+2/-3, 5/2), lengths log-uniform
    lo..hi, traceback on half of the requests."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for _ in range(n_requests):
        t += rng.exponential(1.0 / rate_per_s)
        npairs = int(np.clip(np.rint(np.exp(rng.uniform(0, np.log(max_pairs)))), 1, max_pairs))
        dna = bool(rng.random() < 0.5)
        seqs = []
        for _ in range(npairs):
            L = int(np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
            if dna:
                ref = DNA_LETTERS[rng.integers(0, 4, size=L)]
                qry = _mutate_dna(rng, ref, 0.10, 0.02, 3.0)
            else:
                ref = random_protein(rng, L)
                qry, _ = _mutate_proteins(rng, ref, np.array([L]), np.array([0.5]), 0.05)
            if len(qry) == 0:
                qry = ref[:1]
            seqs += [ref.tobytes(), qry.tobytes()]
        kw = dict(matrix=DNA, gap_open=5, gap_extend=2) if dna else {}
        ps = _pairset_from_lists(seqs, np.arange(2 * npairs).reshape(-1, 2), name="request", **kw)
        reqs.append(Request(t, ps, bool(rng.random() < 0.5)))
    return reqs
