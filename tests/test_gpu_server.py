"""GPU tests of the served form (tsq_server_*): continuous batching with
HBM admission.  Each request's result must be identical whether it runs
alone or mixed with others that arrive while it is on the device."""
import threading
import time

import numpy as np
import pytest

from oracle import oracle as O
from tweakseq_gb300 import _native as N
from tweakseq_gb300 import aligner as A
from tweakseq_gb300 import build as B
from tweakseq_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    B.build()
    O.build()


def _protein_pairs(rng, n, lo, hi):
    seqs, pairs = [], []
    for k in range(n):
        a = W.random_protein(rng, int(rng.integers(lo, hi + 1)))
        b, _ = W._mutate_proteins(rng, a, np.array([len(a)]), np.array([0.5]), 0.05)
        if len(b) == 0:
            b = a[:1]
        seqs += [a.tobytes(), b.tobytes()]
        pairs.append((2 * k, 2 * k + 1))
    return W._pairset_from_lists(seqs, pairs)


def _dna_pairs(rng, n, lo, hi):
    seqs, pairs = [], []
    for k in range(n):
        a = W.DNA_LETTERS[rng.integers(0, 4, int(rng.integers(lo, hi + 1)))]
        seqs += [a.tobytes(), W._mutate_dna(rng, a, 0.1, 0.02, 3.0).tobytes()]
        pairs.append((2 * k, 2 * k + 1))
    return W._pairset_from_lists(seqs, pairs, matrix=W.DNA, gap_open=5, gap_extend=2)


def _requests(seed):
    """A mix of sizes and kinds: single editor realignments, protein score
    batches, DNA alignments with traceback, local identity batches."""
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(14):
        kind = k % 4
        if kind == 0:
            ps, kw = _protein_pairs(rng, 1, 100, 600), dict(output="alignment")
        elif kind == 1:
            ps, kw = _protein_pairs(rng, int(rng.integers(50, 800)), 30, 900), dict(output="score")
        elif kind == 2:
            ps = _dna_pairs(rng, int(rng.integers(1, 6)), 500, 3000)
            kw = dict(matrix="dna", gap_open=5, gap_extend=2, output="alignment", mode="local")
        else:
            ps, kw = _protein_pairs(rng, int(rng.integers(5, 60)), 50, 500), dict(output="identity", mode="local")
        reqs.append((ps, kw))
    return reqs


def _same(a, b):
    for f in ("score", "a_begin", "a_end", "b_begin", "b_end", "n_ident", "n_cols", "status"):
        if not np.array_equal(a.table[f], b.table[f]):
            return False
    return a.aln_a == b.aln_a and a.aln_b == b.aln_b


def test_each_result_is_the_same_alone_and_in_the_mix():
    reqs = _requests(3)
    alone = [A.align_batch(ps, **kw) for ps, kw in reqs]
    with A.Server(slots=3) as srv:
        # Requests alone through the server, one at a time.
        for (ps, kw), want in zip(reqs, alone):
            rid = srv.submit(ps, **kw)
            assert _same(srv.poll(rid), want)
        # The mix: half submitted at once, the rest arriving while the first
        # ones are on the device (from another host thread).
        ids = {}

        def late():
            for k in range(len(reqs) // 2, len(reqs)):
                time.sleep(0.002)
                ids[k] = srv.submit(reqs[k][0], **reqs[k][1])

        for k in range(len(reqs) // 2):
            ids[k] = srv.submit(reqs[k][0], **reqs[k][1])
        th = threading.Thread(target=late)
        th.start()
        th.join()
        for k in range(len(reqs)):
            assert _same(srv.poll(ids[k]), alone[k]), k
        st = srv.stats()
        assert st["completed"] == 2 * len(reqs) and st["p99_ms"] >= st["p50_ms"] > 0
    # And the alone results agree with the oracle (spot checks).
    for k in (0, 2):
        ps, kw = reqs[k]
        local = kw.get("mode") == "local"
        want, sa, sb = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, ps.matrix, ps.gap_open, ps.gap_extend,
                               local, O.MODE_ALIGN, 0, True)
        assert alone[k].aln_a == sa and np.array_equal(alone[k].table["score"], want["score"])


def test_admission_waits_for_memory_and_rejects_what_never_fits():
    rng = np.random.default_rng(8)
    # Alignments of long DNA pairs: traceback planes dominate the memory.
    # About 380 MB of planes and rows each against a 900 MB budget: at most
    # two requests can be on the device at once, so later ones must wait.
    reqs = [_dna_pairs(rng, 12, 7500, 8000) for _ in range(4)]
    alone = [A.align_batch(ps, matrix="dna", gap_open=5, gap_extend=2, output="alignment") for ps in reqs]
    budget = 900 << 20
    with A.Server(slots=4, hbm_budget_bytes=budget) as srv:
        big = _dna_pairs(rng, 40, 9000, 9500)  # about 1.7 GB of planes
        with pytest.raises(N.TsqError) as e:
            srv.submit(big, matrix="dna", gap_open=5, gap_extend=2, output="alignment")
        assert e.value.rc == N.E_REJECTED
        ids = [srv.submit(ps, matrix="dna", gap_open=5, gap_extend=2, output="alignment") for ps in reqs]
        for rid, want in zip(ids, alone):
            assert _same(srv.poll(rid), want)
        st = srv.stats()
        assert st["rejected"] == 1
        assert st["peak_reserved_bytes"] <= budget
        assert st["admission_waits"] > 0  # the requests could not all be admitted at once


def test_cancel_and_invalid_input():
    rng = np.random.default_rng(9)
    with A.Server(slots=1, hbm_budget_bytes=300 << 20) as srv:
        first = srv.submit(_dna_pairs(rng, 4, 3500, 4000), matrix="dna", gap_open=5, gap_extend=2,
                           output="alignment")
        waiting = srv.submit(_dna_pairs(rng, 4, 3500, 4000), matrix="dna", gap_open=5, gap_extend=2,
                             output="alignment")
        rc = srv.cancel(waiting)
        assert rc in (N.TSQ_OK, N.E_PENDING)
        if rc == N.TSQ_OK:
            with pytest.raises(N.TsqError) as e:
                srv.poll(waiting)
            assert e.value.rc == N.E_CANCELLED
        assert srv.poll(first) is not None
        bad = W._pairset_from_lists([b"ACDEFG", b"acdefg"], [(0, 1)])
        rid = srv.submit(bad, output="score")
        res = srv.poll(rid, check=False)
        assert res.table["status"].tolist() == [N.E_INVALID_RESIDUE]
        worse = W._pairset_from_lists([b"ACD", b"ACD"], [(0, 1)])
        worse.b_off = worse.b_off + 10
        with pytest.raises(N.TsqError) as e:
            srv.submit(worse, output="score")
        assert e.value.rc == N.E_INVALID_ARG
        assert srv.cancel(123456789) == N.E_NOT_FOUND


def _resident_requests(seed):
    """Requests for the device-resident loop (score and identity, pairs up
    to 2,048 residues, protein and DNA, global and local) mixed with ones it
    does not take (alignments, a pair longer than 2,048) and one with an
    invalid residue."""
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(16):
        kind = k % 5
        if kind == 0:
            ps, kw = _protein_pairs(rng, int(rng.integers(1, 40)), 20, 700), dict(output="score")
        elif kind == 1:
            ps, kw = _protein_pairs(rng, int(rng.integers(20, 300)), 50, 1200), dict(output="identity", mode="local")
        elif kind == 2:
            ps = _dna_pairs(rng, int(rng.integers(1, 30)), 100, 2000)
            kw = dict(matrix="dna", gap_open=5, gap_extend=2, output="score", mode="local")
        elif kind == 3:
            ps, kw = _protein_pairs(rng, int(rng.integers(1, 4)), 100, 400), dict(output="alignment")
        else:
            ps, kw = _protein_pairs(rng, int(rng.integers(5, 60)), 100, 1800), dict(output="identity")
        reqs.append((ps, kw))
    reqs.append((_protein_pairs(rng, 3, 2100, 2300), dict(output="score")))  # too long for the loop
    # A custom matrix scoring 25 per identical letter: in the loop, pairs
    # whose score bound passes 32767 run the checked int16x2 fill, and the
    # 1,400-residue W:W pair (35,000) comes near 32767 and re-runs in int32;
    # the 1,300-residue one (32,500) stays in int16x2.
    mat = np.full((26, 26), -2, dtype=np.int8)
    np.fill_diagonal(mat, 25)
    custom = (mat, np.ones(26, dtype=np.uint8))
    wseqs = [b"W" * 1400, b"W" * 1400, b"W" * 1300, b"W" * 1300]
    wpairs = [(0, 1), (2, 3)]
    for k in range(6):
        a = W.random_protein(rng, int(rng.integers(900, 2000))).tobytes()
        wseqs += [a, a[::-1]]
        wpairs.append((len(wseqs) - 2, len(wseqs) - 1))
    cps = W._pairset_from_lists(wseqs, wpairs)
    reqs.append((cps, dict(output="score", custom=custom)))
    reqs.append((cps, dict(output="identity", custom=custom)))
    # Lane choices reach the loop: int32 only, and checked int16x2 for all.
    reqs.append((_protein_pairs(rng, 20, 50, 900), dict(output="score", lane="i32")))
    reqs.append((_protein_pairs(rng, 20, 50, 900), dict(output="identity", lane="i16")))
    bad = W._pairset_from_lists([b"ACDEFGHIK", b"ACDEFGHIK", b"AC*EF"], [(0, 1), (0, 2)])
    reqs.append((bad, dict(output="score")))
    return reqs


def test_resident_loop_alone_and_in_the_mix():
    """With the device-resident loop, every request's results equal
    tsq_align_batch's on that request alone, submitted one at a time and
    all at once; the loop takes exactly the eligible requests."""
    reqs = _resident_requests(21)
    alone = [A.align_batch(ps, check=False, **kw) for ps, kw in reqs]
    eligible = sum(1 for ps, kw in reqs if kw["output"] != "alignment" and max(ps.a_len.max(), ps.b_len.max()) <= 2048)
    with A.Server(slots=2, resident=True) as srv:
        for (ps, kw), want in zip(reqs, alone):
            rid = srv.submit(ps, **kw)
            assert _same(srv.poll(rid, check=False), want)
        ids = [srv.submit(ps, **kw) for ps, kw in reqs]
        for k, rid in enumerate(ids):
            assert _same(srv.poll(rid, check=False), alone[k]), k
        st = srv.stats()
        assert st["resident_requests"] == 2 * eligible
        assert st["resident_launches"] >= 1
        assert st["completed"] == 2 * len(reqs)
    assert alone[-1].table["status"].tolist() == [0, N.E_INVALID_RESIDUE]


def test_resident_loop_idle_exit_and_relaunch():
    """The loop's kernel ends after its idle polls run out (a bounded wait,
    reported in mapped memory) and is relaunched by the next request, whose
    results are still exact."""
    rng = np.random.default_rng(22)
    ps = _protein_pairs(rng, 50, 50, 600)
    want = A.align_batch(ps, output="score")
    with A.Server(slots=1, resident=True, resident_idle_polls=200) as srv:
        assert _same(srv.poll(srv.submit(ps, output="score")), want)
        deadline = time.time() + 5.0
        while srv.stats()["resident_idle_exits"] < 1 and time.time() < deadline:
            time.sleep(0.01)
        st = srv.stats()
        assert st["resident_idle_exits"] >= 1
        launches = st["resident_launches"]
        assert _same(srv.poll(srv.submit(ps, output="score")), want)
        assert srv.stats()["resident_launches"] == launches + 1
