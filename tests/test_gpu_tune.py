"""GPU tests of the autotuner: a quick tuning run writes a table covering
every output kind, with a lane width, a lane type and a CTA choice per
length bucket; batches planned with it (and with hand-written tables that
force the int32 lanes and the CTA fill) stay bit-exact against the oracle."""
import json

import numpy as np
import pytest

from oracle import oracle as O
from tweakseq_gb300 import aligner as A
from tweakseq_gb300 import build as B
from tweakseq_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    B.build()
    O.build()
    yield
    # Leave no table in use for the tests that follow.
    import tempfile, os
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "empty.json")
        open(p, "w").write(json.dumps({"entries": []}))
        A.load_tuning(p)


def _mixed_pairs(seed):
    """Protein pairs of 20-1,500 residues plus a few long ones (2,000-3,500)
    that reach the CTA and overflow-checked paths."""
    rng = np.random.default_rng(seed)
    seqs, pairs = [], []
    for k in range(400):
        m = int(rng.integers(20, 1500)) if k >= 12 else int(rng.integers(2000, 3500))
        a = W.random_protein(rng, m)
        b, _ = W._mutate_proteins(rng, a, np.array([m]), np.array([0.6]), 0.05)
        seqs += [a.tobytes(), b.tobytes()]
        pairs.append((2 * k, 2 * k + 1))
    return W._pairset_from_lists(seqs, pairs)


def _check(ps, tuned_output, mode_name="global"):
    local = mode_name == "local"
    for output, omode in (("score", O.MODE_SCORE), ("identity", O.MODE_IDENT), ("alignment", O.MODE_ALIGN)):
        got = A.align_batch(ps, mode=mode_name, output=output, autotune=True)
        if omode == O.MODE_ALIGN:
            want, sa, sb = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, O.BLOSUM62, 11, 1, local, omode, 0,
                                   True)
            assert got.aln_a == sa and got.aln_b == sb, (tuned_output, output)
        else:
            want = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, O.BLOSUM62, 11, 1, local, omode)
        fields = ("score", "n_ident", "n_cols") if output != "score" else ("score",)
        for f in fields:
            assert np.array_equal(got.table[f], want[f]), (tuned_output, output, f)


def test_quick_tuning_then_tuned_batches_bit_exact(tmp_path):
    path = str(tmp_path / "tune.json")
    A.tune(path, quick=True)
    table = json.load(open(path))
    outs = {e["out"] for e in table["entries"]}
    assert outs == {"score", "identity", "alignment"}
    for e in table["entries"]:
        assert e["G"] in (4, 8, 16, 32) and e["i16"] in (0, 1) and e["cta"] in (0, 1) and e["gcups"] > 0
    A.load_tuning(path)
    _check(_mixed_pairs(3), "quick table")


def test_tables_forcing_int32_and_the_cta_fill(tmp_path):
    """Hand-written tables: int32 lanes and the CTA fill for every bucket,
    then int16x2 lanes with 32-lane groups; both bit-exact."""
    ps = _mixed_pairs(4)
    for i16, cta, G in ((0, 1, 8), (1, 0, 32)):
        entries = []
        for out in ("score", "identity", "alignment"):
            entries.append({"out": out, "lo": 0, "hi": 1 << 21, "G": G, "R": 8,
                            "i16": i16, "cta": cta, "gcups": 1.0})
        p = tmp_path / f"t{i16}{cta}.json"
        p.write_text(json.dumps({"entries": entries}))
        A.load_tuning(str(p))
        _check(ps, f"i16={i16} cta={cta}")
    _check(ps.subset(np.arange(60)), "local", "local")
