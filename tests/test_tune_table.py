"""CPU tests of the autotuner's table format (tsq_tune_load parses it on the
host; no device work): the lane width, lane type and CTA choice per length
bucket, tables written before the CTA choice existed, and malformed
entries."""
import json

import pytest

from tweakseq_gb300 import _native as N
from tweakseq_gb300 import build as B


@pytest.fixture(scope="module", autouse=True)
def lib():
    B.build()
    return N.lib()


def _write(tmp_path, entries):
    p = tmp_path / "tune.json"
    p.write_text(json.dumps({"device": "test", "sm": "10.3", "entries": entries}))
    return str(p).encode()


def test_table_with_lane_type_and_cta_loads(lib, tmp_path):
    entries = [{"out": "score", "lo": 0, "hi": 512, "G": 4, "R": 8, "i16": 1, "cta": 0, "gcups": 1.0},
               {"out": "score", "lo": 512, "hi": 4096, "G": 8, "R": 8, "i16": 0, "cta": 1, "gcups": 1.0},
               {"out": "identity", "lo": 0, "hi": 512, "G": 8, "R": 8, "i16": 1, "cta": 0, "gcups": 1.0},
               {"out": "alignment", "lo": 0, "hi": 1 << 21, "G": 32, "R": 8, "i16": 0, "cta": 1, "gcups": 1.0}]
    assert lib.tsq_tune_load(_write(tmp_path, entries)) == N.TSQ_OK
    # A table written before the CTA choice (no "cta" key) still loads.
    old = [{"out": "identity", "lo": 0, "hi": 2048, "G": 16, "R": 8, "i16": 0, "gcups": 1.0}]
    assert lib.tsq_tune_load(_write(tmp_path, old)) == N.TSQ_OK
    assert lib.tsq_tune_load(_write(tmp_path, [])) == N.TSQ_OK  # empty: no table in use


@pytest.mark.parametrize("bad", [
    {"cta": 2},                      # not a flag
    {"i16": 2},                      # not a flag
    {"R": 16},                       # rows per lane are fixed at 8
    {"G": 6},                        # no such lane width
    {"lo": 100, "hi": 100},          # empty bucket
    {"out": "trace"},                # unknown output kind
])
def test_malformed_entries_refused(lib, tmp_path, bad):
    e = {"out": "score", "lo": 0, "hi": 512, "G": 4, "R": 8, "i16": 0, "cta": 0, "gcups": 1.0}
    e.update(bad)
    assert lib.tsq_tune_load(_write(tmp_path, [e])) == N.E_INVALID_ARG
    assert lib.tsq_tune_load(_write(tmp_path, [])) == N.TSQ_OK
