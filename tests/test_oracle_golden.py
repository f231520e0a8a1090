"""The FP32 oracle on the 64x256 workload still gives the committed digests
(tests/golden/oracle_small.json, from tests/golden/make_oracle_golden.py):
particles, row counts, charge, potential and field after set-up and after
steps 1 and 10, and the counters of every step.  No GPU is needed."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "oracle_small.json")


def test_oracle_reproduces_committed_digests(oracle_mod):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_oracle_golden
    with open(GOLDEN) as f:
        gold = json.load(f)
    got = make_oracle_golden.oracle_run()
    assert got["stats"] == gold["stats"]
    for tag, st in gold["states"].items():
        assert got["states"][tag] == st, tag
