"""The oracle reproduces the committed golden digests (tests/golden/make_golden.py)."""
import json
import os

from tests.golden.make_golden import digests


def test_oracle_matches_golden():
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_small.json")
    want = json.load(open(path))
    got = digests()
    assert got == want
