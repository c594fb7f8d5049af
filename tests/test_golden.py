"""The CPU oracle against the committed golden vectors (tests/golden/golden.json,
written by tests/golden/make_golden.py): any change of the oracle's results on
these seeded runs, on any machine, fails here."""
import os
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden as G  # noqa: E402

GOLD = G.load()["cases"]


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_oracle_reproduces_golden(name):
    assert G.run_oracle(name) == GOLD[name]
