"""The CUDA library against the committed golden vectors of the oracle
(tests/golden/golden.json): occupancy, coordinates, the particle field and the
gridded field after every run are bit-identical."""
import os
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden as G  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = G.load()["cases"]


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_gpu_reproduces_golden(name):
    assert G.run_gpu(name) == GOLD[name]
