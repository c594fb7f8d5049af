"""Host logic of the checkpointed reverse sweep, on CPU: which steps keep their
records when the last K segments' records are kept, and that the kept records
cover exactly the segments the reverse sweep then takes from them."""
import pytest

from _harness import jp  # noqa: F401  (puts the package on the path)
from justpic_gb300 import adjoint as A


@pytest.mark.parametrize("nsteps,k,K,first", [
    (100, 10, 1, 90), (100, 10, 5, 50), (100, 10, 10, 0), (100, 10, 12, 0),
    (12, 4, 1, 8), (12, 4, 2, 4), (12, 5, 1, 10), (12, 5, 2, 5), (7, 10, 1, 0),
    (100, 10, 0, 100), (0, 10, 3, 0), (9, 0, 1, 0),
])
def test_first_recorded_step(nsteps, k, K, first):
    assert A.first_recorded_step(nsteps, k, K) == first


@pytest.mark.parametrize("nsteps,k", [(100, 10), (12, 4), (12, 5), (7, 3), (1, 10)])
def test_kept_records_cover_whole_trailing_segments(nsteps, k):
    nseg = -(-nsteps // k)
    for K in range(1, nseg + 2):
        first = A.first_recorded_step(nsteps, k, K)
        assert first % k == 0  # a segment boundary
        kept = list(range(first, nsteps))
        covered = []
        for seg in range(nseg):  # the reverse sweep's slicing of the kept records
            n0, n1 = seg * k, min(seg * k + k, nsteps)
            if n0 >= first:
                covered += kept[n0 - first:n1 - first]
                assert kept[n0 - first:n1 - first] == list(range(n0, n1))
        assert covered == kept
        assert nseg - (nsteps - first + k - 1) // k == max(0, nseg - K)  # segments run again
