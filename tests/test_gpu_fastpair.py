"""GPU parity of FastPair (src/algorithm/neighbour/fastpair.rs:59-182): every
row's entry (nearest later row, distance in the element type) and the closest
pair equal to the oracle's step-by-step restatement and to the reference's
own known answers."""
import numpy as np
import pytest

import oracle
from smartcore_gb300.error import Failed
from smartcore_gb300.neighbors import FastPair, PairwiseDistance
from tests.datagen import blobs

pytestmark = pytest.mark.gpu


def test_reference_kats(kats):
    c = kats["fastpair"]
    fp = FastPair(np.array(c["x"]))
    for i, (node, neighbour, d) in c["distances"].items():
        e = fp.distances[int(i)]
        assert (e.node, e.neighbour) == (node, neighbour)
        assert e.distance == (np.finfo(np.float64).max if d == float("inf") else d)
    for case in c["closest"].values():
        a, b, d = case["expect"]
        assert FastPair(np.array(case["x"])).closest_pair() == PairwiseDistance(a, b, d)
    with pytest.raises(Failed, match=c["error"]):
        FastPair(np.zeros((2, 2)))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("n,d", [(3, 1), (700, 5), (2000, 16), (1500, 40)])
def test_matches_oracle(dtype, n, d):
    x, _ = blobs(n, d, 7, seed=n + d, dtype=dtype)
    fp = FastPair(x)
    nb, dist, closest = oracle.fastpair(x)
    assert [fp.distances[i].neighbour for i in range(n)] == nb.tolist()
    assert np.array_equal(np.array([fp.distances[i].distance for i in range(n)]), dist)
    c = fp.closest_pair()
    assert (c.node, c.neighbour, c.distance) == closest


def test_duplicates_and_ties():
    # integer grid with duplicates: exact ties between later rows go to the lowest index
    rng = np.random.default_rng(9)
    x = rng.integers(0, 5, size=(1200, 3)).astype(np.float32)
    fp = FastPair(x)
    nb, dist, closest = oracle.fastpair(x)
    assert [fp.distances[i].neighbour for i in range(len(x))] == nb.tolist()
    assert (fp.closest_pair().node, fp.closest_pair().neighbour) == closest[:2]
