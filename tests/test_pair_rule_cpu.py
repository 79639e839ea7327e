"""The pair-evaluation rule the benchmark counts (bench.candidate_pairs, the
broad phase's two tests restated in numpy): it must be conservative, so every
polygon pair that the oracle finds crossing is among the pairs handed to the
narrow phase, and the box test only removes pairs from the circle test's.
Systems whose polygons span less than 0.2 of the box (the benchmark's kind;
wider polygons are paired with every polygon on the device)."""
import numpy as np
import pytest

import bench
from oracle import oracle as orc
from pycudapolygon_gb300.systems import load_into, make_system


def _crossing_pairs(system):
    o = load_into(orc.OracleModel(system.num_vertices), system)
    o.updatePolygonGeometry()
    o.updateNeighborCells()
    o.updateNeighbors()
    o.updateOutersections()
    keys = o.getIntersections()
    sj = (keys >> np.uint64(48)).astype(np.int64)
    si = ((keys >> np.uint64(32)) & np.uint64(0xFFFF)).astype(np.int64)
    other = si != sj
    return {(int(min(a, b)), int(max(a, b))) for a, b in zip(si[other], sj[other])}


@pytest.mark.parametrize("P,n,phi,seed", [
    (64, 16, 0.85, 2),
    (96, 20, 0.97, 3),
    (200, 12, 0.90, 5),
    (120, "ragged", 0.88, 7),
])
def test_rule_keeps_every_crossing_pair(P, n, phi, seed):
    if n == "ragged":
        n = np.random.default_rng(seed).integers(5, 41, P)
    s = make_system(P, n, phi, seed=seed)
    crossing = _crossing_pairs(s)
    assert len(crossing) > 0
    pairs = []
    narrow, circle = bench.candidate_pairs(np.asarray(s.positions),
                                           np.asarray(s.start_indices), pairs)
    assert narrow == len(pairs) == len(set(pairs)) <= circle
    assert all(a < b for a, b in pairs)
    missing = crossing - set(pairs)
    assert not missing, sorted(missing)[:5]
    # the box test removes pairs that do not cross (it is why the count is
    # below the circle count)
    assert narrow < circle
