"""Host-side pieces of the learned warm start (pycudapolygon_gb300/warmstart.py):
the contact graph and the node features, on the oracle's records of a
64-polygon system (the tensor-core kernels themselves are tested in
test_gpu_warmstart.py)."""
import numpy as np
import pytest

pytest.importorskip("torch")

from oracle import oracle as orc  # noqa: E402
from pycudapolygon_gb300 import warmstart as ws  # noqa: E402
from pycudapolygon_gb300.systems import load_into, make_system  # noqa: E402


@pytest.fixture(scope="module")
def state():
    s = make_system(64, 16, 0.85, seed=2)
    o = load_into(orc.OracleModel(s.num_vertices), s)
    o.updatePolygonGeometry()
    o.updateNeighborCells()
    o.updateNeighbors()
    o.updateOutersections()
    o.updateForceEnergy()
    o.projectForce()
    return s, o


def test_contact_graph_is_symmetric_and_padded(state):
    s, o = state
    keys = o.getIntersections()
    assert keys.size > 0
    rowptr, col = ws.contact_graph(s.start_indices, keys, s.num_vertices)
    V = s.num_vertices
    Vp = rowptr.size - 1
    assert Vp % 128 == 0 and Vp >= V
    assert np.all(np.diff(rowptr) >= 0) and rowptr[-1] == col.size
    assert np.all(rowptr[V:] == rowptr[V])          # padding rows have no neighbours
    edges = set()
    for i in range(V):
        for j in col[rowptr[i]:rowptr[i + 1]]:
            edges.add((i, int(j)))
    assert all((j, i) in edges for i, j in edges)   # the neighbour sum is its own transpose
    start = s.start_indices
    for p in range(3):                                # ring neighbours are there
        a, b = int(start[p]), int(start[p + 1])
        for v in range(a, b):
            nxt = a + (v - a + 1) % (b - a)
            assert (v, nxt) in edges and (nxt, v) in edges
    # every crossing record joins the start vertices of its two edges
    k = keys[0]
    sj, si = int(k >> np.uint64(48)), int((k >> np.uint64(32)) & np.uint64(0xFFFF))
    i, j = int((k >> np.uint64(16)) & np.uint64(0xFFFF)), int(k & np.uint64(0xFFFF))
    assert (int(start[si]) + i, int(start[sj]) + j) in edges


def test_node_features(state):
    s, o = state
    keys = o.getIntersections()
    feats, scale = ws.node_features(o.getPositions(), s.start_indices, o.getForces(),
                                    o.getAreas(), s.target_areas, keys, s.num_vertices)
    V = s.num_vertices
    assert feats.shape == (ws._pad_rows(V), ws.FEATURES) and feats.dtype == np.float32
    assert np.all(np.isfinite(feats))
    assert np.all(feats[:V, 12] == 1.0) and np.all(feats[V:] == 0.0)
    assert scale == pytest.approx(np.sqrt(np.mean(s.target_areas)))
    # centroid-relative positions average to zero over each polygon
    st = s.start_indices
    for p in range(4):
        assert np.abs(feats[st[p]:st[p + 1], 0:2].mean(axis=0)).max() < 1e-5
    # the force column is scaled to a largest component of one
    assert np.abs(feats[:V, 6:8]).max() == pytest.approx(1.0)
    # crossings are counted on the vertices of crossing edges
    assert feats[:V, 11].sum() == pytest.approx(0.25 * 4 * keys.size)


def test_network_shapes_on_the_host():
    net = ws.WarmStartNet(seed=3, device="cpu")
    assert [tuple(w.shape) for w in net.W] == [(128, 16), (128, 256), (128, 256), (128, 256),
                                               (16, 128)]
    assert float(net.W[-1][2:].abs().sum()) == 0.0    # only two output columns are live
