"""The stateless launchers of the C ABI (the replacements of the reference's
extern "C" wrappers of model.cu, declared at model.cpp:17-56) on
caller-owned device buffers, against the oracle: topology, polygon geometry,
edge-midpoint cells, force projection, SHAKE and the position update.  Two
systems: polygons of 16 vertices (the one-vertex-per-lane kernels) and of
48 (the warp-per-polygon kernels with a workspace)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pycudapolygon_gb300 as pg  # noqa: E402
from fire_shadow import wrapdiff  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from pycudapolygon_gb300 import cabi  # noqa: E402
from pycudapolygon_gb300.systems import load_into, make_system  # noqa: E402

pg.build()
L = cabi.lib()
D = ctypes.c_double


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _dev(a, dtype):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def _empty(n, dtype=torch.float64):
    return torch.empty(max(n, 1), dtype=dtype, device="cuda")


@pytest.mark.parametrize("P,n", [(64, 16), (24, 48)])
def test_stateless_launchers_match_the_oracle(P, n):
    s = make_system(P, n, 0.85, seed=11)
    V = s.num_vertices
    start_h = np.asarray(s.start_indices, dtype=np.int64)
    assert start_h.size == P + 1
    o = load_into(orc.OracleModel(V), s)
    pos = _dev(s.positions, torch.float64)
    start = _dev(start_h, torch.int32)

    # topology: shape id, next and previous vertex of each vertex
    sid, nxt, prv = (_empty(V, torch.int32) for _ in range(3))
    assert L.pcp_topology(_p(start), P, V, _p(sid), _p(nxt), _p(prv), None) == 0
    poly = np.repeat(np.arange(P), np.diff(start_h))
    loc = np.arange(V) - start_h[poly]
    nv = np.diff(start_h)[poly]
    torch.cuda.synchronize()
    assert np.array_equal(sid.cpu().numpy(), o.getShapeId())
    assert np.array_equal(nxt.cpu().numpy(), start_h[poly] + (loc + 1) % nv)
    assert np.array_equal(prv.cpu().numpy(), start_h[poly] + (loc - 1) % nv)

    # polygon geometry
    o.updatePolygonGeometry()
    el, cons = _empty(V), _empty(6 * V)
    areas, cx, cy, per = (_empty(P) for _ in range(4))
    mx = _empty(1)
    assert L.pcp_polygon_geometry(_p(pos), _p(start), P, V, _p(el), _p(areas), _p(cx), _p(cy),
                                  _p(per), _p(cons), _p(mx), None) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(areas.cpu().numpy(), o.getAreas(), rtol=1e-12)
    np.testing.assert_allclose(per.cpu().numpy(), o.getPerimeters(), rtol=1e-12)
    np.testing.assert_allclose(el.cpu().numpy(), o.getEdgeLengths(), rtol=1e-12)
    com = np.concatenate([cx.cpu().numpy(), cy.cpu().numpy()])
    assert np.abs(wrapdiff(com, o.getCOM())).max() < 1e-13
    np.testing.assert_allclose(cons.cpu().numpy(), o.getConstraints(), rtol=1e-10, atol=1e-13)
    assert float(mx.cpu()[0]) == pytest.approx(o.getMaxEdgeLength(), rel=1e-13)

    # edge-midpoint cells at the system's box size
    o.updateNeighborCells()
    B = o.getBoxSize()
    cell = _empty(V, torch.int32)
    assert L.pcp_neighbor_cells(_p(pos), _p(start), _p(sid), V, B, _p(cell), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(cell.cpu().numpy(), o.getNeighborCells())

    # projection of the oracle's overlap force, with the constraints above
    o.updateNeighbors()
    o.updateOutersections()
    o.updateForceEnergy()
    assert o.getNumIntersections() > 0
    f = _dev(o.getForces(), torch.float64)
    assert L.pcp_project_force(_p(pos), _p(start), P, _p(cons), _p(f), None) == 0
    o.projectForce()
    of = o.getForces()
    torch.cuda.synchronize()
    assert np.abs(f.cpu().numpy() - of).max() <= 1e-10 * np.abs(of).max()

    # the position update x = frac(x + dt F), from the projected force
    x0 = o.getPositions()
    o.setForces(f.cpu().numpy())          # the same force on both sides
    assert L.pcp_update_positions(_p(pos), _p(f), V, D(1e-3), None) == 0
    o.updatePositions(1e-3)
    torch.cuda.synchronize()
    assert np.abs(wrapdiff(pos.cpu().numpy(), o.getPositions())).max() <= 1e-15
    assert np.abs(wrapdiff(o.getPositions(), x0)).max() > 0

    # SHAKE onto the target edge lengths and areas
    tl = _dev(s.target_edge_lengths, torch.float64)
    ta = _dev(s.target_areas, torch.float64)
    it = torch.zeros(1, dtype=torch.int32, device="cuda")
    o.setPositions(pos.cpu().numpy())
    assert L.pcp_shake_project(_p(pos), _p(start), P, _p(tl), _p(ta), 100, D(1e-15), _p(it),
                               None) == 0
    it_o = o.shakeProject(100, 1e-15)
    torch.cuda.synchronize()
    assert abs(int(it.cpu()[0]) - it_o) <= 1 and it_o < 100
    assert np.abs(wrapdiff(pos.cpu().numpy(), o.getPositions())).max() < 1e-12


def test_stateless_launchers_refuse_offsets_that_are_not_csr():
    # every buffer is held in a variable for the whole call: the launchers
    # read the offsets back before deciding
    decreasing = _dev([0, 8, 4, 12], torch.int32)
    shifted = _dev([1, 4, 8, 12], torch.int32)
    pos = torch.zeros(24, dtype=torch.float64, device="cuda")
    force = torch.zeros(24, dtype=torch.float64, device="cuda")
    cons = torch.zeros(72, dtype=torch.float64, device="cuda")
    tl = torch.ones(3, dtype=torch.float64, device="cuda")
    ta = torch.ones(3, dtype=torch.float64, device="cuda")
    it = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert L.pcp_shake_project(_p(pos), _p(decreasing), 3, _p(tl), _p(ta), 10, D(1e-15), _p(it),
                               None) == 1
    assert b"never decrease" in L.pcp_last_error()
    assert L.pcp_project_force(_p(pos), _p(shifted), 3, _p(cons), _p(force), None) == 1
    assert b"begin at 0" in L.pcp_last_error()
    torch.cuda.synchronize()
    assert int(it.cpu()[0]) == 7          # nothing launched
