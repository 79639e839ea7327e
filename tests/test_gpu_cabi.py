"""The C ABI driven directly with host buffers (pycudapolygon_gb300/cabi.py,
the way a cgo/JNI/ctypes caller binds include/pcp_gb300.h): contact search,
overlap force, projection and one FIRE step of a 48 x 12 system against the
oracle, the array getters' size query, and the status of calls with a NULL
output."""
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


def _load(system):
    c = cabi.CModel(system.num_vertices)
    c.set_num_vertices(system.num_vertices)
    c.set_start_indices(system.start_indices)
    c.set_positions(system.positions)
    c.set_target_areas(system.target_areas)
    c.set_target_edge_lengths(system.target_edge_lengths)
    c.initialize_neighbor_cells()
    c.set_max_edge_length(system.max_edge_length)
    return c


def test_c_abi_path_matches_the_oracle():
    s = make_system(48, 12, 0.85, seed=3)
    c = _load(s)
    o = load_into(orc.OracleModel(s.num_vertices), s)
    c.shake_project(100)
    o.shakeProject(100, 1e-15)
    assert np.abs(wrapdiff(c.positions(), o.getPositions())).max() <= 1e-12
    o.updatePolygonGeometry()
    o.updateNeighborCells()
    o.updateNeighbors()
    o.updateOutersections()
    o.updateForceEnergy()
    c.update_polygon_geometry()
    c.update_neighbor_cells()
    c.update_neighbors()
    c.update_outersections()
    c.update_force_energy()
    # records bit-exact, sorted the reference's way by both
    assert c.num_intersections() == o.getNumIntersections() > 0
    assert np.array_equal(c.intersections(), o.getIntersections())
    assert np.array_equal(c.outersections(), o.getOutersections())
    assert abs(c.energy() - o.getEnergy()) <= 1e-12 * abs(o.getEnergy())
    of = o.getForces()
    assert np.abs(c.forces() - of).max() <= 1e-10 * np.abs(of).max()
    c.project_force()
    o.projectForce()
    of = o.getForces()
    assert np.abs(c.forces() - of).max() <= 1e-10 * np.abs(of).max()
    ec = c.fire_step(1e-3, 0.1, 0)
    eo = o.minimizeFIREStep(1e-3, 0.1, 0)
    assert abs(ec[0] - eo[0]) <= 1e-9 * abs(eo[0]) + 1e-14
    assert ec[1:] == eo[1:]                         # dt, alpha, nPos
    assert np.abs(wrapdiff(c.positions(), o.getPositions())).max() <= 1e-12
    assert c.narrow_pair_total() > 0 and c.launch_count() > 0


def test_c_abi_size_query_and_null_outputs():
    s = make_system(16, 8, 0.8, seed=5)
    c = _load(s)
    L = c.L
    n = ctypes.c_int(-1)
    # a NULL array output asks for the element count only
    assert L.pcp_model_get_positions(c.h, None, 0, ctypes.byref(n)) == 0
    assert n.value == 2 * s.num_vertices
    small = np.zeros(4)
    assert L.pcp_model_get_positions(c.h, ctypes.c_void_p(small.ctypes.data), 4,
                                     ctypes.byref(n)) == 1
    assert b"needed" in L.pcp_last_error()
    # a scalar getter refuses a NULL output instead of writing through it
    for name in ["get_energy", "get_num_vertices", "get_pair_count", "get_narrow_pair_total",
                 "get_launch_count", "device_positions"]:
        assert getattr(L, "pcp_model_" + name)(c.h, None) == 1, name
        assert b"null output" in L.pcp_last_error()
    assert L.pcp_model_fire_status(c.h, None, None) == 1
    # and the handle still works
    assert c.energy() == c.energy()
    c.close()
