"""The CPU oracle and the CUDA path against the reference's own GPU outputs.

tests/golden/ref_gpu_*.npz were written by tests/golden/make_ref_gpu_golden.py,
which ran the reference's unmodified src/model.cu and src/model.cpp (rebuilt
for sm_103a by oracle/ref_build.py) on seeded systems.  Each fixture holds the
inputs and what the reference's `Model` returned: geometry (model.cu:113-163),
the edge-midpoint cell list (model.cu:308-385), the neighbour slots of the
narrow phase (kernels.cuh:709-812), the sorted crossing records, exit partners
and crossing parameters (model.cpp:351-361), the overlap energy and force
(model.cpp:363-395), the projected force (model.cu:165-206), the grid overlap
estimate (model.cpp:824-847) and the soft-body terms.

Tolerances: integer and record data bit-exact (the crossing parameters are
float-rounded doubles and compared exactly too); areas 1e-12 relative; the
energy 1e-12 relative; forces 1e-10 of the largest component (the reference
sums with FP64 atomics in no fixed order); the projected force 1e-10 of the
largest component (the reference removes the span of the edge gradients by a
batched SVD, the oracle and the CUDA path by a direct solve).

The CPU tests pin the oracle; the tests marked gpu run the same comparison on
the CUDA path, so neither leans on the other.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as orc
from pycudapolygon_gb300.systems import PolygonSystem

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "ref_gpu_*.npz")))
NAMES = [os.path.basename(f)[len("ref_gpu_"):-4] for f in FIXTURES]

AREA_RTOL = 1e-12
ENERGY_RTOL = 1e-12
FORCE_RTOL = 1e-10
F_FORCE, F_PROJECT, F_MC, F_SOFT, F_HYBRID = 1, 2, 4, 8, 16


def load(name):
    z = np.load(os.path.join(HERE, "golden", "ref_gpu_%s.npz" % name))
    return {k: z[k] for k in z.files}


def system_of(fx):
    start = fx["in_start"].astype(np.int32)
    return PolygonSystem(positions=fx["in_positions"].astype(np.float64),
                         n_array=np.diff(start).astype(np.int32), start_indices=start,
                         target_areas=fx["in_target_areas"],
                         target_edge_lengths=fx["in_target_edge_lengths"],
                         max_edge_length=float(fx["in_max_edge_length"][0]), phi=0.0)


def configure(m, s):
    m.setNumVertices(s.num_vertices)
    m.setStartIndices(s.start_indices)
    m.setPositions(s.positions)
    m.setTargetAreas(s.target_areas)
    m.setTargetEdgeLengths(s.target_edge_lengths)
    m.initializeNeighborCells()
    m.setMaxEdgeLength(s.max_edge_length)
    return m


def slots(m, V):
    """Used neighbour slots, vertex-major: counts, neighbour ids, inside flags."""
    cnt = np.asarray(m.getNumNeighbors())
    if hasattr(m, "getNeighborSlots"):          # the oracle
        nb, ins = m.getNeighborSlots()
    else:                                       # the pybind Model: flat V*M lists
        nb = np.asarray(m.getNeighbors()).reshape(V, -1)
        ins = np.asarray(m.getInsideFlag()).reshape(V, -1)
    M = nb.shape[1]
    mask = np.arange(M)[None, :] < np.minimum(cnt, M)[:, None]
    return cnt, nb[mask], ins[mask].astype(np.uint8)


def assert_forces(got, ref):
    got = np.asarray(got, dtype=np.float64)
    scale = max(np.abs(ref).max(), 1e-300)
    err = np.abs(got - ref).max() / scale
    assert err <= FORCE_RTOL, err


def check(m, fx):
    """Run the reference's call sequence on `m` and compare with fixture `fx`."""
    s = system_of(fx)
    V = s.num_vertices
    flags = int(fx["in_flags"][0])
    configure(m, s)

    m.updatePolygonGeometry()
    np.testing.assert_allclose(m.getAreas(), fx["areas"], rtol=AREA_RTOL, atol=1e-18)
    d = (np.asarray(m.getCOM()) - fx["com"] + 0.5) % 1.0 - 0.5
    assert np.abs(d).max() < 1e-13
    np.testing.assert_allclose(m.getEdgeLengths(), fx["edge_lengths"], rtol=1e-15, atol=0)
    if "constraints" in fx:
        np.testing.assert_allclose(m.getConstraints(), fx["constraints"], rtol=1e-10,
                                   atol=1e-13, equal_nan=True)
    assert m.getMaxEdgeLength() == pytest.approx(float(fx["max_edge_length"][0]), rel=1e-15)

    m.updateNeighborCells()
    np.testing.assert_array_equal(m.getNeighborCells(), fx["cell_location"])
    np.testing.assert_array_equal(m.getNeighborIndices(), fx["neighbor_indices"])
    np.testing.assert_array_equal(m.getBoxCounts(), fx["box_counts"])

    m.updateNeighbors()
    cnt, nb, ins = slots(m, V)
    np.testing.assert_array_equal(cnt, fx["num_neighbors"])
    np.testing.assert_array_equal(nb, fx["neighbor_slots"])
    np.testing.assert_array_equal(ins, fx["inside_slots"])

    m.updateOutersections()
    assert m.getNumIntersections() == int(fx["num_intersections"][0])
    np.testing.assert_array_equal(np.asarray(m.getIntersections(), dtype=np.uint64),
                                  fx["intersections"])
    np.testing.assert_array_equal(np.asarray(m.getOutersections(), dtype=np.uint64),
                                  fx["outersections"])
    np.testing.assert_array_equal(np.asarray(m.getTU(), dtype=np.float64), fx["tu"])
    np.testing.assert_array_equal(np.asarray(m.getUT(), dtype=np.float64), fx["ut"])
    np.testing.assert_array_equal(m.getShapeCounts(), fx["shape_counts"])

    if flags & F_FORCE:
        m.updateForceEnergy()
        e = float(fx["energy"][0])
        assert m.getEnergy() == pytest.approx(e, rel=ENERGY_RTOL, abs=1e-300)
        assert_forces(m.getForces(), fx["forces"])
        if flags & F_PROJECT:
            m.projectForce()
            assert_forces(m.getForces(), fx["forces_projected"])
            assert m.getMaxUnbalancedForce() == pytest.approx(
                float(fx["max_unbalanced_force"][0]), rel=FORCE_RTOL)
    if flags & F_MC:
        pd = int(fx["in_point_density"][0])
        m.updateOverlapArea(pd)
        assert m.getOverlapArea() == float(fx["overlap_area"][0])
    if flags & (F_SOFT | F_HYBRID):
        m.setStiffness(float(fx["in_stiffness"][0]))
        m.setCompressibility(float(fx["in_compressibility"][0]))
    for flag, enum, key in ((F_SOFT, 3, "soft"), (F_HYBRID, 5, "hybrid")):
        if flags & flag:
            m.setModelEnum(enum)
            m.updateForceEnergy()
            assert m.getEnergy() == pytest.approx(float(fx[key + "_energy"][0]),
                                                  rel=ENERGY_RTOL, abs=1e-300)
            assert_forces(m.getForces(), fx[key + "_forces"])


def test_fixtures_present():
    """The reference's GPU outputs are committed (they pin the oracle)."""
    assert len(FIXTURES) >= 8, FIXTURES


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_gpu(name):
    fx = load(name)
    check(orc.OracleModel(int(fx["in_start"][-1])), fx)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_cuda_path_matches_reference_gpu(name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import pycudapolygon_gb300 as pg
    pg.build()
    lib = pg.load_module()

    class Adapter:
        """The pybind Model with the model enum taken as an int."""
        def __init__(self, size):
            self.m = lib.Model(size)

        def setModelEnum(self, e):
            self.m.setModelEnum(lib.modelEnum(e))

        def __getattr__(self, k):
            return getattr(self.m, k)
    fx = load(name)
    check(Adapter(int(fx["in_start"][-1])), fx)
