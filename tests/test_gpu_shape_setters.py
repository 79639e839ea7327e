"""The generator and shape setters through the Python `model` class on the
GPU (pyCudaPolygon.py:103-234, polygonUtils.py:55-89), against the
reference's own functions run on the same inputs (tests/golden/
shape_setters.json).  Target areas derived from the device geometry agree
to 1e-12; the areas after the rescaling kernels agree with their targets."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pycudapolygon_gb300 as pg  # noqa: E402

pg.build()
from refdriver import model  # noqa: E402

FIX = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "shape_setters.json")))


def _loaded(case, seed=None):
    start = np.asarray(case["start"], dtype=np.int32)
    m = model(int(start[-1]), seed=seed)
    m.setNumVertices(int(start[-1]))
    m.setStartIndices(start)
    m.setPositions(np.asarray(case["positions"], dtype=np.float64))
    P = len(start) - 1
    m.setTargetAreas(np.ones(P))
    m.setTargetEdgeLengths(np.ones(P))
    m.initializeNeighborCells()
    return m


@pytest.mark.parametrize("case", FIX["generator"], ids=lambda c: f"seed{c['seed']}")
def test_generate_random_polygons(case):
    P, n = case["num_polygons"], case["n"]
    m = model(P * n, seed=case["seed"])
    m.setNumVertices(P * n)
    m.generateRandomPolygons(P, n)
    np.testing.assert_array_equal(np.asarray(m.getPositions()), np.asarray(case["positions"]))


@pytest.mark.parametrize("i", range(len(FIX["set_areas"])))
def test_set_areas(i):
    case = FIX["set_areas"][i]
    m = _loaded(case)
    m.setAreas(np.asarray(case["targets"]))
    # the shoelace's np.dot sums in the BLAS's order, which differs between
    # platforms in the last bits
    np.testing.assert_allclose(np.asarray(m.getPositions()), np.asarray(case["result"]),
                               rtol=0, atol=1e-13)
    np.testing.assert_allclose(np.abs(m.getAreas()), case["targets"], rtol=1e-10)


@pytest.mark.parametrize("i", range(len(FIX["bi_perimeters"])))
def test_set_bi_perimeters(i):
    case = FIX["bi_perimeters"][i]
    m = _loaded(case)
    m.setBiPerimeters(case["kappa"], case["ratio"])
    np.testing.assert_allclose(m.getTargetAreas(), case["target_areas"], rtol=1e-12)
    np.testing.assert_allclose(m.getTargetEdgeLengths(), case["target_edge_lengths"], rtol=1e-12)


@pytest.mark.parametrize("i", range(len(FIX["set_phi"])))
def test_set_phi(i):
    case = FIX["set_phi"][i]
    m = _loaded(case)
    m.setTargetAreas(np.asarray(case["target_areas_in"]))
    m.setTargetEdgeLengths(np.asarray(case["target_edge_lengths_in"]))
    m.setPhi(case["phi"])
    np.testing.assert_allclose(m.getTargetAreas(), case["target_areas"], rtol=1e-14)
    np.testing.assert_allclose(m.getTargetEdgeLengths(), case["target_edge_lengths"], rtol=1e-14)
    assert np.sum(m.getTargetAreas()) == pytest.approx(case["phi"], rel=1e-14)
    # resetAreas (kernels.cuh:1440-1455) scaled every polygon to its target
    np.testing.assert_allclose(np.abs(m.getAreas()), case["target_areas"], rtol=1e-10)


# ------------------------------------------------------------ GD minimiser
from oracle import oracle as orc  # noqa: E402
from pycudapolygon_gb300.systems import load_into, make_system  # noqa: E402


class _OracleGD(orc.OracleModel):
    """The oracle with the names the Python GD driver calls; the driver
    functions themselves are the package's, so both sides run the same
    sequence of model calls (pyCudaPolygon.py:573-647)."""

    def __init__(self, V, model_name):
        super().__init__(V)
        self._name = model_name

    def getModelEnum(self):
        return self._name

    def getnArray(self):
        return np.diff(self.getStartIndices())

    def getMaxEffectiveForce(self, dt, minimizerType="GD"):
        return orc.OracleModel.getMaxEffectiveForce(self, dt, minimizerType != "GD")

    minimizeGDStep = model.minimizeGDStep
    minimizeGD = model.minimizeGD
    getConstraintViolation = model.getConstraintViolation


@pytest.mark.parametrize("name,enum", [("normal", 0), ("softBody", 3), ("hybrid", 5)])
def test_gd_minimiser_parity(name, enum):
    s = make_system(64, 16, 0.85, seed=3)
    g = load_into(model(s.num_vertices), s)
    o = load_into(_OracleGD(s.num_vertices, name), s)
    g.setModelEnum(name)
    o.setModelEnum(enum)
    for m in (g, o):
        if name == "normal":
            m.shakeProject(200, 1e-15)
        else:
            m.setTargetAreas(s.target_areas * 1.05)
            m.setTargetEdgeLengths(s.target_edge_lengths * 0.97)
            m.setStiffness(1.0)
            m.setCompressibility(1.0)
    rg = g.minimizeGD(None, dt=1e-3, maxSteps=15, maxDisplacement=0.5)
    ro = o.minimizeGD(None, dt=1e-3, maxSteps=15, maxDisplacement=0.5)
    assert rg[0] == pytest.approx(ro[0], rel=1e-9, abs=1e-14)
    assert rg[1] == ro[1]
    d = (np.asarray(g.getPositions()) - o.getPositions() + 0.5) % 1.0 - 0.5
    assert np.abs(d).max() < 1e-10
