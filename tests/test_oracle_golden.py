"""The CPU oracle against the reference's own known answers and Python twins
(fixtures made by tests/golden/make_golden.py from the reference tree)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc


def _load(golden_dir, name):
    return json.load(open(os.path.join(golden_dir, name)))


def _testsaver_model(fx, positions=None):
    pos = np.asarray(fx["positions"] if positions is None else positions)
    n_array = np.asarray(fx["n_array"])
    V = int(n_array.sum())
    m = orc.OracleModel(V)
    m.setNumVertices(V)
    m.setStartIndices(np.concatenate([[0], np.cumsum(n_array)]))
    m.setPositions(pos)
    # neighborTesting.ipynb cell 3: setMaxEdgeLength(0.25), initializeNeighborCells
    # (whose Python wrapper then resets maxEdgeLength to 0.5, pyCudaPolygon.py:54-57)
    m.setMaxEdgeLength(fx["notebook_max_edge_length"])
    m.initializeNeighborCells()
    m.setMaxEdgeLength(0.5)
    m.updateNeighborCells()
    m.updateNeighbors()
    return m


def test_testsaver_neighbour_known_answer(golden_dir):
    fx = _load(golden_dir, "testsaver.json")
    m = _testsaver_model(fx)
    nb = {int(k): v.tolist() for k, v in m.getNeighbors().items()}
    assert nb == {int(k): v for k, v in fx["expected_neighbors"].items()}
    ins = {int(k): v.tolist() for k, v in m.getInsideFlags().items()}
    assert ins == {int(k): v for k, v in fx["expected_inside"].items()}


def test_testsaver_shift_invariance(golden_dir):
    fx = _load(golden_dir, "testsaver.json")
    pos = np.asarray(fx["positions"]).reshape(-1, 2)
    shifted = ((pos - pos.mean(axis=0)) % 1.0).reshape(-1)
    m = _testsaver_model(fx, shifted)
    nb = {int(k): v.tolist() for k, v in m.getNeighbors().items()}
    assert nb == {int(k): v for k, v in fx["expected_neighbors"].items()}


@pytest.mark.parametrize("B", [1, 2, 3, 4, 5])
def test_testsaver_any_cell_size(golden_dir, B):
    """The crossing set does not depend on the cell grid while the cells are
    at least one edge long."""
    fx = _load(golden_dir, "testsaver.json")
    m = _testsaver_model(fx)
    m.setMaxEdgeLength(1.0 / B)
    m.updateNeighborCells()
    m.updateNeighbors()
    nb = {int(k): v.tolist() for k, v in m.getNeighbors().items()}
    assert nb == {1: [7, 8]}


def test_getdf_matches_python_twin(golden_dir):
    fx = _load(golden_dir, "getdf.json")
    for c in fx["cases"]:
        got = orc.getDf(c["vi"], c["vzi"], c["vj"], c["vzj"])
        want = np.asarray(c["df"])
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())


def test_projection_matches_python_twin(golden_dir):
    fx = _load(golden_dir, "projection.json")
    for c in fx["cases"]:
        pos = np.asarray(c["positions"])
        start = np.asarray(c["start"])
        V = int(start[-1])
        m = orc.OracleModel(V)
        m.setNumVertices(V)
        m.setStartIndices(start)
        m.setPositions(pos)
        m.initializeNeighborCells()
        m.updatePolygonGeometry()
        m.setForces(np.asarray(c["force"]))
        m.projectForce()
        got = m.getForces()
        want = np.asarray(c["projected"])
        scale = np.abs(np.asarray(c["force"])).max()
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-10 * scale)


def test_com_and_area_match_python_twins(golden_dir):
    fx = _load(golden_dir, "com_area.json")
    for c in fx["cases"]:
        pos = np.asarray(c["positions"])
        start = np.asarray(c["start"])
        V = int(start[-1])
        P = start.size - 1
        m = orc.OracleModel(V)
        m.setNumVertices(V)
        m.setStartIndices(start)
        m.setPositions(pos)
        m.initializeNeighborCells()
        m.updatePolygonGeometry()
        com = m.getCOM()
        want = np.asarray(c["com"]).reshape(P, 2)
        got = np.stack([com[:P], com[P:]], axis=1)
        d = (got - want + 0.5) % 1.0 - 0.5      # the CUDA COM is wrapped into [0,1)
        assert np.abs(d).max() < 1e-12
        np.testing.assert_allclose(np.abs(m.getAreas()), c["areas"], rtol=1e-12)


def test_wrap_range():
    for x in [-1.7, -0.5, -0.25, 0.0, 0.25, 0.4999, 0.5, 0.75, 1.3]:
        w = orc.wrap(x)
        assert -0.5 <= w < 0.5
        assert abs(((x - w) + 0.5) % 1.0 - 0.5) < 1e-15
