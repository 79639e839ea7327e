"""The reference's on-disk format (pyCudaPolygon.py:733-817: scalars.dat,
state.npy, arrays.npz) on the CUDA model, through the reference's save and
load logic (restated in tests/refdriver.py, since the reference's Python
layer does not travel to the GPU machine).

  * the reference's own saved state (tests/testSaver, copied byte for byte)
    loads: two pentagons, its positions, and the neighbour known answer of
    tests/neighborTesting.ipynb ({1: [7, 8]}, inside flags [True, False]);
  * saveModel then loadModel on a new model restores the polygons, positions,
    targets, stiffness and compressibility exactly, and the restored model
    evaluates the same records, energy and force.
"""
import os
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from pycudapolygon_gb300.systems import load_into, make_system  # noqa: E402
from refdriver import model  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def _evaluate(m):
    m.updatePolygonGeometry()
    m.updateNeighborCells()
    m.updateNeighbors()
    m.updateOutersections()
    m.updateForceEnergy()
    return (np.asarray(m.getIntersections(), dtype=np.uint64), m.getEnergy(),
            np.asarray(m.getForces()))


def test_load_reference_saved_state(tmp_path):
    d = tmp_path / "testSaver"
    shutil.copytree(os.path.join(HERE, "golden", "testSaver"), d)
    m = model()
    m.loadModel(str(d))          # its modelEnum "0" is not a name: the loader falls back to normal
    st = np.load(d / "state.npy")
    assert m.getNumVertices() == 10
    np.testing.assert_array_equal(m.getnArray(), [5, 5])
    np.testing.assert_array_equal(np.asarray(m.getPositions()), st[2:])
    m.setMaxEdgeLength(0.25)     # the notebook's cell size (tests/neighborTesting.ipynb:53)
    m.updateNeighborCells()
    m.updateNeighbors()
    assert {k: list(v) for k, v in m.getNeighbors().items()} == {1: [7, 8]}
    assert list(m.getInsideFlags()[1]) == [True, False]


def test_save_load_round_trip(tmp_path):
    s = make_system(64, 16, 0.85, seed=9)
    a = load_into(model(s.num_vertices), s)
    a.setStiffness(0.25)
    a.setCompressibility(0.5)
    a.shakeProject(100, 1e-15)
    keys_a, e_a, f_a = _evaluate(a)
    a.saveModel(str(tmp_path / "state"))
    with pytest.raises(Exception):
        a.saveModel(str(tmp_path / "state"))          # exists: refused without overwrite
    a.saveModel(str(tmp_path / "state"), overwrite=True)
    b = model()
    b.loadModel(str(tmp_path / "state"))
    assert b.getNumVertices() == s.num_vertices
    np.testing.assert_array_equal(b.getnArray(), s.n_array)
    np.testing.assert_array_equal(np.asarray(b.getPositions()), np.asarray(a.getPositions()))
    np.testing.assert_array_equal(b.getTargetAreas(), a.getTargetAreas())
    np.testing.assert_array_equal(b.getTargetEdgeLengths(), a.getTargetEdgeLengths())
    assert (b.getStiffness(), b.getCompressibility()) == (0.25, 0.5)
    assert b.getModelEnum() == "normal"
    keys_b, e_b, f_b = _evaluate(b)
    np.testing.assert_array_equal(keys_b, keys_a)
    assert e_b == pytest.approx(e_a, rel=1e-12)
    assert np.abs(f_b - f_a).max() <= 1e-10 * np.abs(f_a).max()
