"""The committed copy of the reference's saved-state fixture
(tests/golden/testSaver, pyCudaPolygon.py:733-817 format) agrees with the
JSON re-encoding the neighbour known-answer tests read, and, where the
reference checkout is available (PCP_REFERENCE), with the reference's files
byte for byte."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def test_testsaver_copy_matches_json():
    st = np.load(os.path.join(GOLD, "testSaver", "state.npy"))
    fx = json.load(open(os.path.join(GOLD, "testsaver.json")))
    scal = open(os.path.join(GOLD, "testSaver", "scalars.dat")).read().splitlines()
    kv = dict(line.split("\t") for line in scal)
    nv = int(kv["numVertices:"])
    assert nv == 10 and float(kv["maxEdgeLength:"]) == fx["max_edge_length_saved"]
    assert st[:-2 * nv].astype(int).tolist() == fx["n_array"]
    assert st[-2 * nv:].tolist() == fx["positions"]


def test_testsaver_copy_is_the_reference_file():
    ref = os.environ.get("PCP_REFERENCE")
    if not ref:
        pytest.skip("PCP_REFERENCE not set")
    for f in ("state.npy", "scalars.dat"):
        a = open(os.path.join(GOLD, "testSaver", f), "rb").read()
        b = open(os.path.join(ref, "tests", "testSaver", f), "rb").read()
        assert a == b
