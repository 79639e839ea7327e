"""The generator and the setAreas rescaling (host-side numpy restatements in
pycudapolygon_gb300/systems.py) against the reference's own functions run
on the same inputs (tests/golden/shape_setters.json, written by
tests/golden/make_golden.py): polygonUtils.py:55-89 and
pyCudaPolygon.py:103-144.  No GPU."""
import json
import os

import numpy as np
import pytest

from pycudapolygon_gb300.systems import random_polygons, unwrapped_scale

FIX = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "shape_setters.json")))


@pytest.mark.parametrize("case", FIX["generator"], ids=lambda c: f"seed{c['seed']}")
def test_generator_matches_reference_draw_for_draw(case):
    got = random_polygons(np.random.default_rng(case["seed"]), case["num_polygons"], case["n"])
    np.testing.assert_array_equal(got, np.asarray(case["positions"]))


@pytest.mark.parametrize("case", FIX["set_areas"], ids=lambda c: f"P{len(c['start']) - 1}")
def test_set_areas_rescaling_matches_reference(case):
    got = unwrapped_scale(case["positions"], case["start"], np.asarray(case["targets"]))
    # np.dot (the shoelace) sums in the BLAS's order: last bits differ by platform
    np.testing.assert_allclose(got, np.asarray(case["result"]), rtol=0, atol=1e-13)
