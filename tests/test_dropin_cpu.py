"""The reference's own, unchanged Python layer (pyCudaPolygon/pyCudaPolygon.py,
its mixins, enums.py, pyCudaPolygonLink.py) on top of this repository's
libpyCudaPolygon module.

The reference's checkout is needed (PCP_REFERENCE names its root); without
it the test is skipped.  It needs no GPU: it imports the reference's package
against the module (matplotlib, which the reference imports for plotting and
which is not installed, is replaced by an empty stand-in), checks that its
`model` class derives from the module's `Model`, that enums.py finds the
module's enums, and that every `lpcp.Model.<method>` the reference's Python
calls exists on the module -- except the three the reference's own module
does not bind either (initializeRandomSeed, getRandomSeed, getAreaPerOverlap,
absent from src/pybindWrapper.cpp), which must be absent here too.
"""
import importlib
import os
import re
import sys
import types

import pytest

import pycudapolygon_gb300 as pg

REF = os.environ.get("PCP_REFERENCE")
pytestmark = pytest.mark.skipif(not REF, reason="PCP_REFERENCE not set")

UNBOUND_IN_REFERENCE = {"initializeRandomSeed", "getRandomSeed", "getAreaPerOverlap"}


def _import_reference_package():
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", mpl.pyplot)
    pg.build()
    lib = pg.load_module()                 # our module first on sys.path
    pkg = os.path.join(REF, "pyCudaPolygon")
    if pkg not in sys.path:
        sys.path.insert(1, pkg)
    for name in ("pyCudaPolygon", "enums", "pyCudaPolygonLink", "polygonMixins"):
        sys.modules.pop(name, None)
    mod = importlib.import_module("pyCudaPolygon")
    return lib, mod


def test_reference_python_layer_runs_on_this_module():
    lib, mod = _import_reference_package()
    import enums
    import pyCudaPolygonLink
    assert pyCudaPolygonLink.libpyCudaPolygon is lib
    assert issubclass(mod.model, lib.Model)
    assert enums.modelEnum is lib.modelEnum and enums.minimizerEnum is lib.minimizerEnum
    called = set()
    for path in [os.path.join(REF, "pyCudaPolygon", "pyCudaPolygon.py")]:
        called |= set(re.findall(r"lpcp\.Model\.([A-Za-z_]\w*)", open(path).read()))
    assert len(called) > 50
    missing = sorted(n for n in called if not hasattr(lib.Model, n))
    assert set(missing) == UNBOUND_IN_REFERENCE, missing
    wrapper = open(os.path.join(REF, "src", "pybindWrapper.cpp")).read()
    for n in UNBOUND_IN_REFERENCE:
        assert '"%s"' % n not in wrapper
