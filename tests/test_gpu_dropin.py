"""The reference's own, unchanged Python layer (pyCudaPolygon/pyCudaPolygon.py,
its mixins, enums.py, pyCudaPolygonLink.py) driving this repository's
libpyCudaPolygon module on the GPU.

`python oracle/ref_build.py stage` (PCP_REFERENCE naming a reference
checkout) copies those files into the git-ignored oracle/_ref/py/; the test
is skipped when they are not there.  The reference's package imports
matplotlib (plotting) and tqdm (progress bars); where either is not
installed an empty stand-in takes its place, since the minimiser uses
neither for its results.

A 64-polygon, 16-vertex system at packing fraction 0.85 is minimised by the
reference's own model.minimizeFIRE (pyCudaPolygon.py:674-731): its
initForceEnergy and small gradient step, then its per-step Python loop of
minimizeFIREStep and getMaxUnbalancedForce until |F|max <= 1e-10 or six
steps without an energy change.  Every step of that run is compared with one
oracle step started from the CUDA path's state, under the rules of
tests/fire_shadow.py.
"""
import importlib
import sys
import types

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from oracle import ref_build  # noqa: E402

PKG = ref_build.python_staged()
if PKG is None:
    pytest.skip("the reference's Python layer is not staged (oracle/ref_build.py stage)",
                allow_module_level=True)

import pycudapolygon_gb300 as pg  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from pycudapolygon_gb300.systems import load_into, make_system  # noqa: E402
from fire_shadow import FireShadow  # noqa: E402


class _Progress:
    """Stand-in for tqdm.tqdm (a progress bar with no output)."""

    def __init__(self, iterable=None, *a, **k):
        self.iterable = iterable

    def __iter__(self):
        return iter(self.iterable if self.iterable is not None else ())

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def update(self, n=1):
        pass


def _stand_ins():
    try:
        importlib.import_module("matplotlib.pyplot")
    except ImportError:
        mpl = types.ModuleType("matplotlib")
        mpl.pyplot = types.ModuleType("matplotlib.pyplot")
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.pyplot"] = mpl.pyplot
    try:
        importlib.import_module("tqdm")
    except ImportError:
        tq = types.ModuleType("tqdm")
        tq.tqdm = _Progress
        sys.modules["tqdm"] = tq


def _reference_package():
    _stand_ins()
    pg.build()
    lib = pg.load_module()                 # this repository's module, first on sys.path
    if PKG not in sys.path:
        sys.path.insert(1, PKG)
    for name in ("pyCudaPolygon", "enums", "pyCudaPolygonLink", "polygonMixins"):
        sys.modules.pop(name, None)
    return lib, importlib.import_module("pyCudaPolygon")


def test_reference_python_minimiser_runs_on_this_module():
    lib, ref = _reference_package()
    import pyCudaPolygonLink
    assert pyCudaPolygonLink.libpyCudaPolygon is lib
    assert issubclass(ref.model, lib.Model)
    s = make_system(64, 16, 0.85, seed=3)
    g = load_into(ref.model(s.num_vertices, seed=0), s)
    o = load_into(orc.OracleModel(s.num_vertices), s)
    for m in (g, o):
        m.shakeProject(100, 1e-15)
    sh = FireShadow(g, o, gstep=lambda *a: lib.Model.minimizeFIREStep(g, *a))
    g.minimizeFIREStep = sh.step           # the reference's loop calls self.minimizeFIREStep
    _, _, steps, shake_stats = g.minimizeFIRE(1e-10, 1e-3, 5000)
    assert 0 < steps < 5000 and sh.n == steps
    sh.check_counts()
    assert "reset" in sh.kinds and "advance" in sh.kinds
    assert shake_stats[2] >= shake_stats[0] >= 0
