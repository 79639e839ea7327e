"""Regenerate the golden fixtures in tests/golden/ from the reference.

Run where the reference tree is available, with PCP_REFERENCE set to its
root.  The fixtures it writes are committed, so nothing at test time reads the
reference:

  testSaver/        the reference's saved-state fixture files, byte for byte
  testsaver.json    the reference's own saved two-pentagon state
                    (tests/testSaver/state.npy, scalars.dat) and the neighbour
                    known answer of tests/neighborTesting.ipynb (cells 6, 9,
                    14: vertex 1 crosses 7 and 8, unchanged by a global shift)
  getdf.json        the reference's Python getDf (pyCudaPolygon.py:348-393)
                    on seeded non-degenerate edge pairs
  projection.json   the reference's getConstrainedForcePython
                    (pyCudaPolygon.py:441-487) on seeded polygon sets with
                    a random force
  com_area.json     getCentersOfMass (pyCudaPolygon.py:325-338) and the
                    unwrapped shoelace of setAreas (pyCudaPolygon.py:114-125)
  pybind_methods.json  the method names the reference binds on `Model`
                    (src/pybindWrapper.cpp:25-107)
  shape_setters.json   the reference's generateRandomPolygons
                    (polygonMixins/polygonUtils.py:61-89) from seeded
                    generators, and its setAreas, setBiPerimeters and setPhi
                    (pyCudaPolygon.py:103-234) run on a numpy stand-in for
                    the compiled model (signed shoelace areas)

The reference's model module imports matplotlib, tqdm and its compiled
`libpyCudaPolygon`; small stand-ins are put on sys.path for the import only.
The Python twins used here touch no compiled code.
"""
import importlib
import json
import os
import re
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("PCP_REFERENCE")
if not REF:
    raise SystemExit("set PCP_REFERENCE to the root of the reference checkout")


def _import_reference_model():
    """Import pyCudaPolygon/pyCudaPolygon.py with stand-ins for its imports."""
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)
    if "tqdm" not in sys.modules:
        try:
            importlib.import_module("tqdm")
        except ImportError:
            tq = types.ModuleType("tqdm")
            tq.tqdm = lambda *a, **k: None
            sys.modules["tqdm"] = tq
    lib = types.ModuleType("libpyCudaPolygon")

    class Model:  # base class placeholder; the twins below use no methods of it
        def __init__(self, *a, **k):
            pass

    class _Enum:
        pass

    lib.Model = Model
    lib.modelEnum = _Enum
    lib.minimizerEnum = _Enum
    sys.modules["libpyCudaPolygon"] = lib
    link = types.ModuleType("pyCudaPolygonLink")
    link.libpyCudaPolygon = lib
    sys.modules["pyCudaPolygonLink"] = link
    pkg_dir = os.path.join(REF, "pyCudaPolygon")
    sys.path.insert(0, pkg_dir)
    try:
        mod = importlib.import_module("pyCudaPolygon")
    finally:
        sys.path.remove(pkg_dir)
    return mod


class _FakeState:
    """Minimal stand-in exposing the getters the Python twins call."""

    def __init__(self, positions, start):
        self._pos = np.asarray(positions, dtype=np.float64)
        self._start = np.asarray(start, dtype=np.int64)

    def getStartIndices(self):
        return list(self._start)

    def getnArray(self):
        return np.diff(self._start)

    def getPositions(self):
        return self._pos.copy()

    def getNumPolygons(self):
        return len(self._start) - 1


def _star_polygons(rng, ns, radius=0.04):
    pos = []
    for n in ns:
        c = rng.random(2)
        th = rng.random() * 2 * np.pi
        k = np.arange(n)
        r = radius * (1 + 0.1 * rng.uniform(-1, 1, n))
        a = th + 2 * np.pi * k / n
        pts = np.stack([c[0] + r * np.cos(a), c[1] + r * np.sin(a)], axis=1) % 1.0
        pos.append(pts)
    pos = np.concatenate(pos)
    start = np.concatenate([[0], np.cumsum(ns)])
    return pos.reshape(-1), start


def _numpy_base_methods():
    """Methods of the compiled `Model` that the reference's shape setters
    call through `lpcp.Model.<name>(self, ...)`, on numpy state: positions,
    CSR starts, targets, the signed shoelace areas of updatePolygonGeometry
    (kernels.cuh:295-333) and a record of the calls that touch the device."""
    def shoelace_areas(self):
        xy = self._pos.reshape(-1, 2)
        out = []
        for p in range(len(self._start) - 1):
            poly = xy[self._start[p]:self._start[p + 1]]
            d = poly - poly[0]
            d = d - np.round(d)
            x, y = d[:, 0], d[:, 1]
            out.append(0.5 * (np.dot(x, np.roll(y, -1)) - np.dot(np.roll(x, -1), y)))
        return np.array(out)
    m = {
        "setMaxEdgeLength": lambda self, v: self._calls.append(("setMaxEdgeLength", float(v))),
        "initializeNeighborCells": lambda self: self._calls.append(("initializeNeighborCells",)),
        "updateNeighborCells": lambda self: None,
        "updateNeighbors": lambda self: None,
        "updatePolygonGeometry": lambda self: setattr(self, "_areas", shoelace_areas(self)),
        "getAreas": lambda self: list(self._areas),
        "getPositions": lambda self: list(self._pos),
        "setPositions": lambda self, p: setattr(self, "_pos", np.asarray(p, dtype=np.float64)),
        "getStartIndices": lambda self: list(self._start),
        "setStartIndices": lambda self, s: setattr(self, "_start", np.asarray(s, dtype=np.int64)),
        "getNumVertices": lambda self: int(self._start[-1]),
        "getNumPolygons": lambda self: len(self._start) - 1,
        "setTargetAreas": lambda self, a: setattr(self, "_ta", np.asarray(a, dtype=np.float64)),
        "getTargetAreas": lambda self: list(self._ta),
        "setTargetEdgeLengths": lambda self, a: setattr(self, "_tl", np.asarray(a, dtype=np.float64)),
        "getTargetEdgeLengths": lambda self: list(self._tl),
        "resetAreas": lambda self: self._calls.append(("resetAreas",)),
    }
    return m


def _shape_setter_cases(ref):
    """The reference's generator and shape setters on a numpy stand-in."""
    base = sys.modules["libpyCudaPolygon"].Model
    for name, fn in _numpy_base_methods().items():
        setattr(base, name, fn)

    class Stand(ref.model):
        def __init__(self, seed, start, positions=None):
            self.rng = np.random.default_rng(seed)
            self._start = np.asarray(start, dtype=np.int64)
            self._pos = np.zeros(2 * int(self._start[-1])) if positions is None else \
                np.asarray(positions, dtype=np.float64)
            self._ta = np.ones(len(start) - 1)
            self._tl = np.ones(len(start) - 1)
            self._calls = []

    out = {"source": "polygonMixins/polygonUtils.py:55-89 (generateRandomPolygons), "
                     "pyCudaPolygon.py:103-144 (setAreas), :182-203 (setBiPerimeters), "
                     ":223-234 (setPhi, the definition in effect)",
           "generator": [], "set_areas": [], "bi_perimeters": [], "set_phi": []}
    for seed, P, n in [(7, 6, 11), (123, 20, 16), (2024, 3, 5)]:
        st = Stand(seed, np.arange(P + 1) * n)
        ref.model.generateRandomPolygons(st, P, n)
        out["generator"].append({"seed": seed, "num_polygons": P, "n": n,
                                 "positions": st._pos.tolist()})
    rng = np.random.default_rng(99)
    for case in range(4):
        P = int(rng.integers(2, 9))
        ns = rng.integers(5, 30, size=P)
        positions, start = _star_polygons(rng, ns)
        targets = rng.uniform(5e-4, 3e-3, size=P)
        st = Stand(0, start, positions)
        ref.model.setAreas(st, targets)
        out["set_areas"].append({"positions": positions.tolist(), "start": start.tolist(),
                                 "targets": targets.tolist(), "result": st._pos.tolist()})
        st = Stand(0, start, positions)
        kappa = float(rng.uniform(3.6, 4.5))
        ref.model.setBiPerimeters(st, kappa, 1.4)
        out["bi_perimeters"].append({"positions": positions.tolist(), "start": start.tolist(),
                                     "kappa": kappa, "ratio": 1.4,
                                     "target_areas": st._ta.tolist(),
                                     "target_edge_lengths": st._tl.tolist(),
                                     "calls": [list(c) for c in st._calls]})
        st = Stand(0, start, positions)
        st._ta = rng.uniform(1e-3, 2e-3, size=P)
        st._tl = rng.uniform(0.01, 0.02, size=P)
        ta0, tl0 = st._ta.copy(), st._tl.copy()
        phi = float(rng.uniform(0.5, 0.9))
        ref.model.setPhi(st, phi)
        out["set_phi"].append({"positions": positions.tolist(), "start": start.tolist(),
                               "phi": phi, "target_areas_in": ta0.tolist(),
                               "target_edge_lengths_in": tl0.tolist(),
                               "target_areas": st._ta.tolist(),
                               "target_edge_lengths": st._tl.tolist(),
                               "calls": [list(c) for c in st._calls]})
    return out


def copy_testsaver():
    """The reference's saved-state fixture itself (tests/testSaver/state.npy and
    scalars.dat, the format of pyCudaPolygon.py:733-817), copied byte for
    byte to tests/golden/testSaver/ for the save/load tests."""
    import shutil
    out = os.path.join(HERE, "testSaver")
    os.makedirs(out, exist_ok=True)
    for f in ("state.npy", "scalars.dat"):
        shutil.copyfile(os.path.join(REF, "tests", "testSaver", f), os.path.join(out, f))


def main():
    ref = _import_reference_model()
    Model = ref.model
    rng = np.random.default_rng(20240611)

    # ---- testSaver fixture + neighbour known answer ----
    st = np.load(os.path.join(REF, "tests", "testSaver", "state.npy"))
    scal = open(os.path.join(REF, "tests", "testSaver", "scalars.dat")).read()
    nv = int(re.search(r"numVertices:\t(\d+)", scal).group(1))
    n_array = st[:-2 * nv].astype(int).tolist()
    pos = st[-2 * nv:].tolist()
    json.dump({
        "source": "tests/testSaver/state.npy, tests/testSaver/scalars.dat",
        "n_array": n_array, "positions": pos,
        "max_edge_length_saved": float(re.search(r"maxEdgeLength:\t([0-9.eE+-]+)", scal).group(1)),
        "notebook_max_edge_length": 0.25,
        "expected_neighbors": {"1": [7, 8]},
        "expected_inside": {"1": [True, False]},
        "answer_source": "tests/neighborTesting.ipynb cells 6, 9 and 14 ({1: [7, 8]}, "
                         "also after the global shift (pos - mean(pos)) % 1)",
    }, open(os.path.join(HERE, "testsaver.json"), "w"), indent=1)

    copy_testsaver()

    # ---- getDf twin ----
    cases = []
    for _ in range(64):
        while True:
            vi = rng.random(2)
            di = rng.uniform(-0.02, 0.02, 2)
            dj = rng.uniform(-0.02, 0.02, 2)
            vj = (vi + rng.uniform(-0.01, 0.01, 2)) % 1.0
            w = dj[0] * di[1] - dj[1] * di[0]
            if w * w > 1e-6 * np.dot(di, di) * np.dot(dj, dj):
                break
        vzi = (vi + di) % 1.0
        vzj = (vj + dj) % 1.0
        df = Model.getDf(None, vi, vzi, vj, vzj)
        cases.append({"vi": vi.tolist(), "vzi": vzi.tolist(), "vj": vj.tolist(),
                      "vzj": vzj.tolist(), "df": np.asarray(df).tolist()})
    json.dump({"source": "pyCudaPolygon/pyCudaPolygon.py:348-393 (model.getDf)",
               "cases": cases}, open(os.path.join(HERE, "getdf.json"), "w"))

    # ---- constrained force projection twin ----
    proj = []
    for case in range(12):
        P = int(rng.integers(1, 6))
        ns = rng.integers(3, 40, size=P) if case % 2 else np.full(P, int(rng.integers(3, 40)))
        positions, start = _star_polygons(rng, ns)
        force = rng.normal(size=positions.size)
        fake = _FakeState(positions, start)
        out = Model.getConstrainedForcePython(fake, force)
        proj.append({"positions": positions.tolist(), "start": start.tolist(),
                     "force": force.tolist(), "projected": np.asarray(out).tolist()})
    json.dump({"source": "pyCudaPolygon/pyCudaPolygon.py:441-487 "
                         "(model.getConstrainedForcePython)", "cases": proj},
              open(os.path.join(HERE, "projection.json"), "w"))

    # ---- centre of mass and shoelace twins ----
    comcases = []
    for case in range(8):
        P = int(rng.integers(1, 8))
        ns = rng.integers(3, 40, size=P)
        positions, start = _star_polygons(rng, ns)
        fake = _FakeState(positions, start)
        com = Model.getCentersOfMass(fake)
        # setAreas' unwrapped shoelace (pyCudaPolygon.py:114-125), per polygon
        areas = []
        pxy = positions.reshape(-1, 2)
        for p in range(P):
            poly = pxy[start[p]:start[p + 1]].copy()
            refv = poly[0].copy()
            for j in range(1, len(poly)):
                d = poly[j] - refv
                d = d - np.round(d)
                poly[j] = refv + d
            x, y = poly[:, 0], poly[:, 1]
            areas.append(0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(np.roll(x, -1), y)))
        comcases.append({"positions": positions.tolist(), "start": start.tolist(),
                         "com": np.asarray(com).tolist(), "areas": areas})
    json.dump({"source": "pyCudaPolygon/pyCudaPolygon.py:325-338 (getCentersOfMass), "
                         ":114-125 (setAreas shoelace)", "cases": comcases},
              open(os.path.join(HERE, "com_area.json"), "w"))

    # ---- pybind method table ----
    src = open(os.path.join(REF, "src", "pybindWrapper.cpp")).read()
    names = []
    for nm in re.findall(r'\.def\("([A-Za-z0-9_]+)"', src):
        if nm not in names:
            names.append(nm)
    enums = {}
    for enum_name, body in re.findall(r'enum_<[^>]+>\(m, "(\w+)"\)((?:\s*\.value\([^)]*\))+)', src):
        enums[enum_name] = re.findall(r'\.value\("(\w+)"', body)
    json.dump({"source": "src/pybindWrapper.cpp:12-108", "methods": names,
               "enums": enums}, open(os.path.join(HERE, "pybind_methods.json"), "w"),
              indent=1)
    # ---- generator and shape setters ----
    json.dump(_shape_setter_cases(ref), open(os.path.join(HERE, "shape_setters.json"), "w"))
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
