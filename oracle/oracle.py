"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE).

`OracleModel` exposes the oracle (oracle/pcp_oracle.c) with the method names
of the reference's pybind `Model` (src/pybindWrapper.cpp:25-107), so a test
can drive the CUDA model and the oracle with the same call sequence.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU legs import this module.
Its SHAKE and FIRE parts are parity unpinned (the reference ships no source
for them); the rest is pinned as pcp_oracle.c's header says.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        D = ctypes.c_double
        I = ctypes.c_int
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        sig = {
            "orc_wrap": (D, [D]),
            "orc_h": (D, [dp, dp, dp]),
            "orc_g12": (None, [dp, dp, dp, dp, dp]),
            "orc_getDf": (None, [dp, dp, dp, dp, dp]),
            "orc_cross": (I, [dp, dp, dp, dp, dp, dp, dp]),
            "orc_midpoint_cell": (I, [dp, ip, ip, I, I, I]),
            "orc_create": (P, [I]),
            "orc_destroy": (None, [P]),
            "orc_set_threads": (None, [I]),
            "orc_set_num_vertices": (None, [P, I]),
            "orc_set_positions": (I, [P, dp, I]),
            "orc_set_forces": (None, [P, dp, I]),
            "orc_set_velocities": (None, [P, dp, I]),
            "orc_set_energy": (None, [P, D]),
            "orc_set_start_indices": (None, [P, ip, I]),
            "orc_set_target_areas": (None, [P, dp, I]),
            "orc_set_target_edge_lengths": (None, [P, dp, I]),
            "orc_set_max_edge_length": (None, [P, D]),
            "orc_set_model_enum": (None, [P, I]),
            "orc_set_stiffness": (None, [P, D]),
            "orc_set_compressibility": (None, [P, D]),
            "orc_initialize_neighbor_cells": (None, [P]),
            "orc_update_polygon_geometry": (None, [P]),
            "orc_update_neighbor_cells": (None, [P]),
            "orc_update_neighbors": (I, [P]),
            "orc_update_outersections": (None, [P]),
            "orc_update_force_energy": (None, [P]),
            "orc_project_force": (None, [P]),
            "orc_shake_project": (I, [P, I, D]),
            "orc_update_overlap_area": (D, [P, I]),
            "orc_xpbd_project": (I, [P, I, D]),
            "orc_update_positions": (None, [P, D]),
            "orc_reset_velocities": (None, [P]),
            "orc_reset_areas": (None, [P]),
            "orc_save_tentative_positions": (None, [P]),
            "orc_get_max_effective_force": (D, [P, D, I]),
            "orc_get_max_unbalanced_force": (D, [P]),
            "orc_fire_step": (None, [P, D, D, I, D, D, D, D, D, I, I, dp]),
            "orc_minimize_fire": (None, [P, D, D, I, D, D, D, D, D, I, I, dp]),
        }
        for name in ["orc_num_vertices", "orc_num_polygons", "orc_num_intersections",
                     "orc_max_neighbors", "orc_box_size", "orc_last_shake_iters",
                     "orc_fire_first_shake_iters"]:
            sig[name] = (I, [P])
        for name in ["orc_energy", "orc_max_edge_length"]:
            sig[name] = (D, [P])
        for name in ["orc_positions", "orc_forces", "orc_velocities", "orc_areas",
                     "orc_com_x", "orc_com_y", "orc_edge_lengths", "orc_constraints",
                     "orc_perimeters", "orc_tu", "orc_ut", "orc_target_areas",
                     "orc_target_edge_lengths"]:
            sig[name] = (dp, [P])
        for name in ["orc_shape_id", "orc_cell_location", "orc_neighbor_indices",
                     "orc_box_starts", "orc_neighbors", "orc_num_neighbors",
                     "orc_shape_counts", "orc_start_indices"]:
            sig[name] = (ip, [P])
        sig["orc_inside"] = (ctypes.POINTER(ctypes.c_uint8), [P])
        sig["orc_intersections"] = (ctypes.POINTER(ctypes.c_uint64), [P])
        sig["orc_outersections"] = (ctypes.POINTER(ctypes.c_uint64), [P])
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _copy(ptr, n, dtype):
    if n <= 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def set_threads(n):
    lib().orc_set_threads(int(n))


# ---- stateless helpers (kernels.cuh:115-222) ----
def wrap(x):
    return lib().orc_wrap(float(x))


def getDf(vi, vzi, vj, vzj):
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (vi, vzi, vj, vzj)]
    out = np.zeros(16)
    lib().orc_getDf(*[_dptr(v) for v in a], _dptr(out))
    # df[col*2 + row] -> (2, 8) matrix like the reference's Python twin
    return out.reshape(8, 2).T.copy()


def h(pt1, pt2, sp):
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (pt1, pt2, sp)]
    return lib().orc_h(*[_dptr(v) for v in a])


def g12(pt1, pt2, sp):
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (pt1, pt2, sp)]
    g1 = np.zeros(2)
    g2 = np.zeros(2)
    lib().orc_g12(*[_dptr(v) for v in a], _dptr(g1), _dptr(g2))
    return g1, g2


MODEL_ENUM = {"normal": 0, "edgeOnly": 1, "areaOnly": 2, "softBody": 3,
              "abnormal": 4, "hybrid": 5}


class OracleModel:
    """CPU oracle with the reference `Model` method names (model.hpp:18-107)."""

    def __init__(self, size=0):
        self._L = lib()
        self._m = self._L.orc_create(int(size))

    def __del__(self):
        try:
            if self._m:
                self._L.orc_destroy(self._m)
                self._m = None
        except Exception:
            pass

    # setters
    def setNumVertices(self, n):
        self._L.orc_set_num_vertices(self._m, int(n))

    def setPositions(self, pos):
        a = np.ascontiguousarray(pos, dtype=np.float64)
        return self._L.orc_set_positions(self._m, _dptr(a), int(a.size))

    def setForces(self, f):
        a = np.ascontiguousarray(f, dtype=np.float64)
        self._L.orc_set_forces(self._m, _dptr(a), int(a.size))

    def setVelocities(self, v):
        """FIRE state from another implementation (test use only)."""
        a = np.ascontiguousarray(v, dtype=np.float64)
        self._L.orc_set_velocities(self._m, _dptr(a), int(a.size))

    def setEnergy(self, e):
        """Energy the next FIRE step takes as its start energy (test use only)."""
        self._L.orc_set_energy(self._m, float(e))

    def setStartIndices(self, si):
        a = np.ascontiguousarray(si, dtype=np.int32)
        self._L.orc_set_start_indices(self._m, _iptr(a), int(a.size))

    def setTargetAreas(self, v):
        a = np.ascontiguousarray(v, dtype=np.float64)
        self._L.orc_set_target_areas(self._m, _dptr(a), int(a.size))

    def setTargetEdgeLengths(self, v):
        a = np.ascontiguousarray(v, dtype=np.float64)
        self._L.orc_set_target_edge_lengths(self._m, _dptr(a), int(a.size))

    def setMaxEdgeLength(self, v):
        self._L.orc_set_max_edge_length(self._m, float(v))

    def setModelEnum(self, e):
        if isinstance(e, str):
            e = MODEL_ENUM[e]
        self._L.orc_set_model_enum(self._m, int(e))

    def setStiffness(self, k):
        self._L.orc_set_stiffness(self._m, float(k))

    def setCompressibility(self, c):
        self._L.orc_set_compressibility(self._m, float(c))

    # updaters
    def initializeNeighborCells(self):
        self._L.orc_initialize_neighbor_cells(self._m)

    def updatePolygonGeometry(self):
        self._L.orc_update_polygon_geometry(self._m)

    def updateNeighborCells(self):
        self._L.orc_update_neighbor_cells(self._m)

    def updateNeighbors(self):
        return self._L.orc_update_neighbors(self._m)

    def updateOutersections(self):
        self._L.orc_update_outersections(self._m)

    def updateForceEnergy(self):
        self._L.orc_update_force_energy(self._m)

    def projectForce(self):
        self._L.orc_project_force(self._m)

    def updateOverlapArea(self, pointDensity):
        self._overlap = self._L.orc_update_overlap_area(self._m, int(pointDensity))

    def getOverlapArea(self):
        return self._overlap

    def shakeProject(self, nIter=100, tol=1e-15):
        return self._L.orc_shake_project(self._m, int(nIter), float(tol))

    def xpbdProject(self, nIter=100, tol=0.0):
        return self._L.orc_xpbd_project(self._m, int(nIter), float(tol))

    def updatePositions(self, dt):
        self._L.orc_update_positions(self._m, float(dt))

    def resetVelocities(self):
        self._L.orc_reset_velocities(self._m)

    def resetAreas(self):
        self._L.orc_reset_areas(self._m)

    def saveTentativePositions(self):
        self._L.orc_save_tentative_positions(self._m)

    def getMaxEffectiveForce(self, dt, fire=False):
        return self._L.orc_get_max_effective_force(self._m, float(dt), int(bool(fire)))

    def minimizeFIREStep(self, dt, alpha, nPos, dtMax=0.1, alphaStart=0.1, fAlpha=0.99,
                         fInc=1.1, fDec=0.5, nMin=5, shakeIter=5):
        out = np.zeros(4)
        self._L.orc_fire_step(self._m, dt, alpha, int(nPos), dtMax, alphaStart, fAlpha,
                              fInc, fDec, int(nMin), int(shakeIter), _dptr(out))
        return float(out[0]), float(out[1]), float(out[2]), int(out[3])

    def minimizeFIRE(self, thr, dt0, maxSteps, dtMax=0.1, alphaStart=0.1, fAlpha=0.99,
                     fInc=1.1, fDec=0.5, nMin=5, shakeIter=5):
        out = np.zeros(3)
        self._L.orc_minimize_fire(self._m, thr, dt0, int(maxSteps), dtMax, alphaStart,
                                  fAlpha, fInc, fDec, int(nMin), int(shakeIter), _dptr(out))
        return float(out[0]), float(out[1]), int(out[2])

    # getters
    def getNumVertices(self):
        return self._L.orc_num_vertices(self._m)

    def getNumPolygons(self):
        return self._L.orc_num_polygons(self._m)

    def getNumIntersections(self):
        return self._L.orc_num_intersections(self._m)

    def getMaxNeighbors(self):
        return self._L.orc_max_neighbors(self._m)

    def getBoxSize(self):
        return self._L.orc_box_size(self._m)

    def getLastShakeIters(self):
        return self._L.orc_last_shake_iters(self._m)

    def getFireFirstShakeIters(self):
        """Iterations of the first SHAKE call of the last FIRE step (at the
        step's shakeIter the step retried; test use only)."""
        return self._L.orc_fire_first_shake_iters(self._m)

    def getEnergy(self):
        return self._L.orc_energy(self._m)

    def getMaxEdgeLength(self):
        return self._L.orc_max_edge_length(self._m)

    def getMaxUnbalancedForce(self):
        return self._L.orc_get_max_unbalanced_force(self._m)

    def _V(self):
        return self.getNumVertices()

    def _P(self):
        return self.getNumPolygons()

    def getPositions(self):
        return _copy(self._L.orc_positions(self._m), 2 * self._V(), np.float64)

    def getForces(self):
        return _copy(self._L.orc_forces(self._m), 2 * self._V(), np.float64)

    def getVelocities(self):
        return _copy(self._L.orc_velocities(self._m), 2 * self._V(), np.float64)

    def getAreas(self):
        return _copy(self._L.orc_areas(self._m), self._P(), np.float64)

    def getCOM(self):
        P = self._P()
        return np.concatenate([_copy(self._L.orc_com_x(self._m), P, np.float64),
                               _copy(self._L.orc_com_y(self._m), P, np.float64)])

    def getEdgeLengths(self):
        return _copy(self._L.orc_edge_lengths(self._m), self._V(), np.float64)

    def getPerimeters(self):
        return _copy(self._L.orc_perimeters(self._m), self._P(), np.float64)

    def getConstraints(self):
        return _copy(self._L.orc_constraints(self._m), 6 * self._V(), np.float64)

    def getShapeId(self):
        return _copy(self._L.orc_shape_id(self._m), self._V(), np.int64)

    def getNeighborCells(self):
        return _copy(self._L.orc_cell_location(self._m), self._V(), np.int64)

    def getNeighborIndices(self):
        return _copy(self._L.orc_neighbor_indices(self._m), self._V(), np.int64)

    def getBoxCounts(self):
        B = self.getBoxSize()
        return _copy(self._L.orc_box_starts(self._m), B * B, np.int64)

    def getNumNeighbors(self):
        return _copy(self._L.orc_num_neighbors(self._m), self._V(), np.int64)

    def getNeighborSlots(self):
        M = self.getMaxNeighbors()
        V = self._V()
        nb = _copy(self._L.orc_neighbors(self._m), V * M, np.int64).reshape(V, M)
        ins = _copy(self._L.orc_inside(self._m), V * M, np.uint8).reshape(V, M)
        return nb, ins

    def getNeighbors(self):
        """dict {vertex: neighbour vertices} like model.getNeighbors
        (pyCudaPolygon.py:265-277)."""
        nb, _ = self.getNeighborSlots()
        cnt = self.getNumNeighbors()
        out = {}
        for i in range(nb.shape[0]):
            c = min(int(cnt[i]), nb.shape[1])
            if c:
                out[i] = nb[i, :c].copy()
        return out

    def getInsideFlags(self):
        nb, ins = self.getNeighborSlots()
        cnt = self.getNumNeighbors()
        out = {}
        for i in range(nb.shape[0]):
            c = min(int(cnt[i]), nb.shape[1])
            if c:
                out[i] = ins[i, :c].astype(bool)
        return out

    def getShapeCounts(self):
        return _copy(self._L.orc_shape_counts(self._m), self._P(), np.int64)

    def getIntersections(self):
        return _copy(self._L.orc_intersections(self._m), self.getNumIntersections(), np.uint64)

    def getOutersections(self):
        return _copy(self._L.orc_outersections(self._m), self.getNumIntersections(), np.uint64)

    def getTU(self):
        return _copy(self._L.orc_tu(self._m), 2 * self.getNumIntersections(), np.float64)

    def getUT(self):
        return _copy(self._L.orc_ut(self._m), 2 * self.getNumIntersections(), np.float64)

    def getTargetAreas(self):
        return _copy(self._L.orc_target_areas(self._m), self._P(), np.float64)

    def getTargetEdgeLengths(self):
        return _copy(self._L.orc_target_edge_lengths(self._m), self._P(), np.float64)

    def getStartIndices(self):
        return _copy(self._L.orc_start_indices(self._m), self._P() + 1, np.int64)
