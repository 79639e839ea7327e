"""ctypes view of the C ABI in include/pcp_gb300.h (libpcp_gb300.so).

`CModel` drives one pcp_model handle with host arrays, the way a cgo/JNI/
ctypes caller of the library would.  Every failing status raises
`PcpError` with the library's message.
"""
import ctypes
import os
import re

import numpy as np

from . import BUILD_DIR

_lib = None
HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "include", "pcp_gb300.h")


class PcpError(RuntimeError):
    pass


def declared_functions(header=HEADER):
    """Names of the functions include/pcp_gb300.h declares."""
    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pcp_[a-z0-9_]+)\s*\(", src)))


def lib(path=None):
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(path or os.path.join(BUILD_DIR, "libpcp_gb300.so"))
        _lib.pcp_last_error.restype = ctypes.c_char_p
        _lib.pcp_version.restype = ctypes.c_char_p
    return _lib


def _ck(rc):
    if rc != 0:
        raise PcpError("pcp status %d: %s" % (rc, lib().pcp_last_error().decode()))


_D = ctypes.c_double
_I = ctypes.c_int
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _dptr(a):
    # a void* of the data (cheaper than data_as; the functions are unprototyped)
    return ctypes.c_void_p(a.ctypes.data)


def _iptr(a):
    return a.ctypes.data_as(_ip)


class CModel:
    """One model handle driven through the C ABI with host buffers."""

    def __init__(self, size):
        self.L = lib()
        self.h = ctypes.c_void_p()
        self._out4 = (ctypes.c_double * 4)()
        _ck(self.L.pcp_model_create(_I(int(size)), ctypes.byref(self.h)))

    def close(self):
        if self.h:
            self.L.pcp_model_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def call(self, name, *args):
        _ck(getattr(self.L, "pcp_model_" + name)(self.h, *args))

    # setters
    def set_num_vertices(self, n):
        self.call("set_num_vertices", _I(n))

    def set_positions(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.call("set_positions", _dptr(a), _I(a.size))

    def set_forces(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.call("set_forces", _dptr(a), _I(a.size))

    def set_start_indices(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        self.call("set_start_indices", _iptr(a), _I(a.size))

    def set_target_areas(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.call("set_target_areas", _dptr(a), _I(a.size))

    def set_target_edge_lengths(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.call("set_target_edge_lengths", _dptr(a), _I(a.size))

    def set_max_edge_length(self, v):
        self.call("set_max_edge_length", _D(v))

    def set_model_enum(self, e):
        self.call("set_model_enum", _I(e))

    # updaters
    def initialize_neighbor_cells(self):
        self.call("initialize_neighbor_cells")

    def update_polygon_geometry(self):
        self.call("update_polygon_geometry")

    def update_neighbor_cells(self):
        self.call("update_neighbor_cells")

    def update_neighbors(self):
        self.call("update_neighbors")

    def update_outersections(self):
        self.call("update_outersections")

    def update_force_energy(self):
        self.call("update_force_energy")

    def project_force(self):
        self.call("project_force")

    def shake_project(self, n_iter, tol=1e-15):
        it = _I(0)
        self.call("shake_project", _I(n_iter), _D(tol), ctypes.byref(it))
        return it.value

    def fire_step(self, dt, alpha, n_pos, dt_max=0.1, alpha_start=0.1, f_alpha=0.99,
                  f_inc=1.1, f_dec=0.5, n_min=5, shake_iter=5):
        out = self._out4
        self.call("fire_step", _D(dt), _D(alpha), _I(n_pos), _D(dt_max), _D(alpha_start),
                  _D(f_alpha), _D(f_inc), _D(f_dec), _I(n_min), _I(shake_iter), out)
        return float(out[0]), float(out[1]), float(out[2]), int(out[3])

    def minimize_fire(self, thr, dt0, max_steps, dt_max=0.1, alpha_start=0.1, f_alpha=0.99,
                      f_inc=1.1, f_dec=0.5, n_min=5, shake_iter=5):
        out = np.zeros(3)
        self.call("minimize_fire", _D(thr), _D(dt0), _I(max_steps), _D(dt_max),
                  _D(alpha_start), _D(f_alpha), _D(f_inc), _D(f_dec), _I(n_min),
                  _I(shake_iter), _dptr(out))
        return float(out[0]), float(out[1]), int(out[2])

    # getters
    def _scalar(self, name, ctype):
        v = ctype()
        self.call(name, ctypes.byref(v))
        return v.value

    def energy(self):
        return self._scalar("get_energy", _D)

    def max_unbalanced_force(self):
        return self._scalar("get_max_unbalanced_force", _D)

    def num_intersections(self):
        return self._scalar("get_num_intersections", _I)

    def pair_count(self):
        return self._scalar("get_pair_count", ctypes.c_longlong)

    def narrow_pair_total(self):
        return self._scalar("get_narrow_pair_total", ctypes.c_longlong)

    def launch_count(self):
        return self._scalar("get_launch_count", ctypes.c_longlong)

    def _array(self, name, dtype, ctype):
        n = _I(0)
        self.call("get_" + name, None, _I(0), ctypes.byref(n))
        out = np.zeros(n.value, dtype=dtype)
        if n.value:
            self.call("get_" + name, out.ctypes.data_as(ctypes.POINTER(ctype)), _I(n.value),
                      ctypes.byref(n))
        return out

    def positions(self):
        return self._array("positions", np.float64, ctypes.c_double)

    def get_positions_into(self, out):
        n = _I(0)
        self.call("get_positions", _dptr(out), _I(out.size), ctypes.byref(n))
        return out

    def forces(self):
        return self._array("forces", np.float64, ctypes.c_double)

    def intersections(self):
        return self._array("intersections", np.uint64, ctypes.c_uint64)

    def outersections(self):
        return self._array("outersections", np.uint64, ctypes.c_uint64)

    def tu(self):
        return self._array("tu", np.float64, ctypes.c_double)

    def ut(self):
        return self._array("ut", np.float64, ctypes.c_double)
