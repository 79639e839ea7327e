"""GB300-native (sm_103a) polygon overlap path of pyCudaPolygon.

Layers:
  include/pcp_gb300.h + _build/libpcp_gb300.so   C ABI and CUDA kernels
  _build/libpyCudaPolygon*.so                    pybind11 module with the reference's
                                                 `Model` method table (drop-in)
  cabi.py                                        ctypes view of the C ABI
  systems.py                                     seeded synthetic polygon systems

The reference's own Python layer (pyCudaPolygon.py, its mixins and enums)
runs unchanged on `libpyCudaPolygon`.

Nothing here falls back to a CPU path: if the compiled library is missing the
import of `libpyCudaPolygon` fails, and every call needs a CUDA device.
"""
import os
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_HERE, "_build")


def build(force=False):
    """Compile the CUDA library and the Python module in-tree."""
    from . import buildlib as _b
    return _b.build(force=force)


def load_module():
    """Import and return the compiled `libpyCudaPolygon` module."""
    if BUILD_DIR not in sys.path:
        sys.path.insert(0, BUILD_DIR)
    import libpyCudaPolygon  # noqa: E402
    return libpyCudaPolygon


def library_path():
    return os.path.join(BUILD_DIR, "libpcp_gb300.so")
