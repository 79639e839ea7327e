"""Host-only checks of the compiled library: it builds, loads without a GPU,
exports every symbol include/pcp_gb300.h declares, and the Python module
carries the reference's method table and enums."""
import ctypes
import json
import os

import pytest

import pycudapolygon_gb300 as pg
from pycudapolygon_gb300 import cabi


@pytest.fixture(scope="module")
def built():
    return pg.build()


def test_library_exports_header_symbols(built):
    lib = ctypes.CDLL(built[0])
    names = cabi.declared_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []


def test_version_and_error_strings(built):
    lib = cabi.lib(built[0])
    assert b"sm_103a" in lib.pcp_version()
    assert lib.pcp_last_error() is not None


def test_null_handle_is_an_error_not_a_crash(built):
    lib = cabi.lib(built[0])
    assert lib.pcp_model_update_neighbors(None) == 1   # PCP_ERR_ARG
    assert b"null model" in lib.pcp_last_error()


def test_module_has_reference_method_table(built, golden_dir):
    mod = pg.load_module()
    ref = json.load(open(os.path.join(golden_dir, "pybind_methods.json")))
    missing = [n for n in ref["methods"] if not hasattr(mod.Model, n)]
    assert missing == []
    for enum_name, values in ref["enums"].items():
        e = getattr(mod, enum_name)
        assert sorted(v for v in e.__members__) == sorted(values)


def test_unbound_reference_methods_stay_unbound(built):
    # the reference binds neither of these (pybindWrapper.cpp); its Python
    # wrappers raise AttributeError, and so must a drop-in
    mod = pg.load_module()
    for n in ["initializeRandomSeed", "getRandomSeed", "getAreaPerOverlap"]:
        assert not hasattr(mod.Model, n)
