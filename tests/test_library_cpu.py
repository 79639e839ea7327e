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


def test_warm_start_kernels_check_arguments_first(built):
    """The warm start's entry points refuse bad arguments before touching
    the device (no GPU needed): K not a multiple of 8, misaligned operands
    or outputs, ReLU with a split K, an odd row width."""
    lib = cabi.lib(built[0])
    fake = ctypes.c_void_p(1 << 20)          # never dereferenced: the checks come first
    odd = ctypes.c_void_p((1 << 20) + 8)
    assert lib.pcp_gemm_bf16(fake, fake, fake, 128, 128, 7, None, 0, 1, None) == 1
    assert b"multiple of 8" in lib.pcp_last_error()
    assert lib.pcp_gemm_bf16(odd, fake, fake, 128, 128, 64, None, 0, 1, None) == 1
    assert b"aligned" in lib.pcp_last_error()
    # C takes 16-byte row stores
    assert lib.pcp_gemm_bf16(fake, fake, odd, 128, 128, 64, None, 0, 1, None) == 1
    assert b"aligned" in lib.pcp_last_error()
    assert lib.pcp_gemm_bf16(fake, fake, fake, 128, 128, 64, None, 1, 4, None) == 1
    assert b"ReLU" in lib.pcp_last_error()
    assert lib.pcp_gemm_bf16(fake, fake, fake, 128, 128, 64, None, 0, 0, None) == 1
    assert lib.pcp_gemm_bf16(None, fake, fake, 128, 128, 64, None, 0, 1, None) == 1
    assert lib.pcp_gemm_bf16(fake, fake, fake, 0, 128, 64, None, 0, 1, None) == 0   # empty
    assert lib.pcp_graph_sum_bf16(fake, fake, fake, fake, 10, 7, ctypes.c_float(1.0), None) == 1
    assert b"even" in lib.pcp_last_error()
    half = ctypes.c_void_p((1 << 20) + 2)     # BF16 pairs are read and written as 4-byte words
    assert lib.pcp_graph_sum_bf16(fake, fake, half, fake, 10, 8, ctypes.c_float(1.0), None) == 1
    assert b"4-byte" in lib.pcp_last_error()


def test_stateless_launchers_check_arguments_first(built):
    """The stateless launchers refuse negative sizes, NULL buffers and a
    box size below one before any launch (no GPU needed)."""
    lib = cabi.lib(built[0])
    fake = ctypes.c_void_p(1 << 20)          # never dereferenced: the checks come first
    d = ctypes.c_double
    assert lib.pcp_topology(fake, -1, 10, fake, fake, fake, None) == 1
    assert lib.pcp_topology(fake, 4, 10, None, fake, fake, None) == 1
    assert b"null" in lib.pcp_last_error()
    assert lib.pcp_topology(None, 0, 0, None, None, None, None) == 0   # empty: nothing to do
    assert lib.pcp_polygon_geometry(fake, fake, 4, 40, fake, fake, fake, fake, fake, fake, None,
                                    None) == 1
    assert lib.pcp_neighbor_cells(fake, fake, fake, 40, 0, fake, None) == 1
    assert b"box_size" in lib.pcp_last_error()
    assert lib.pcp_project_force(fake, fake, -2, fake, fake, None) == 1
    assert lib.pcp_project_force(fake, None, 3, fake, fake, None) == 1
    assert lib.pcp_shake_project(fake, fake, 3, fake, fake, 5, d(1e-15), None, None) == 1
    assert lib.pcp_shake_project(None, fake, 3, fake, fake, 5, d(1e-15), fake, None) == 1
    assert lib.pcp_update_positions(fake, None, 10, d(1e-3), None) == 1
    assert lib.pcp_update_positions(fake, fake, -1, d(1e-3), None) == 1


def test_integration_notes_list_every_extra_method(built, golden_dir):
    """Every method the module adds to the reference's table is named in
    INTEGRATION.md's list of deliberate differences."""
    mod = pg.load_module()
    ref = set(json.load(open(os.path.join(golden_dir, "pybind_methods.json")))["methods"])
    extra = sorted(n for n in dir(mod.Model) if not n.startswith("_") and n not in ref)
    doc = open(os.path.join(os.path.dirname(golden_dir), "..", "INTEGRATION.md")).read()
    assert [n for n in extra if n not in doc] == []
