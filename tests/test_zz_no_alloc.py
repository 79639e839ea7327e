"""pcp_shake_project_noalloc (static device workspace, no allocation) against
pcp_shake_project, both called through the C ABI on device buffers.

Collected last on purpose: it must hold in a fresh process (the first call
on the device looks up the static array) and after every other test of the
suite has run in the same process.  Positions agree within the SHAKE
tolerance of the oracle parity tests (1e-12, minimum image); the iteration
counts agree exactly.  The entry point exists for callers that cannot
allocate device memory, so one test checks that a call leaves the device's
free memory unchanged, and others that inputs it cannot hold are refused
before anything runs.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pycudapolygon_gb300 as pg  # noqa: E402
from pycudapolygon_gb300 import cabi  # noqa: E402
from pycudapolygon_gb300.systems import make_system  # noqa: E402

pg.build()
L = cabi.lib()
_vp = ctypes.c_void_p
for _name in ("pcp_shake_project", "pcp_shake_project_noalloc"):
    getattr(L, _name).argtypes = [_vp, _vp, ctypes.c_int, _vp, _vp, ctypes.c_int, ctypes.c_double,
                                  _vp, _vp]
    getattr(L, _name).restype = ctypes.c_int

MAX_VERTICES = 16384      # PCP_SHAKE_NOALLOC_MAX_VERTICES
POS_TOL = 1e-12


def _dev(system):
    d = torch.device("cuda:0")
    return dict(
        pos=torch.tensor(system.positions, dtype=torch.float64, device=d),
        start=torch.tensor(system.start_indices, dtype=torch.int32, device=d),
        tl=torch.tensor(system.target_edge_lengths, dtype=torch.float64, device=d),
        ta=torch.tensor(system.target_areas, dtype=torch.float64, device=d),
        iters=torch.full((1,), -7, dtype=torch.int32, device=d),
    )


def _call(name, b, num_polygons, max_iter=100, tol=1e-15):
    rc = getattr(L, name)(b["pos"].data_ptr(), b["start"].data_ptr(), num_polygons,
                          b["tl"].data_ptr(), b["ta"].data_ptr(), max_iter, tol,
                          b["iters"].data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 0, L.pcp_last_error().decode()
    return b["pos"].cpu().numpy(), int(b["iters"].item())


def _compare(system):
    P = len(system.start_indices) - 1
    ref_pos, ref_it = _call("pcp_shake_project", _dev(system), P)
    got_pos, got_it = _call("pcp_shake_project_noalloc", _dev(system), P)
    assert got_it == ref_it
    assert 0 < got_it < 100
    d = (got_pos - ref_pos + 0.5) % 1.0 - 0.5
    assert np.abs(d).max() <= POS_TOL


def test_noalloc_shake_matches_shake_on_two_calls_in_a_row():
    # the larger system first, so the second call runs over a workspace that
    # still holds the first call's values
    big = make_system(num_polygons=256, n=np.random.default_rng(21).integers(12, 97, 256),
                      phi=0.86, seed=13)
    small = make_system(num_polygons=96, n=20, phi=0.85, seed=4)
    assert int(big.start_indices[-1]) <= MAX_VERTICES
    _compare(big)
    _compare(small)


def test_noalloc_shake_rejects_more_vertices_than_its_workspace():
    d = torch.device("cuda:0")
    n = MAX_VERTICES + 1
    start = torch.tensor([0, n], dtype=torch.int32, device=d)
    pos = torch.zeros(2 * n, dtype=torch.float64, device=d)
    tl = torch.ones(1, dtype=torch.float64, device=d)
    iters = torch.full((1,), -7, dtype=torch.int32, device=d)
    rc = L.pcp_shake_project_noalloc(pos.data_ptr(), start.data_ptr(), 1, tl.data_ptr(),
                                     tl.data_ptr(), 10, 1e-15, iters.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 3                      # PCP_ERR_CAPACITY
    assert str(MAX_VERTICES) in L.pcp_last_error().decode()
    assert int(iters.item()) == -7      # nothing launched


def test_noalloc_shake_allocates_no_device_memory():
    """After a first call (which looks up the array and loads the kernels),
    a call on a larger system leaves the device's free memory unchanged."""
    warm = make_system(num_polygons=32, n=16, phi=0.85, seed=2)
    big = make_system(num_polygons=200, n=np.random.default_rng(3).integers(24, 97, 200),
                      phi=0.86, seed=17)
    assert int(warm.start_indices[-1]) < int(big.start_indices[-1]) <= MAX_VERTICES
    bw, bb = _dev(warm), _dev(big)
    P_w, P_b = warm.num_polygons, big.num_polygons
    _call("pcp_shake_project_noalloc", bw, P_w)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rc = L.pcp_shake_project_noalloc(bb["pos"].data_ptr(), bb["start"].data_ptr(), P_b,
                                     bb["tl"].data_ptr(), bb["ta"].data_ptr(), 100, 1e-15,
                                     bb["iters"].data_ptr(), None)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert rc == 0, L.pcp_last_error().decode()
    assert 0 < int(bb["iters"].item()) < 100
    assert free_after == free_before


def test_noalloc_shake_rejects_offsets_that_are_not_csr():
    """A decreasing start array would place a polygon's workspace outside the
    array; the call refuses it before the SHAKE kernel runs."""
    d = torch.device("cuda:0")
    start = torch.tensor([0, 10, 5, 20], dtype=torch.int32, device=d)
    pos = torch.zeros(40, dtype=torch.float64, device=d)
    tl = torch.ones(3, dtype=torch.float64, device=d)
    iters = torch.full((1,), -7, dtype=torch.int32, device=d)
    rc = L.pcp_shake_project_noalloc(pos.data_ptr(), start.data_ptr(), 3, tl.data_ptr(),
                                     tl.data_ptr(), 10, 1e-15, iters.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == 1                      # PCP_ERR_ARG
    assert "never decrease" in L.pcp_last_error().decode()
    assert int(iters.item()) == -7      # nothing launched
