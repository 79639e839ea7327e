"""The reciprocal the projection uses in place of a division
(pcp_rcp_newton: two Newton-Raphson steps from the FP32 reciprocal) against
1/x, over the magnitudes it serves and both signs: within 4 ulp."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pycudapolygon_gb300 as pg  # noqa: E402
from pycudapolygon_gb300 import cabi  # noqa: E402

pg.build()
L = cabi.lib()
L.pcp_rcp_newton.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
L.pcp_rcp_newton.restype = ctypes.c_int


def test_rcp_newton_within_4_ulp():
    rng = np.random.default_rng(0)
    e = np.floor(rng.uniform(-125.0, 125.9, 400000)).astype(int)
    x = np.ldexp(rng.uniform(1.0, 2.0, e.size), e) * rng.choice([-1.0, 1.0], e.size)
    x = np.concatenate([x, [1.0, -1.0, 2.0, 3.0, 0.1, 1e-28, 1.0000000000000002, 2.0 ** 125]])
    dx = torch.tensor(x, dtype=torch.float64, device="cuda")
    dy = torch.empty_like(dx)
    assert L.pcp_rcp_newton(dx.data_ptr(), dy.data_ptr(), dx.numel(), None) == 0
    torch.cuda.synchronize()
    y = dy.cpu().numpy()
    ref = 1.0 / x
    err = np.abs(y - ref) / np.spacing(np.abs(ref))
    assert err.max() <= 4.0, err.max()
