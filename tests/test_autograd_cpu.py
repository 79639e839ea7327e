"""The autograd wiring of pycudapolygon_gb300/autograd.py on the CPU, with a
stand-in system whose energy is a known quadratic (the GPU kernel itself is
tested in test_gpu_autograd.py): the forward returns the system's energies,
the backward its gradient times the incoming gradient, for one configuration
and for a batch."""
import pytest

torch = pytest.importorskip("torch")

from pycudapolygon_gb300.autograd import OverlapEnergy  # noqa: E402


class _Quadratic:
    """E(x) = sum(c * x^2) per configuration, dE/dx = 2 c x."""

    def __init__(self, c):
        self.c = c

    def evaluate(self, x, mode=1):
        assert mode == 1
        return (self.c * x * x).sum(dim=1), 2 * self.c * x


def test_single_configuration():
    c = torch.tensor([1.0, 2.0, 3.0, 4.0], dtype=torch.float64)
    x = torch.tensor([0.1, -0.2, 0.3, 0.5], dtype=torch.float64, requires_grad=True)
    e = OverlapEnergy.apply(x, _Quadratic(c))
    assert e.dim() == 0
    assert float(e) == pytest.approx(float((c * x * x).sum()))
    (g,) = torch.autograd.grad(3.0 * e, x)
    torch.testing.assert_close(g, 3.0 * 2 * c * x.detach())


def test_batch_with_weights():
    c = torch.tensor([1.0, 0.5, 2.0, 1.5], dtype=torch.float64)
    x = torch.randn(5, 4, dtype=torch.float64, requires_grad=True)
    e = OverlapEnergy.apply(x, _Quadratic(c))
    assert e.shape == (5,)
    w = torch.arange(1, 6, dtype=torch.float64)
    (g,) = torch.autograd.grad((w * e).sum(), x)
    torch.testing.assert_close(g, w[:, None] * 2 * c * x.detach())
    assert torch.autograd.gradcheck(lambda y: OverlapEnergy.apply(y, _Quadratic(c)), (x,))
