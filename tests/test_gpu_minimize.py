"""FIRE minimisation to the reference driver's stop, CUDA path against the oracle.

The reference's Python driver (pyCudaPolygon.py:674-731) stops when
|F|max <= maxForceThreshold, or once six steps (not necessarily in a row)
returned an energy within 1e-15 of the step before.  With the reference's
overlap energy and force (kernels.cuh:1067-1424) plain FIRE does not reach
|F|max <= 1e-10 on the 64-polygon, 16-vertex, phi 0.85 systems: the force is
not the gradient of the energy (it holds each chain's start point fixed), the
energy jumps when crossings appear or vanish, and the energy-increase rollback
(model.cpp:450-470) then shrinks dt step after step.  Runs stop by the
stagnation rule after a few dozen to a few hundred steps.

A FIRE run amplifies last-bit differences: the CUDA path adds forces and
energies with FP64 atomics in an order that changes from run to run (as the
reference's kernels do, model.cpp:450-451), the oracle adds them in its own
order, and after some tens of steps the two trajectories part.  So every step
of a CUDA run is checked against one oracle step started from the CUDA
path's own state (positions, velocities, forces, energy, dt, alpha, nPos):
step energies 1e-9 relative; dt, alpha and nPos exact; positions 1e-12
(minimum image); forces 1e-10 of their largest
component; velocities 1e-10 of their largest component or 8 ulp(1)/dt,
whichever is larger: a step rederives v from its displacement
(x_SHAKE - x_Verlet)/dt (model.cpp:436), so one ulp of a position near 0.5
(1.1e-16) is already 1.1e-13 of velocity at dt = 1e-3.  SHAKE's stop test
(max |s_k|/L, |A - A0| < 1e-15) sits at the FP64 rounding floor of its
residuals: once a step's violation is that small the iteration count follows
the rounding (one side may stop at 0 iterations where the other takes 4), so
the test requires the same outcome of SHAKE in every step (converged within
shakeIter, retried, or failed: the branch the step takes) and the same count
in at least 90% of the steps; a step where the outcome itself differs (one
side stops at the floor, the other runs into its limit) takes another
branch and is counted, at most 5% of the steps.  The energy tolerance is
1e-9 rather than 1e-12 for the same reason: both SHAKEs solve their Newton
corrections in FP32 (parallel cyclic reduction), so after a large correction
the two land on points of the constraint manifold up to ~1e-13 apart, and
the reference's float rounding of the crossing parameters
(kernels.cuh:857-858) turns such a difference into an energy step of up to
~1e-9 relative when a parameter sits at a float rounding boundary.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from oracle import oracle as orc  # noqa: E402
from pycudapolygon_gb300 import load_module  # noqa: E402
from pycudapolygon_gb300.systems import load_into, make_system  # noqa: E402
from refdriver import model  # noqa: E402

THR = 1e-10
E_RTOL = 1e-9
V_RTOL = 1e-10
F_RTOL = 1e-10
X_ATOL = 1e-12


def _wrapdiff(a, b):
    return (np.asarray(a) - np.asarray(b) + 0.5) % 1.0 - 0.5


def _rel_max(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


class _Shadow:
    """Wraps the CUDA model's minimizeFIREStep: before each step the oracle
    takes the CUDA path's state and runs the same step; after it the two
    results are compared."""

    def __init__(self, g, o):
        self.g, self.o = g, o
        self.step = g.minimizeFIREStep
        self.n = 0
        self.same_iters = 0
        self.floor_steps = []
        self.kinds = set()
        g.minimizeFIREStep = self

    def __call__(self, *a):
        g, o = self.g, self.o
        o.setPositions(g.getPositions())
        o.setVelocities(g.getVelocities())
        o.setForces(g.getForces())
        o.setEnergy(g.getEnergy())
        ro = o.minimizeFIREStep(*a)
        rg = self.step(*a)
        k = self.n
        self.n += 1
        it_g, it_o = g.getLastShakeIters(), o.getLastShakeIters()
        lim = a[9]
        outcome = lambda it: 0 if it < lim else (1 if it < 10 * lim else 2)   # noqa: E731
        if outcome(it_g) != outcome(it_o):
            # SHAKE converged on one side and not on the other at its
            # rounding floor: the step takes another branch; counted, bounded
            self.floor_steps.append((k, it_g, it_o))
            return rg
        assert rg[0] == pytest.approx(ro[0], rel=E_RTOL, abs=1e-300), ("E", k, rg, ro, it_g, it_o)
        assert (rg[1], rg[2], rg[3]) == (ro[1], ro[2], ro[3]), ("dt/alpha/nPos", k, rg, ro)
        self.same_iters += it_g == it_o
        assert np.abs(_wrapdiff(g.getPositions(), o.getPositions())).max() <= X_ATOL, ("x", k)
        vg, vo = np.asarray(g.getVelocities()), np.asarray(o.getVelocities())
        vtol = max(V_RTOL * np.abs(vo).max(), 8 * 2.0 ** -52 / a[0])
        assert np.abs(vg - vo).max() <= vtol, ("v", k, np.abs(vg - vo).max(), vtol)
        assert _rel_max(g.getForces(), o.getForces()) <= F_RTOL, ("F", k)
        self.kinds.add("reset" if rg[3] == 0 and rg[2] == a[4] else "advance")
        return rg


def _pair(seed, phi=0.85):
    s = make_system(64, 16, phi, seed=seed)
    g = load_into(model(s.num_vertices), s)
    o = load_into(orc.OracleModel(s.num_vertices), s)
    for m in (g, o):
        m.shakeProject(100, 1e-15)
    return s, g, o


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_every_step_of_a_run_to_the_driver_stop_matches_oracle(seed):
    s, g, o = _pair(seed)
    sh = _Shadow(g, o)
    r = g.minimizeFIRE(THR, 1e-3, 5000)
    assert 0 < r[2] < 5000 and sh.n == r[2]
    assert len(sh.floor_steps) <= 0.05 * sh.n, sh.floor_steps
    compared = sh.n - len(sh.floor_steps)
    assert sh.same_iters >= 0.9 * compared, (sh.same_iters, compared)
    assert "reset" in sh.kinds and "advance" in sh.kinds
    assert g.getMaxUnbalancedForce() > THR         # stopped by the stagnation rule


def test_device_driver_runs_the_python_driver_rule():
    """minimizeFIREDevice: the same calls before the loop, the loop on the
    device.  Its first 20 steps follow the Python driver's (run on the same
    state to the same step limit, before the trajectories can part), and a
    full run stops by the same stagnation rule."""
    s, g1, _ = _pair(1)
    g2 = load_into(model(s.num_vertices), s)
    g2.shakeProject(100, 1e-15)
    r1 = g1.minimizeFIRE(THR, 1e-3, 20)
    r2 = g2.minimizeFIREDevice(THR, 1e-3, 20)
    assert r1[2] == r2[2] == 20
    assert r2[0] == pytest.approx(r1[0], rel=1e-12)
    assert r2[1] == r1[1]
    np.testing.assert_array_equal(r2[3], r1[3])
    assert np.abs(_wrapdiff(g2.getPositions(), g1.getPositions())).max() < 1e-12
    g3 = load_into(model(s.num_vertices), s)
    g3.shakeProject(100, 1e-15)
    r3 = g3.minimizeFIREDevice(THR, 1e-3, 5000)
    stagnated, lo, total, hi = g3.fireRunStats()
    assert stagnated == 1 and 0 < r3[2] < 5000
    assert (lo, total / 5000, hi) == tuple(r3[3])


def test_cpp_minimize_fire_stalls_on_both_sides():
    """Model::minimizeFIRE (model.cpp:488-504) stops only on |F|max or the
    step limit: neither the CUDA path nor the oracle gets below 1e-10 in 400
    steps, and both shrink dt by orders of magnitude (the stall the module
    docstring describes)."""
    s, g, o = _pair(3)
    Model = load_module().Model          # the C++ method under the Python driver's name
    rg = Model.minimizeFIRE(g, THR, 1e-3, 400)
    ro = orc.OracleModel.minimizeFIRE(o, THR, 1e-3, 400)
    assert rg[2] == ro[2] == 400
    assert g.getMaxUnbalancedForce() > 1e-6 and o.getMaxUnbalancedForce() > 1e-6
    assert rg[1] < 1e-5 and ro[1] < 1e-5
