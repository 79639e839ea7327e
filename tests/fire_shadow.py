"""Step-by-step FIRE comparison of the CUDA path with the oracle (TEST
INFRASTRUCTURE).

A FIRE run amplifies last-bit differences: the CUDA path adds forces and
energies with FP64 atomics in an order that changes from run to run (as the
reference's kernels do), the oracle adds them in its own order, and after
some tens of steps two free-running trajectories part.  So each step of a
CUDA run is checked against one oracle step started from the CUDA path's own
state: positions, velocities, forces, energy, the step arguments (dt, alpha,
nPos, ...) and the cell size (the Python driver's initForceEnergy sets the
reference's default maxEdgeLength 0.5, pyCudaPolygon.py:54-57; the oracle
takes the same box size).

Every step: dt, alpha and nPos exact (the branch the step took,
model.cpp:405-486).  A plain step (SHAKE converged within shakeIter
iterations, or no SHAKE) and a step whose SHAKE failed on both sides
(positions put back exactly, model.cpp:431-435): energy 1e-12 relative
plus 2 (d + 1e-16) sum |F| for a position difference d (the first-order
change d can make; the energy, a sum of signed chain terms, can be far
smaller than its terms), positions 1e-12 (minimum image), forces 1e-10 of their largest component,
velocities 1e-10 of their largest component or 1e-14/dt, whichever is
larger: a step rederives v from its displacement (x_SHAKE - x_Verlet)/dt,
model.cpp:437, so a position difference d becomes d/dt of velocity, and the
SHAKE kernels take their last, small updates in an FP32 form whose error
is below 6e-15 (1e-14/dt of velocity: 1e-11 at dt = 1e-3).  The SHAKE iteration counts of plain steps
must be equal in at least 80% of them (the tests may ask for more): SHAKE's stop test (max |s_k|/L, |A - A0| <
1e-15) sits at the FP64 rounding floor of its residuals, so a count can
follow the rounding.

A step whose first SHAKE call reached its limit and retried with ten times
the iterations (model.cpp:423-430) mostly meets the same bounds; where it
does not, it is compared within 1e-6 (energy relative, positions absolute)
and counted: the retry starts from the first call's unconverged
iterate, which the two implementations reach only up to the rounding of
their FP32 Newton corrections (relative 6e-8 of the last correction), and the
retry's converged point moves along the constraint manifold with its start
point.  Measured on 64-polygon systems: 2.4e-12 on a polygon whose first
call stopped one iteration short, 2.8e-9 on one whose first call wandered;
every polygon without the retry agreed to 1e-15.  A step where the SHAKE
outcome itself differs (one side converges at the rounding floor, the other
runs into its limit) takes another branch.  Both kinds are counted; the
tests bound how many there may be.
"""
import numpy as np
import pytest

E_RTOL = 1e-12
RETRY_TOL = 1e-6
V_RTOL = 1e-10
F_RTOL = 1e-10
X_ATOL = 1e-12
X_SHAKE_FLOOR = 1e-14
FIRE_DEFAULTS = (0.1, 0.1, 0.99, 1.1, 0.5, 5, 5)   # dtMax .. shakeIter (model.hpp:106-107)


def wrapdiff(a, b):
    return (np.asarray(a) - np.asarray(b) + 0.5) % 1.0 - 0.5


def rel_max(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


class FireShadow:
    """`step(*args)` runs one FIRE step on the CUDA model `g` (through
    `gstep`, default g.minimizeFIREStep) and one oracle step from g's state,
    compares them and returns g's result."""

    def __init__(self, g, o, gstep=None, shake=True):
        self.g, self.o = g, o
        self.gstep = gstep if gstep is not None else g.minimizeFIREStep
        self.shake = shake
        self.n = 0
        self.plain = 0
        self.same_iters = 0
        self.floor_steps = []
        self.retry_steps = []
        self.kinds = set()

    def step(self, *a):
        g, o = self.g, self.o
        full = tuple(a) + FIRE_DEFAULTS[len(a) - 3:]
        if o.getBoxSize() != g.getBoxSize():
            o.setMaxEdgeLength(1.0 / (g.getBoxSize() + 0.5))
        o.setPositions(g.getPositions())
        o.setVelocities(g.getVelocities())
        o.setForces(g.getForces())
        o.setEnergy(g.getEnergy())
        ro = o.minimizeFIREStep(*full)
        rg = self.gstep(*a)
        k = self.n
        self.n += 1
        lim = full[9]
        retried = failed_o = failed_g = False
        if self.shake:
            it_g, it_o = g.getLastShakeIters(), o.getLastShakeIters()
            retried = o.getFireFirstShakeIters() >= lim
            failed_o, failed_g = retried and it_o >= 10 * lim, it_g >= 10 * lim
        if failed_o != failed_g:
            self.floor_steps.append((k, it_g, it_o))
            return rg
        assert (rg[1], rg[2], rg[3]) == (ro[1], ro[2], ro[3]), ("dt/alpha/nPos", k, rg, ro)
        xd = np.abs(wrapdiff(g.getPositions(), o.getPositions())).max()
        info = (k, rg, ro, xd, it_g, it_o, o.getFireFirstShakeIters()) if self.shake else (k, rg, ro, xd)
        if retried and not failed_o and (xd > X_ATOL or rg[0] != pytest.approx(ro[0], rel=E_RTOL)):
            assert rg[0] == pytest.approx(ro[0], rel=RETRY_TOL), ("E retry",) + info
            assert xd <= RETRY_TOL, ("x retry",) + info
            self.retry_steps.append((k, xd))
            return rg
        # 1e-12 relative, plus the first-order change the measured position
        # difference xd can make: sum |F| * xd (the energy is a sum of signed
        # chain terms and can be far smaller than the terms themselves)
        fo = np.asarray(o.getForces())
        e_tol = E_RTOL * abs(ro[0]) + 2.0 * (xd + 1e-16) * np.abs(fo).sum()
        assert abs(rg[0] - ro[0]) <= e_tol, ("E", e_tol) + info
        assert xd <= X_ATOL, ("x",) + info
        self.plain += 1
        if self.shake:
            self.same_iters += it_g == it_o
        vg, vo = np.asarray(g.getVelocities()), np.asarray(o.getVelocities())
        vtol = max(V_RTOL * np.abs(vo).max(), X_SHAKE_FLOOR / a[0])
        assert np.abs(vg - vo).max() <= vtol, ("v", k, np.abs(vg - vo).max(), vtol)
        assert rel_max(g.getForces(), o.getForces()) <= F_RTOL, ("F", k)
        assert g.getMaxUnbalancedForce() == pytest.approx(o.getMaxUnbalancedForce(), rel=F_RTOL)
        self.kinds.add("reset" if rg[3] == 0 and rg[2] == full[4] else "advance")
        return rg

    def check_counts(self, floor_frac=0.05, retry_frac=0.1, same_frac=0.8):
        assert len(self.floor_steps) <= floor_frac * self.n, self.floor_steps
        assert len(self.retry_steps) <= retry_frac * self.n, self.retry_steps
        if self.shake:
            assert self.same_iters >= same_frac * self.plain, (self.same_iters, self.plain)
