"""Parity of the CUDA path (through the reference-facing Model API, which calls
the C ABI) with the CPU oracle on identical seeded inputs.

Tolerances (stated by the benchmark spec for this path): contact lists bit-exact;
areas relative 1e-12; forces 1e-10 relative to the largest force component;
energies 1e-12 relative.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pycudapolygon_gb300 as pg  # noqa: E402
from pycudapolygon_gb300.systems import PolygonSystem, load_into, make_system  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from fire_shadow import FireShadow  # noqa: E402

pg.build()
lib = pg.load_module()

FORCE_RTOL = 1e-10
AREA_RTOL = 1e-12
ENERGY_RTOL = 1e-12


def pair(system):
    g = load_into(lib.Model(system.num_vertices), system)
    o = load_into(orc.OracleModel(system.num_vertices), system)
    return g, o


def contacts(m):
    m.updatePolygonGeometry()
    m.updateNeighborCells()
    m.updateNeighbors()
    m.updateOutersections()


def assert_records_equal(g, o):
    assert g.getNumIntersections() == o.getNumIntersections()
    np.testing.assert_array_equal(np.asarray(g.getIntersections(), dtype=np.uint64),
                                  o.getIntersections())
    np.testing.assert_array_equal(np.asarray(g.getOutersections(), dtype=np.uint64),
                                  o.getOutersections())
    np.testing.assert_array_equal(np.asarray(g.getTU()), o.getTU())
    np.testing.assert_array_equal(np.asarray(g.getUT()), o.getUT())


def assert_forces_close(gf, of):
    gf = np.asarray(gf)
    scale = max(np.abs(of).max(), 1e-300)
    assert np.abs(gf - of).max() <= FORCE_RTOL * scale, np.abs(gf - of).max() / scale


SYSTEMS = {
    "small_64x16": dict(num_polygons=64, n=16, phi=0.85, seed=1),
    "mid_256x24": dict(num_polygons=256, n=24, phi=0.87, seed=7),
    "tri_quads": dict(num_polygons=40, n=4, phi=0.9, seed=3),
    "varn_200": dict(num_polygons=200, n=np.random.default_rng(5).integers(12, 49, 200), phi=0.86, seed=11),
    # ragged polygons of at most 32 vertices: the one-vertex-per-lane kernels
    # with idle lanes and a different n in every warp
    "varn_small": dict(num_polygons=150, n=np.random.default_rng(8).integers(5, 33, 150), phi=0.86, seed=12),
}


@pytest.fixture(params=list(SYSTEMS))
def system(request):
    return make_system(**SYSTEMS[request.param])


# ------------------------------------------------------------------ known answer
def test_testsaver_known_answer():
    fx = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "testsaver.json")))
    pos = np.asarray(fx["positions"])
    n_array = np.asarray(fx["n_array"])
    for shift in (False, True):
        p = pos.reshape(-1, 2)
        p = ((p - p.mean(axis=0)) % 1.0).reshape(-1) if shift else pos
        m = lib.Model(10)
        m.setNumVertices(10)
        m.setStartIndices(np.concatenate([[0], np.cumsum(n_array)]).astype(np.int32))
        m.setPositions(p)
        m.setMaxEdgeLength(0.25)
        m.initializeNeighborCells()
        m.setMaxEdgeLength(0.5)
        m.updateNeighborCells()
        m.updateNeighbors()
        nb = np.asarray(m.getNeighbors()).reshape(10, -1)
        cnt = np.asarray(m.getNumNeighbors())
        got = {i: nb[i, :cnt[i]].tolist() for i in range(10) if cnt[i]}
        assert got == {1: [7, 8]}
        ins = np.asarray(m.getInsideFlag()).reshape(10, -1)
        assert ins[1, :2].tolist() == [True, False]


# ------------------------------------------------------------------ geometry
def test_geometry_parity(system):
    g, o = pair(system)
    g.updatePolygonGeometry()
    o.updatePolygonGeometry()
    np.testing.assert_allclose(g.getAreas(), o.getAreas(), rtol=AREA_RTOL)
    np.testing.assert_allclose(g.getPerimeters(), o.getPerimeters(), rtol=1e-12)
    np.testing.assert_allclose(g.getEdgeLengths(), o.getEdgeLengths(), rtol=1e-12)
    d = (np.asarray(g.getCOM()) - o.getCOM() + 0.5) % 1.0 - 0.5
    assert np.abs(d).max() < 1e-13
    np.testing.assert_allclose(g.getConstraints(), o.getConstraints(), rtol=1e-10, atol=1e-13)
    assert g.getMaxEdgeLength() == pytest.approx(o.getMaxEdgeLength(), rel=1e-13)


# ------------------------------------------------------------------ contacts
@pytest.mark.parametrize("box", ["system", 2, 1, 7])
def test_contact_records_bit_exact(system, box):
    g, o = pair(system)
    if box != "system":
        g.setMaxEdgeLength(1.0 / box)
        o.setMaxEdgeLength(1.0 / box)
    contacts(g)
    contacts(o)
    assert o.getNumIntersections() > 0 or system.num_polygons < 50
    assert_records_equal(g, o)
    np.testing.assert_array_equal(g.getNeighborCells(), o.getNeighborCells())
    np.testing.assert_array_equal(g.getNeighborIndices(), o.getNeighborIndices())
    np.testing.assert_array_equal(g.getBoxCounts(), o.getBoxCounts())


def _odd_system():
    """Polygons the self-crossing search must handle: a bow tie, a pentagram,
    a reflex (non-star from vertex 0) hexagon, a polygon with a repeated
    vertex, a thin sliver, plus regular polygons overlapping them and one
    straddling the periodic boundary."""
    rings = []
    def at(c, pts, s):
        return [((c[0] + s * x) % 1.0, (c[1] + s * y) % 1.0) for x, y in pts]
    rings.append(at((0.20, 0.20), [(0, 0), (1, 1), (1, 0), (0, 1)], 0.05))
    star = [(np.cos(np.pi / 2 + 4 * np.pi * k / 5), np.sin(np.pi / 2 + 4 * np.pi * k / 5))
            for k in range(5)]
    rings.append(at((0.50, 0.50), star, 0.04))
    rings.append(at((0.80, 0.25), [(0, 0), (2, 0), (2, 2), (1, 0.4), (0, 2), (-0.2, 1)], 0.02))
    rings.append(at((0.30, 0.70), [(0, 0), (1, 0), (1, 0), (1, 1), (0, 1)], 0.04))
    rings.append(at((0.70, 0.70), [(0, 0), (1, 0.001), (2, 0), (1, -0.001)], 0.03))
    reg = lambda n: [(np.cos(2 * np.pi * k / n), np.sin(2 * np.pi * k / n)) for k in range(n)]
    for c in [(0.22, 0.23), (0.52, 0.48), (0.81, 0.27), (0.31, 0.71), (0.72, 0.70), (0.995, 0.5)]:
        rings.append(at(c, reg(12), 0.03))
    n_array = np.array([len(r) for r in rings], dtype=np.int32)
    start = np.concatenate([[0], np.cumsum(n_array)]).astype(np.int32)
    pos = np.array([xy for r in rings for xy in r], dtype=np.float64).reshape(-1)
    P = len(rings)
    sysobj = PolygonSystem(positions=pos, n_array=n_array, start_indices=start,
                           target_areas=np.full(P, 1e-3), target_edge_lengths=np.full(P, 0.01),
                           max_edge_length=0.1, phi=0.0)
    return sysobj


@pytest.mark.parametrize("box", ["system", 1, 3])
def test_self_crossing_records_bit_exact(box):
    system = _odd_system()
    g, o = pair(system)
    if box != "system":
        g.setMaxEdgeLength(1.0 / box)
        o.setMaxEdgeLength(1.0 / box)
    contacts(g)
    contacts(o)
    keys = o.getIntersections().astype(np.uint64)
    si = (keys >> np.uint64(32)) & np.uint64(0xFFFF)
    sj = keys >> np.uint64(48)
    assert np.count_nonzero(si == sj) >= 6      # bow tie 2, pentagram 5 (at least)
    assert_records_equal(g, o)


def _scrambled_system():
    """A 64-polygon system after a FIRE step whose Verlet move flung some
    polygons' vertices across the box (as a step with huge forces does before
    SHAKE gives up and puts them back): three polygons with vertices spread
    over the whole box, one stretched over more than half of it along x, one
    along the diagonal, the others as generated."""
    s = make_system(64, 16, 0.85, seed=5)
    x = s.positions.reshape(-1, 2).copy()
    rng = np.random.default_rng(11)
    st = s.start_indices
    for p in (3, 17, 40):
        x[st[p]:st[p + 1]] = rng.random((st[p + 1] - st[p], 2))
    for p, d in ((25, (0.7, 0.0)), (52, (0.45, 0.45))):
        k = np.arange(st[p + 1] - st[p]) / (st[p + 1] - st[p])
        spread = np.abs(2.0 * k - 1.0)[:, None] * np.asarray(d)[None, :]
        x[st[p]:st[p + 1]] = (x[st[p]:st[p + 1]] + spread) % 1.0
    return PolygonSystem(positions=x.reshape(-1), n_array=s.n_array,
                         start_indices=s.start_indices, target_areas=s.target_areas,
                         target_edge_lengths=s.target_edge_lengths,
                         max_edge_length=s.max_edge_length, phi=s.phi)


@pytest.mark.parametrize("box", ["system", 2, 7])
def test_records_bit_exact_with_polygons_spanning_the_box(box):
    """Polygons that span more than half the box: the edge pairs the
    reference tests (kernels.cuh:709-812, each difference wrapped on its
    own) are all tested, whatever frame the narrow phase's culls use."""
    system = _scrambled_system()
    g, o = pair(system)
    if box != "system":
        g.setMaxEdgeLength(1.0 / box)
        o.setMaxEdgeLength(1.0 / box)
    contacts(g)
    contacts(o)
    assert o.getNumIntersections() > 0
    assert_records_equal(g, o)
    g.updateForceEnergy()
    o.updateForceEnergy()
    assert g.getEnergy() == pytest.approx(o.getEnergy(), rel=ENERGY_RTOL)
    assert_forces_close(g.getForces(), o.getForces())


def test_records_bit_exact_when_most_pairs_overflow():
    """Every polygon scrambled (random vertices over the whole box, as after a
    FIRE step with a huge force): 400 polygons of 24 vertices at box size 2
    give about 80,000 candidate pairs with dozens of crossings each, more
    than the warps of the narrow phase can finish themselves, so the
    overflow kernel (k_narrow_over) and the grid-wide fixup take most of the
    work.  Records, outersections, energy and force against the oracle."""
    s = make_system(400, 24, 0.85, seed=21)
    x = np.random.default_rng(5).random(s.positions.size)
    system = PolygonSystem(positions=x, n_array=s.n_array, start_indices=s.start_indices,
                           target_areas=s.target_areas, target_edge_lengths=s.target_edge_lengths,
                           max_edge_length=s.max_edge_length, phi=s.phi)
    g, o = pair(system)
    g.setMaxEdgeLength(0.5)
    o.setMaxEdgeLength(0.5)
    contacts(g)
    contacts(o)
    keys = o.getIntersections().astype(np.uint64)
    a = (keys >> np.uint64(48)).astype(np.int64)
    b = ((keys >> np.uint64(32)) & np.uint64(0xFFFF)).astype(np.int64)
    _, per_pair = np.unique(np.minimum(a, b) * 65536 + np.maximum(a, b), return_counts=True)
    # more pairs over a warp's 32-record slot than the warps finish
    # themselves: 16 per warp, 4 warps per block of the default grid
    blocks = lib.Model(8).getLaunchShape()[0]
    assert np.count_nonzero(per_pair > 32) > 16 * 4 * blocks
    assert_records_equal(g, o)
    g.updateForceEnergy()
    o.updateForceEnergy()
    assert g.getEnergy() == pytest.approx(o.getEnergy(), rel=ENERGY_RTOL)
    assert_forces_close(g.getForces(), o.getForces())


def test_geometry_parity_odd_shapes():
    """Geometry of the odd shapes: a repeated vertex (a zero-length edge,
    whose unit tangent the reference computes as 0/0), a bow tie, a sliver,
    a polygon across the periodic boundary."""
    system = _odd_system()
    g, o = pair(system)
    g.updatePolygonGeometry()
    o.updatePolygonGeometry()
    np.testing.assert_allclose(g.getAreas(), o.getAreas(), rtol=AREA_RTOL, atol=1e-17)
    np.testing.assert_allclose(g.getPerimeters(), o.getPerimeters(), rtol=1e-12)
    np.testing.assert_allclose(g.getEdgeLengths(), o.getEdgeLengths(), rtol=1e-12)
    np.testing.assert_allclose(g.getConstraints(), o.getConstraints(), rtol=1e-10, atol=1e-13,
                               equal_nan=True)
    assert np.isnan(np.asarray(o.getConstraints())).any()


@pytest.mark.parametrize("density", [64, 211])
def test_overlap_area_estimate_parity(system, density):
    """The grid-point overlap estimate (updateOverlapAreaKernel,
    kernels.cuh:879-979; Model::updateOverlapArea, model.cpp:824-847): the
    count of polygon pairs over the grid points, divided by their number.
    The counts are integers, so the estimates agree exactly."""
    g, o = pair(system)
    for m in (g, o):
        m.updatePolygonGeometry()
        m.updateNeighborCells()
        m.updateOverlapArea(density)
    assert g.getOverlapArea() == o.getOverlapArea()
    assert o.getOverlapArea() > 0.0 or system.num_polygons < 50


def test_neighbor_slots_bit_exact(system):
    g, o = pair(system)
    contacts(g)
    contacts(o)
    nb_o, ins_o = o.getNeighborSlots()
    cnt_o = o.getNumNeighbors()
    np.testing.assert_array_equal(g.getNumNeighbors(), cnt_o)
    M = g.getMaxNeighbors()
    assert M == o.getMaxNeighbors()
    nb_g = np.asarray(g.getNeighbors()).reshape(-1, M)
    ins_g = np.asarray(g.getInsideFlag()).reshape(-1, M)
    for v in np.nonzero(cnt_o)[0]:
        c = cnt_o[v]
        assert nb_g[v, :c].tolist() == nb_o[v, :c].tolist()
        assert ins_g[v, :c].astype(bool).tolist() == ins_o[v, :c].astype(bool).tolist()


def test_contacts_unchanged_by_stale_cells(system):
    """updateNeighbors uses the cells of the last updateNeighborCells, as the
    reference does, even when positions moved in between."""
    g, o = pair(system)
    for m in (g, o):
        m.updatePolygonGeometry()
        m.updateNeighborCells()
        m.updateForceEnergy()
        m.updatePositions(1e-3)
        m.updateNeighbors()
        m.updateOutersections()
    assert_records_equal(g, o)


# ------------------------------------------------------------------ force / energy
def test_overlap_force_energy_parity(system):
    g, o = pair(system)
    for m in (g, o):
        contacts(m)
        m.updateForceEnergy()
    e_o = o.getEnergy()
    assert g.getEnergy() == pytest.approx(e_o, rel=ENERGY_RTOL, abs=1e-300)
    assert_forces_close(g.getForces(), o.getForces())
    assert g.getMaxUnbalancedForce() == pytest.approx(o.getMaxUnbalancedForce(), rel=1e-10)


def test_projection_parity(system):
    g, o = pair(system)
    for m in (g, o):
        contacts(m)
        m.updateForceEnergy()
        m.projectForce()
    assert_forces_close(g.getForces(), o.getForces())


def test_soft_body_parity(system):
    # targets moved off the current shape so that the springs carry real force
    ta = system.target_areas * 1.1
    tl = system.target_edge_lengths * 0.95
    for mt, k, c in [(3, 1.0, 1.0), (1, 2.0, 0.0), (2, 0.0, 3.0), (5, 1.0, 1.0)]:
        g, o = pair(system)
        g.setModelEnum(lib.modelEnum(mt))
        o.setModelEnum(mt)
        for m in (g, o):
            m.setTargetAreas(ta)
            m.setTargetEdgeLengths(tl)
            m.setStiffness(k)
            m.setCompressibility(c)
            contacts(m)
            m.updateForceEnergy()
        assert g.getEnergy() == pytest.approx(o.getEnergy(), rel=1e-11)
        assert_forces_close(g.getForces(), o.getForces())


# ------------------------------------------------------------------ constraints
def test_shake_parity(system):
    g, o = pair(system)
    it_g = g.shakeProject(100, 1e-15)
    it_o = o.shakeProject(100, 1e-15)
    assert abs(it_g - it_o) <= 1
    assert it_g < 100
    d = (np.asarray(g.getPositions()) - o.getPositions() + 0.5) % 1.0 - 0.5
    assert np.abs(d).max() < 1e-12
    g.updatePolygonGeometry()
    np.testing.assert_allclose(g.getAreas(), system.target_areas, rtol=1e-10)
    el = np.asarray(g.getEdgeLengths())
    np.testing.assert_allclose(el, np.repeat(system.target_edge_lengths, system.n_array),
                               rtol=1e-10)


@pytest.mark.parametrize("P,n", [(4096, 32), (4096, 16), (2048, 24)])
def test_shake_parity_at_scale(P, n):
    """Thousands of polygons: many warps resident on every SM at once, the
    conditions of the FIRE workload.  The iteration count and the positions
    follow the oracle, and a second run gives the same bits."""
    s = make_system(P, n, 0.88, seed=5)
    g, o = pair(s)
    it_o = o.shakeProject(200, 1e-15)
    it_g = g.shakeProject(200, 1e-15)
    x_g = np.asarray(g.getPositions()).copy()
    assert abs(it_g - it_o) <= 1
    d = (x_g - o.getPositions() + 0.5) % 1.0 - 0.5
    assert np.abs(d).max() < 1e-12
    g2 = load_into(lib.Model(s.num_vertices), s)
    assert g2.shakeProject(200, 1e-15) == it_g
    assert np.array_equal(np.asarray(g2.getPositions()), x_g)


def test_xpbd_parity(system):
    g, o = pair(system)
    ig = g.xpbdProject(5, 0.0)
    io = o.xpbdProject(5, 0.0)
    assert ig == io == 5
    d = (np.asarray(g.getPositions()) - o.getPositions() + 0.5) % 1.0 - 0.5
    assert np.abs(d).max() < 1e-12


# ------------------------------------------------------------------ FIRE
def test_fire_steps_parity():
    _fire_steps_parity(make_system(64, 16, 0.85, seed=2), 30)


def test_fire_steps_parity_general_kernels():
    """Polygons of 12 to 48 vertices: inside the step graph the projection is
    the warp-per-polygon form with a shared-memory workspace, SHAKE the
    shared-memory form, and the force forms its own edge vectors (the
    one-vertex-per-lane kernels and the precomputed tangents and edge vectors
    serve polygons of at most 32 vertices only)."""
    n = np.random.default_rng(21).integers(12, 49, 120)
    assert n.max() > 32
    _fire_steps_parity(make_system(120, n, 0.86, seed=13), 15)


def test_fire_steps_parity_thread_per_polygon():
    """20000 polygons, more than 128 per SM: inside the step graph the
    projection takes its thread-per-polygon form."""
    # the SHAKE count is the largest over 20000 polygons, so one polygon at
    # the rounding floor of the stop test moves it: half the steps equal
    # (3 of 4 were in the runs so far)
    _fire_steps_parity(make_system(20000, 8, 0.85, seed=17), 4, same_frac=0.5)


def _fire_steps_parity(s, steps, same_frac=0.8):
    """Each FIRE step of the CUDA path against one oracle step from the CUDA
    path's state (tests/fire_shadow.py: energy 1e-12, positions 1e-12,
    forces and velocities 1e-10 on plain steps).  The velocities read
    between steps include the step's deferred bend (model.cpp:471-484), and
    the next step does not bend them again."""
    g, o = pair(s)
    for m in (g, o):
        m.shakeProject(200, 1e-15)
        contacts(m)
        m.updateForceEnergy()
        m.projectForce()
    sh = FireShadow(g, o)
    st = (1e-3, 0.1, 0)
    for _ in range(steps):
        st = sh.step(*st)[1:]
    sh.check_counts(same_frac=same_frac)
    assert sh.plain > 0


@pytest.mark.parametrize("mt,k,c,dt0", [(3, 1.0, 1.0, 1.0), (5, 1.0, 1.0, 0.1), (1, 2.0, 0.0, 0.3),
                                        (2, 0.0, 3.0, 0.3)])
def test_fire_steps_soft_models_parity(mt, k, c, dt0):
    """FIRE steps of the models without SHAKE (softBody, hybrid, edgeOnly,
    areaOnly): the velocity half-kick and the sums in k_fire_velocity, the
    energy rollback ending with k_fire_maxf (softBody and hybrid roll back
    here), the step bookkeeping and the bend deferred to the next step."""
    s = make_system(64, 16, 0.85, seed=2)
    g, o = pair(s)
    g.setModelEnum(lib.modelEnum(mt))
    o.setModelEnum(mt)
    for m in (g, o):
        m.setTargetAreas(s.target_areas * 1.05)
        m.setTargetEdgeLengths(s.target_edge_lengths * 0.97)
        m.setStiffness(k)
        m.setCompressibility(c)
        contacts(m)
        m.updateForceEnergy()
    sh = FireShadow(g, o, shake=False)
    st = (dt0, 0.1, 0)
    for _ in range(25):
        st = sh.step(*st, 1.0)[1:]
    assert sh.plain == 25


def test_fire_rollback_state_matches_reference():
    """An energy-increase rollback (model.cpp:450-470) leaves the step's start
    positions, the force, energy and max |F| there, and the contact records of
    those positions: the oracle recomputes them all, as the reference does;
    the GPU restores its step-start snapshot and refreshes the records when
    they are read.  This system's FIRE run rolls back at step 42."""
    s = make_system(32, 12, 0.88, seed=9)
    g, o = pair(s)
    for m in (g, o):
        m.shakeProject(200, 1e-15)
        contacts(m)
        m.updateForceEnergy()
        m.projectForce()
    sh = FireShadow(g, o)
    st = (1e-3, 0.1, 0)
    rolled = None
    for step in range(60):
        x_g = np.asarray(g.getPositions()).copy()
        rg = sh.step(*st)
        st = rg[1:]
        if np.array_equal(np.asarray(g.getPositions()), x_g) and g.getLastShakeIters() < 50:
            rolled = step
            break
    assert rolled is not None and sh.plain == sh.n
    # the oracle's step from the same state rolled back too and recomputed
    # the records there
    assert np.array_equal(np.asarray(o.getPositions()), x_g)
    assert_records_equal(g, o)
    # and the run continues from the restored state
    sh.step(*st)


@pytest.mark.parametrize("seed,dt,shake_iter,fails", [(1, 0.2, 1, False), (1, 1.0, 1, True),
                                                      (2, 0.5, 2, True)])
def test_fire_step_shake_retry_and_failure_match_reference(seed, dt, shake_iter, fails):
    """Large first steps: SHAKE needs its retry with ten times the iterations
    (model.cpp:431-436), and where the retry fails too, the step restores its
    start positions and zeroes the velocities (model.cpp:437-449); the force
    and its projection at the end are then those of the restored positions."""
    s = make_system(64, 16, 0.85, seed=seed)
    g, o = pair(s)
    for m in (g, o):
        m.shakeProject(200, 1e-15)
        contacts(m)
        m.updateForceEnergy()
        m.projectForce()
    xg0 = np.asarray(g.getPositions()).copy()
    xo0 = np.asarray(o.getPositions()).copy()
    args = (dt, 0.1, 0, 0.1, 0.1, 0.99, 1.1, 0.5, 5, shake_iter)
    rg = g.minimizeFIREStep(*args)
    ro = o.minimizeFIREStep(*args)
    assert o.getLastShakeIters() >= shake_iter          # the retry ran
    assert g.getLastShakeIters() == pytest.approx(o.getLastShakeIters(), abs=1)
    assert np.array_equal(np.asarray(o.getPositions()), xo0) == fails
    assert np.array_equal(np.asarray(g.getPositions()), xg0) == fails
    assert rg[1:] == ro[1:]
    d = (np.asarray(g.getPositions()) - o.getPositions() + 0.5) % 1.0 - 0.5
    if fails:
        # back at the step-start state: the usual tolerances.  The force
        # there comes from records of the moved positions (huge), so the
        # next steps are short ones: the first rolls back on an energy
        # increase, the others proceed.
        assert rg[0] == pytest.approx(ro[0], rel=1e-12)
        assert np.abs(d).max() < 1e-12
        assert_forces_close(g.getForces(), o.getForces())
        assert g.getMaxUnbalancedForce() == pytest.approx(o.getMaxUnbalancedForce(), rel=1e-10)
        sh = FireShadow(g, o)
        st = (1e-5,) + tuple(rg[2:])
        for _ in range(3):
            st = sh.step(*st)[1:]
        assert sh.plain == 3
    else:
        # the retry starts from the first call's unconverged iterate, which
        # the two SHAKEs reach only up to the rounding of their FP32 Newton
        # corrections; the retry's end point moves with it along the
        # constraint manifold (tests/fire_shadow.py), and the energy and
        # force follow
        assert rg[0] == pytest.approx(ro[0], rel=1e-9)
        assert np.abs(d).max() < 1e-9
        of = np.asarray(o.getForces())
        assert np.abs(np.asarray(g.getForces()) - of).max() <= 1e-7 * np.abs(of).max()


def test_minimize_fire_matches_step_loop():
    """Model::minimizeFIRE (graph loop with the stop test on the device) walks
    the same trajectory as repeated minimizeFIREStep calls."""
    s = make_system(64, 16, 0.85, seed=4)
    a = load_into(lib.Model(s.num_vertices), s)
    b = load_into(lib.Model(s.num_vertices), s)
    for m in (a, b):
        m.shakeProject(200, 1e-15)
        contacts(m)
    ea, dta, steps = a.minimizeFIRE(1e-10, 1e-3, 40)
    b.resetVelocities()
    b.updatePolygonGeometry()
    b.updateForceEnergy()
    b.projectForce()
    st = (1e-3, 0.1, 0)
    for _ in range(40):
        r = b.minimizeFIREStep(*st)
        st = r[1:]
    assert steps == 40
    assert dta == pytest.approx(st[0], rel=1e-12)
    assert a.getEnergy() == pytest.approx(b.getEnergy(), rel=1e-9)


def test_large_system_contacts_and_force():
    """4096 polygons of 32 vertices (131,072 vertices): bit-exact records and
    force parity for one evaluation."""
    s = make_system(4096, 32, 0.88, seed=42)
    g, o = pair(s)
    for m in (g, o):
        contacts(m)
        m.updateForceEnergy()
    assert_records_equal(g, o)
    assert g.getEnergy() == pytest.approx(o.getEnergy(), rel=ENERGY_RTOL)
    assert_forces_close(g.getForces(), o.getForces())


def test_wrong_position_length_is_ignored_like_reference(capfd):
    s = make_system(8, 6, 0.5, seed=0)
    g = load_into(lib.Model(s.num_vertices), s)
    before = np.asarray(g.getPositions()).copy()
    g.setPositions(np.zeros(3))
    out = capfd.readouterr().out
    assert "Update numVertices" in out
    np.testing.assert_array_equal(g.getPositions(), before)
