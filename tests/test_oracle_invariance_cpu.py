"""Symmetries of the reference's overlap path, checked on the oracle.

The contact records, their partners, the energy and the force of the
reference (kernels.cuh:709-1424) depend on the polygons, not on where the
box's origin is or how polygons and vertices are numbered:
  * a periodic translation of every vertex leaves the records and
    outersections bit-identical, the energy within 1e-12 relative and the
    force within 1e-10 of its largest component;
  * renumbering the polygons and rotating each polygon's vertex numbering
    maps the records, partners and forces onto each other the same way;
  * a half turn (x -> -x) keeps the records and the energy and negates the
    force.
A quarter turn keeps the records but not the energy: a lens's energy
carries (Qx - Px)(Qy - Py) of its two crossings besides the overlap area
(the check in test_energy_semantics_cpu.py), and that term changes sign
under a quarter turn.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from pycudapolygon_gb300.systems import PolygonSystem, load_into, make_system


def _with_positions(s, xy, n_array=None, start=None, ta=None, tl=None):
    return PolygonSystem(positions=np.asarray(xy, dtype=np.float64).reshape(-1),
                         n_array=s.n_array if n_array is None else n_array,
                         start_indices=s.start_indices if start is None else start,
                         target_areas=s.target_areas if ta is None else ta,
                         target_edge_lengths=s.target_edge_lengths if tl is None else tl,
                         max_edge_length=s.max_edge_length, phi=s.phi)


def _evaluate(s):
    o = load_into(orc.OracleModel(s.num_vertices), s)
    o.updatePolygonGeometry()
    o.updateNeighborCells()
    o.updateNeighbors()
    o.updateOutersections()
    o.updateForceEnergy()
    return (o.getIntersections(), o.getOutersections(), o.getEnergy(),
            np.asarray(o.getForces()).reshape(-1, 2))


def _fields(keys):
    k = np.asarray(keys, dtype=np.uint64)
    return ((k >> np.uint64(48)).astype(np.int64), ((k >> np.uint64(32)) & np.uint64(0xFFFF)).astype(np.int64),
            ((k >> np.uint64(16)) & np.uint64(0xFFFF)).astype(np.int64),
            (k & np.uint64(0xFFFF)).astype(np.int64))


@pytest.fixture(scope="module")
def base():
    n = np.random.default_rng(3).integers(8, 25, 128)
    s = make_system(128, n, 0.88, seed=21)
    return s, _evaluate(s)


@pytest.mark.parametrize("d", [(0.3, 0.7), (0.123456, 0.987654), (0.5, 0.0)])
def test_periodic_translation(base, d):
    s, (k, u, E, F) = base
    x = np.asarray(s.positions).reshape(-1, 2)
    k2, u2, E2, F2 = _evaluate(_with_positions(s, (x + d) % 1.0))
    assert k.size > 100
    assert np.array_equal(k, k2) and np.array_equal(u, u2)
    assert abs(E2 - E) <= 1e-12 * abs(E)
    assert np.abs(F2 - F).max() <= 1e-10 * np.abs(F).max()


def test_renumbering_polygons_and_vertices(base):
    s, (k, u, E, F) = base
    x = np.asarray(s.positions).reshape(-1, 2)
    st = np.asarray(s.start_indices)
    n = np.diff(st)
    rng = np.random.default_rng(5)
    perm = rng.permutation(n.size)              # new polygon q is old polygon perm[q]
    inv = np.empty_like(perm)
    inv[perm] = np.arange(perm.size)
    rot = rng.integers(0, 1000, n.size) % n     # new vertex l is old vertex (l + rot) mod n
    rings = [np.roll(x[st[p]:st[p + 1]], -rot[p], axis=0) for p in perm]
    n2 = n[perm].astype(np.int32)
    st2 = np.concatenate([[0], np.cumsum(n2)]).astype(np.int32)
    s2 = _with_positions(s, np.concatenate(rings), n_array=n2, start=st2,
                         ta=np.asarray(s.target_areas)[perm],
                         tl=np.asarray(s.target_edge_lengths)[perm])
    k2, u2, E2, F2 = _evaluate(s2)

    def renumber(key_fields):
        sj, si, i, j = key_fields
        return list(zip(inv[sj].tolist(), inv[si].tolist(), ((i - rot[si]) % n[si]).tolist(),
                        ((j - rot[sj]) % n[sj]).tolist()))
    old = dict(zip(renumber(_fields(k)), renumber(_fields(u))))
    new = dict(zip(zip(*[f.tolist() for f in _fields(k2)]), zip(*[f.tolist() for f in _fields(u2)])))
    assert old == new                           # the same records with the same partners
    assert abs(E2 - E) <= 1e-12 * abs(E)
    poly = np.repeat(np.arange(n.size), n)
    loc = np.arange(x.shape[0]) - st[poly]
    where = st2[inv[poly]] + (loc - rot[poly]) % n[poly]
    assert np.abs(F2[where] - F).max() <= 1e-10 * np.abs(F).max()


def test_half_turn_and_quarter_turn(base):
    s, (k, u, E, F) = base
    x = np.asarray(s.positions).reshape(-1, 2)
    turns = [x, np.stack([-x[:, 1], x[:, 0]], 1), -x, np.stack([x[:, 1], -x[:, 0]], 1)]
    out = [_evaluate(_with_positions(s, t % 1.0)) for t in turns]
    for k2, u2, _, _ in out:
        assert np.array_equal(k, k2) and np.array_equal(u, u2)
    e = [o[2] for o in out]
    # half turns: the same energy, the force negated
    assert abs(e[2] - e[0]) <= 1e-12 * abs(e[0]) and abs(e[3] - e[1]) <= 1e-12 * abs(e[1])
    assert np.abs(out[2][3] + F).max() <= 1e-10 * np.abs(F).max()
    # quarter turn: the chord terms change sign
    assert abs(e[1] - e[0]) > 1e-3 * abs(e[0])
