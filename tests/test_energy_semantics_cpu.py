"""What the reference's overlap energy measures (kernels.cuh:139-159 for h,
:1067-1273 and :1354-1424 for the chains), checked on the oracle against an
exact polygon clipping: for two convex polygons whose boundaries cross twice,
at P and Q, the energy is the overlap area plus (Qx - Px)(Qy - Py).

Each record's chain (the boundary of one polygon inside the other, from its
entry crossing to its exit) sums trapezoids relative to its own entry point;
the two chains of a lens start at different crossings, and the shift between
them adds the chord term.  So the energy is not the overlap area and is not
invariant under rotation, which is one reason the FIRE runs of the reference
stop by stagnation instead of reaching a vanishing force.

Tolerance 1e-6 relative: the reference takes the crossing points from
float-rounded parameters (kernels.cuh:853-858).
"""
import numpy as np

from oracle import oracle as orc
from pycudapolygon_gb300.systems import PolygonSystem, load_into


def _clip(subject, clipper):
    """Sutherland-Hodgman: subject polygon clipped by a convex,
    counter-clockwise clipper."""
    out = [np.asarray(p, dtype=np.float64) for p in subject]
    n = len(clipper)
    for k in range(n):
        a, b = np.asarray(clipper[k]), np.asarray(clipper[(k + 1) % n])
        inside = lambda p: (b[0] - a[0]) * (p[1] - a[1]) - (b[1] - a[1]) * (p[0] - a[0]) >= 0  # noqa: E731

        def cut(p, q):
            r, s = q - p, b - a
            t = ((a[0] - p[0]) * s[1] - (a[1] - p[1]) * s[0]) / (r[0] * s[1] - r[1] * s[0])
            return p + t * r
        src, out = out, []
        if not src:
            break
        prev = src[-1]
        for p in src:
            if inside(p):
                if not inside(prev):
                    out.append(cut(prev, p))
                out.append(p)
            elif inside(prev):
                out.append(cut(prev, p))
            prev = p
    return out


def _area(pts):
    p = np.asarray(pts)
    x, y = p[:, 0], p[:, 1]
    return 0.5 * (np.dot(x, np.roll(y, -1)) - np.dot(np.roll(x, -1), y))


def _regular(c, r, n, theta):
    k = np.arange(n)
    return np.stack([c[0] + r * np.cos(theta + 2 * np.pi * k / n),
                     c[1] + r * np.sin(theta + 2 * np.pi * k / n)], axis=1)


def _crossing(x, start, key):
    sj, si = int(key >> np.uint64(48)), int((key >> np.uint64(32)) & np.uint64(0xFFFF))
    i, j = int((key >> np.uint64(16)) & np.uint64(0xFFFF)), int(key & np.uint64(0xFFFF))
    b1, n1 = start[si], start[si + 1] - start[si]
    b2, n2 = start[sj], start[sj + 1] - start[sj]
    p, q = x[b1 + i], x[b2 + j]
    r, s = x[b1 + (i + 1) % n1] - p, x[b2 + (j + 1) % n2] - q
    t = ((q[0] - p[0]) * s[1] - (q[1] - p[1]) * s[0]) / (r[0] * s[1] - r[1] * s[0])
    return p + t * r


def test_lens_energy_is_area_plus_chord_term():
    rng = np.random.default_rng(0)
    checked = off = 0
    for _ in range(60):
        n1, n2 = (int(v) for v in rng.integers(5, 13, 2))
        a = _regular((0.5, 0.5), 0.1, n1, rng.random() * 6.0)
        b = _regular((0.5 + 0.15 * rng.random(), 0.5 + 0.08 * rng.random()), 0.08, n2,
                     rng.random() * 6.0)
        x = np.concatenate([a, b])
        start = np.array([0, n1, n1 + n2], dtype=np.int32)
        system = PolygonSystem(positions=x.reshape(-1), n_array=np.diff(start), start_indices=start,
                               target_areas=np.ones(2), target_edge_lengths=np.ones(2),
                               max_edge_length=0.5, phi=0.1)
        o = load_into(orc.OracleModel(n1 + n2), system)
        o.updatePolygonGeometry()
        o.updateNeighborCells()
        o.updateNeighbors()
        o.updateOutersections()
        o.updateForceEnergy()
        keys = o.getIntersections()
        if len(keys) != 2:
            continue
        p, q = (_crossing(x, start, k) for k in keys)
        area = _area(_clip(list(a), list(b)))
        expect = area + (q[0] - p[0]) * (q[1] - p[1])
        e = o.getEnergy()
        assert abs(e - expect) <= 1e-6 * abs(expect) + 1e-12, (e, expect, area)
        checked += 1
        off += abs(e - area) > 0.01 * area
    assert checked >= 20
    assert off >= checked // 2      # the energy is, as a rule, not the overlap area
