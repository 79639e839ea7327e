"""Seeded synthetic polygon systems (the inputs the hot path runs on).

The reference publishes no benchmark inputs, so systems are generated the way
its own generator and setters shape them (pyCudaPolygon/polygonMixins/
polygonUtils.py:52-89 for star polygons around a centre, pyCudaPolygon.py:
182-203 for the 50:50 bidisperse split with the small half first):

  * centre ~ U[0,1)^2, rotation ~ U[0, 2 pi)
  * vertex k at angle theta + 2 pi k / n, radius R_p (1 + 0.1 u_k), u ~ U[-1,1]
    (counter-clockwise, positive area)
  * first half of the polygons small, second half 1.4x larger radius
  * one global scale so that the sum of the shoelace areas equals phi
  * positions wrapped into [0, 1)
  * targetAreas = initial areas, targetEdgeLengths = perimeter / n (one
    scalar per polygon, as the reference stores it, model.cpp:553)
  * maxEdgeLength = the longest actual edge (pyCudaPolygon.py:166-179)

Everything is FP64 numpy; positions are interleaved x, y per vertex.
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class PolygonSystem:
    positions: np.ndarray        # float64 [2V], interleaved, in [0, 1)
    n_array: np.ndarray          # int32 [P]
    start_indices: np.ndarray    # int32 [P+1]
    target_areas: np.ndarray     # float64 [P]
    target_edge_lengths: np.ndarray  # float64 [P]
    max_edge_length: float
    phi: float

    @property
    def num_vertices(self):
        return int(self.start_indices[-1])

    @property
    def num_polygons(self):
        return int(self.n_array.size)


def _shoelace(xy):
    x, y = xy[:, 0], xy[:, 1]
    return 0.5 * (np.dot(x, np.roll(y, -1)) - np.dot(np.roll(x, -1), y))


def random_polygon(rng, n):
    """One random star polygon around the origin (polygonUtils.py:55-61):
    cumulative random angles scaled to a full turn, random radii, size 1/8.
    The same draws from `rng` in the same order as the reference."""
    angles = np.cumsum(np.concatenate(([0.0], rng.random(n - 1))))
    angles *= 2 * np.pi / angles[-1]
    radii = rng.random(n)
    return np.stack([radii * np.cos(angles), radii * np.sin(angles)], axis=1) / 8


def random_polygons(rng, num_polygons, n):
    """Positions [2 P n] of `num_polygons` random polygons of `n` vertices
    (polygonUtils.py:63-91): each is rotated about its vertex mean by a
    random angle, translated by a random offset and wrapped into the unit
    box.  The same draws from `rng` in the same order as the reference, so a
    generator seeded alike gives the same positions."""
    out = np.zeros((num_polygons * n, 2))
    for i in range(num_polygons):
        pos = random_polygon(rng, n)
        ang = rng.random() * 2 * np.pi
        c = pos.mean(axis=0)
        ca, sa = np.cos(ang), np.sin(ang)
        rot = np.empty_like(pos)
        for k in range(n):     # vertex by vertex, as the reference's rotate()
            dx, dy = pos[k, 0] - c[0], pos[k, 1] - c[1]
            rot[k] = (dx * ca - dy * sa + c[0], dx * sa + dy * ca + c[1])
        rot[:, 0] += rng.random()
        rot[:, 1] += rng.random()
        rot = (rot + 2) % 1
        out[i * n:(i + 1) * n] = rot
    out = (out + 1) % 1
    return out.reshape(-1)


def unwrapped_scale(positions, start, target_areas):
    """Each polygon rescaled about its vertex mean to its target area
    (setAreas, pyCudaPolygon.py:103-144): unwrapped relative to its first
    vertex, shoelace area (absolute value), scaled by sqrt(target / area) and
    wrapped into [0, 1).  Polygons of zero area are left as they are."""
    xy = np.asarray(positions, dtype=np.float64).reshape(-1, 2).copy()
    for i in range(len(start) - 1):
        s, e = int(start[i]), int(start[i + 1])
        poly = xy[s:e].copy()
        ref = poly[0].copy()
        for j in range(1, e - s):
            d = poly[j] - ref
            d = d - np.round(d)
            poly[j] = ref + d
        x, y = poly[:, 0], poly[:, 1]
        area = 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(np.roll(x, -1), y))
        if area <= 0:
            continue
        scale = np.sqrt(target_areas[i] / area)
        centroid = poly.mean(axis=0)
        xy[s:e] = np.mod((poly - centroid) * scale + centroid, 1.0)
    return xy.reshape(-1)


def make_system(num_polygons, n, phi, seed, ratio=1.4, jitter=0.1):
    """Generate one system.  `n` is an int (uniform) or an int array [P]."""
    rng = np.random.default_rng(seed)
    P = int(num_polygons)
    n_array = np.full(P, int(n), dtype=np.int32) if np.isscalar(n) else \
        np.asarray(n, dtype=np.int32).copy()
    assert n_array.size == P and np.all(n_array >= 3)
    centres = rng.random((P, 2))
    theta0 = rng.random(P) * 2.0 * np.pi
    radius = np.ones(P)
    radius[P // 2:] = ratio
    shapes = []
    for p in range(P):
        k = np.arange(n_array[p])
        u = rng.uniform(-1.0, 1.0, n_array[p])
        ang = theta0[p] + 2.0 * np.pi * k / n_array[p]
        r = radius[p] * (1.0 + jitter * u)
        shapes.append(np.stack([r * np.cos(ang), r * np.sin(ang)], axis=1))
    total = sum(_shoelace(s) for s in shapes)
    scale = np.sqrt(phi / total)
    V = int(n_array.sum())
    pos = np.zeros((V, 2))
    start = np.concatenate([[0], np.cumsum(n_array)]).astype(np.int32)
    areas = np.zeros(P)
    perims = np.zeros(P)
    for p in range(P):
        local = shapes[p] * scale
        areas[p] = _shoelace(local)
        perims[p] = np.sum(np.linalg.norm(np.roll(local, -1, axis=0) - local, axis=1))
        pos[start[p]:start[p + 1]] = np.mod(local + centres[p], 1.0)
    pos = np.mod(pos, 1.0)
    # longest actual edge under the minimum image (pyCudaPolygon.py:166-179)
    nxt = np.arange(V) + 1
    nxt[start[1:] - 1] = start[:-1]
    d = pos[nxt] - pos
    d = (d + 1.5) % 1.0 - 0.5
    max_edge = float(np.max(np.sqrt(np.sum(d * d, axis=1))))
    return PolygonSystem(positions=pos.reshape(-1).copy(), n_array=n_array,
                         start_indices=start, target_areas=areas,
                         target_edge_lengths=perims / n_array,
                         max_edge_length=max_edge, phi=float(phi))


def batched_specs(num_systems, seed, p_range=(64, 1024), n_range=(12, 48),
                  phi_range=(0.80, 0.92)):
    """Per-system (P, n array, phi, seed) for the many-systems workload:
    P ~ U{64..1024}, n per polygon ~ U{12..48}, phi ~ U[0.80, 0.92]."""
    rng = np.random.default_rng(seed)
    specs = []
    for s in range(num_systems):
        P = int(rng.integers(p_range[0], p_range[1] + 1))
        n = rng.integers(n_range[0], n_range[1] + 1, size=P).astype(np.int32)
        phi = float(rng.uniform(*phi_range))
        specs.append((P, n, phi, int(rng.integers(0, 2**31 - 1))))
    return specs


def shard_by_vertices(vertex_counts, world_size):
    """Assign independent systems to ranks with balanced total vertex counts
    (largest first, each to the least-loaded rank; ties to the lower rank).
    Returns one sorted list of system indices per rank.  Systems never
    exchange data, so the shards need no collective on the data path."""
    counts = [int(c) for c in vertex_counts]
    order = sorted(range(len(counts)), key=lambda i: (-counts[i], i))
    loads = [0] * world_size
    shards = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (loads[k], k))
        shards[r].append(i)
        loads[r] += counts[i]
    return [sorted(x) for x in shards]


def load_into(model, system, model_type=None):
    """Configure a reference-API model object (the pybind `Model`, or any
    object with the same method names) with a generated system.  The cell
    size is set after initializeNeighborCells, so the Python wrapper's reset
    to 0.5 (pyCudaPolygon.py:54-57) does not undo it."""
    model.setNumVertices(system.num_vertices)
    model.setStartIndices(system.start_indices)
    model.setPositions(system.positions)
    model.setTargetAreas(system.target_areas)
    model.setTargetEdgeLengths(system.target_edge_lengths)
    if model_type is not None:
        model.setModelEnum(model_type)
    model.initializeNeighborCells()
    model.setMaxEdgeLength(system.max_edge_length)
    return model
