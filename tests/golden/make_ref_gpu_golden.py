"""Golden vectors from the reference's own GPU kernels (run on a GPU machine).

The reference has no CPU implementation of the overlap path, so its outputs
come from its own CUDA code: oracle/ref_build.py compiles the reference's
src/model.cu and src/model.cpp (sources staged beforehand into the
git-ignored oracle/_ref/src) with the driver oracle/ref_golden.cpp, which
calls the reference's `Model` methods.  This script generates the systems,
runs that binary once per case and writes tests/golden/ref_gpu_<case>.npz
holding the inputs and everything the reference computed.  The fixtures are
committed; tests/test_ref_gpu_golden.py checks the CPU oracle (and, on a GPU,
the CUDA path) against them.

Usage (on a machine with a GPU and the staged sources):
    python tests/golden/make_ref_gpu_golden.py --out DIR

Before a case runs its overlap-force kernels on the GPU, the CPU oracle checks
that every crossing record has an exit partner.  The reference's exterior
kernel (src/kernels.cuh:1067-1273) returns early for a record without one,
before a block barrier and without writing its shared-memory slot of the
energy sum; such cases are run for their contact records only.
"""
import argparse
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from oracle import ref_build  # noqa: E402
from pycudapolygon_gb300.systems import PolygonSystem, make_system  # noqa: E402

F_FORCE, F_PROJECT, F_MC, F_SOFT, F_HYBRID = 1, 2, 4, 8, 16
TYPES = {0: np.float64, 1: np.int32, 2: np.uint64, 3: np.uint8}


def testsaver_system():
    fx = json.load(open(os.path.join(HERE, "testsaver.json")))
    n_array = np.asarray(fx["n_array"], dtype=np.int32)
    pos = np.asarray(fx["positions"], dtype=np.float64)
    start = np.concatenate([[0], np.cumsum(n_array)]).astype(np.int32)
    P = n_array.size
    # targets as the saved state's own areas and mean edge lengths
    xy = pos.reshape(-1, 2)
    ta = np.zeros(P)
    tl = np.zeros(P)
    for p in range(P):
        ring = xy[start[p]:start[p + 1]]
        d = np.roll(ring, -1, axis=0) - ring
        d = (d + 1.5) % 1.0 - 0.5
        rel = np.concatenate([[np.zeros(2)], np.cumsum(d[:-1], axis=0)])
        x, y = rel[:, 0], rel[:, 1]
        ta[p] = 0.5 * (np.dot(x, np.roll(y, -1)) - np.dot(np.roll(x, -1), y))
        tl[p] = np.sum(np.linalg.norm(d, axis=1)) / ring.shape[0]
    return PolygonSystem(positions=pos, n_array=n_array, start_indices=start,
                         target_areas=ta, target_edge_lengths=tl,
                         max_edge_length=0.25, phi=0.0)


def odd_system():
    """Polygons the crossing search must handle: a bow tie, a pentagram, a
    reflex hexagon, a polygon with a repeated vertex, a thin sliver, regular
    polygons overlapping them and one across the periodic boundary."""
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

    def reg(n):
        return [(np.cos(2 * np.pi * k / n), np.sin(2 * np.pi * k / n)) for k in range(n)]
    for c in [(0.22, 0.23), (0.52, 0.48), (0.81, 0.27), (0.31, 0.71), (0.72, 0.70), (0.995, 0.5)]:
        rings.append(at(c, reg(12), 0.03))
    n_array = np.array([len(r) for r in rings], dtype=np.int32)
    start = np.concatenate([[0], np.cumsum(n_array)]).astype(np.int32)
    pos = np.array([xy for r in rings for xy in r], dtype=np.float64).reshape(-1)
    P = len(rings)
    return PolygonSystem(positions=pos, n_array=n_array, start_indices=start,
                         target_areas=np.full(P, 1e-3), target_edge_lengths=np.full(P, 0.01),
                         max_edge_length=0.1, phi=0.0)


def cases():
    """(name, system, max_edge_length, flags, point_density, stiffness, compressibility)."""
    c1 = make_system(64, 16, 0.85, seed=11)
    dense = make_system(96, 20, 0.97, seed=23)
    varn = make_system(120, np.random.default_rng(31).integers(5, 41, 120), 0.88, seed=32)
    mid = make_system(256, 24, 0.87, seed=6)
    # one crossing record of this system has no exit partner
    mid_unpaired = make_system(256, 24, 0.87, seed=5)
    every = F_FORCE | F_PROJECT | F_MC | F_SOFT | F_HYBRID
    return [
        ("testsaver", testsaver_system(), 0.25, every, 128, 1.0, 1.0),
        ("c1_64x16", c1, c1.max_edge_length, every, 256, 1.0, 1.0),
        ("c1_64x16_box2", c1, 0.5, F_FORCE | F_PROJECT, 0, 0.0, 0.0),
        ("c1_64x16_box1", c1, 1.0, F_FORCE, 0, 0.0, 0.0),
        ("dense_96x20", dense, dense.max_edge_length, F_FORCE | F_PROJECT | F_MC, 200, 0.0, 0.0),
        # ragged polygons: the reference's projection assumes one n for every
        # polygon (model.cpp:570), so it is not run here
        ("ragged_120", varn, varn.max_edge_length, F_FORCE | F_SOFT | F_HYBRID, 0, 2.0, 0.5),
        ("mid_256x24", mid, mid.max_edge_length, F_FORCE | F_PROJECT, 0, 0.0, 0.0),
        ("mid_256x24_unpaired", mid_unpaired, mid_unpaired.max_edge_length, F_FORCE, 0, 0.0, 0.0),
        ("odd_shapes", odd_system(), 0.1, F_FORCE | F_MC, 160, 0.0, 0.0),
        ("odd_shapes_box3", odd_system(), 1.0 / 3, F_FORCE, 0, 0.0, 0.0),
    ]


def all_paired(system, max_edge):
    """True when the oracle finds an exit partner for every crossing record."""
    m = orc.OracleModel(system.num_vertices)
    m.setNumVertices(system.num_vertices)
    m.setStartIndices(system.start_indices)
    m.setPositions(system.positions)
    m.setTargetAreas(system.target_areas)
    m.setTargetEdgeLengths(system.target_edge_lengths)
    m.initializeNeighborCells()
    m.setMaxEdgeLength(max_edge)
    m.updatePolygonGeometry()
    m.updateNeighborCells()
    m.updateNeighbors()
    m.updateOutersections()
    keys = m.getIntersections()
    outs = m.getOutersections()
    return bool(np.all(keys != outs)), int(keys.size)


def write_input(path, system, max_edge, flags, pd, k, c):
    V, P = system.num_vertices, system.num_polygons
    with open(path, "wb") as f:
        f.write(struct.pack("<6i", 0x47504350, 1, V, P, flags, pd))
        f.write(struct.pack("<3d", max_edge, k, c))
        f.write(np.asarray(system.start_indices, dtype="<i4").tobytes())
        f.write(np.asarray(system.positions, dtype="<f8").tobytes())
        f.write(np.asarray(system.target_areas, dtype="<f8").tobytes())
        f.write(np.asarray(system.target_edge_lengths, dtype="<f8").tobytes())


def read_output(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    o = 0
    while o < len(data):
        (n,) = struct.unpack_from("<i", data, o)
        o += 4
        name = data[o:o + n].decode()
        o += n
        t, count = struct.unpack_from("<iq", data, o)
        o += 12
        dt = np.dtype(TYPES[t]).newbyteorder("<")
        arr = np.frombuffer(data, dtype=dt, count=count, offset=o).copy()
        o += count * dt.itemsize
        out[name] = arr
    return out


def compact_slots(out, V):
    """Keep only the used neighbour slots (vertex-major, numNeighbors each)."""
    cnt = out.pop("num_neighbors")
    M = out["neighbors"].size // V
    nb = out.pop("neighbors").reshape(V, M)
    ins = out.pop("inside").reshape(V, M)
    used = np.minimum(cnt, M)
    mask = np.arange(M)[None, :] < used[:, None]
    out["num_neighbors"] = cnt
    out["neighbor_slots"] = nb[mask]
    out["inside_slots"] = ins[mask]
    out["max_neighbors"] = np.array([M], dtype=np.int32)


def run(out_dir, only=None):
    binary = ref_build.build()
    os.makedirs(out_dir, exist_ok=True)
    summary = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, system, max_edge, flags, pd, k, c in cases():
            if only and name not in only:
                continue
            paired, n_rec = all_paired(system, max_edge)
            if not paired:
                flags &= ~(F_FORCE | F_PROJECT | F_HYBRID)
            fin = os.path.join(tmp, name + ".in")
            fout = os.path.join(tmp, name + ".out")
            write_input(fin, system, max_edge, flags, pd, k, c)
            subprocess.run([binary, fin, fout], check=True, timeout=300)
            out = read_output(fout)
            compact_slots(out, system.num_vertices)
            out.pop("shape_id", None)
            if system.num_vertices > 3000:
                # the constraint vectors of the large cases (6V doubles) are
                # left out to keep the fixtures small; smaller cases hold them
                out.pop("constraints", None)
            if "intersections_counter" in out:
                ic = out.pop("intersections_counter")
                nz = np.nonzero(ic)[0].astype(np.int32)
                out["counter_index"] = nz
                out["counter_value"] = ic[nz]
            inputs = dict(in_positions=system.positions, in_start=system.start_indices,
                          in_target_areas=system.target_areas,
                          in_target_edge_lengths=system.target_edge_lengths,
                          in_max_edge_length=np.array([max_edge]),
                          in_flags=np.array([flags], dtype=np.int32),
                          in_point_density=np.array([pd], dtype=np.int32),
                          in_stiffness=np.array([k]), in_compressibility=np.array([c]))
            np.savez_compressed(os.path.join(out_dir, "ref_gpu_%s.npz" % name), **inputs, **out)
            summary[name] = dict(V=system.num_vertices, P=system.num_polygons, flags=flags,
                                 records=int(out["num_intersections"][0]),
                                 oracle_records=n_rec, all_paired=paired,
                                 energy=float(out["energy"][0]) if "energy" in out else None)
            print(name, summary[name], flush=True)
    with open(os.path.join(out_dir, "ref_gpu_summary.json"), "w") as f:
        json.dump(summary, f, indent=1)
    return summary


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--only", nargs="*")
    a = ap.parse_args()
    run(a.out, a.only)
