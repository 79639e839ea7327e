"""The reference's own kernels beside this repository's, on the same GPU and
the same system (TEST INFRASTRUCTURE: a measurement, not part of the library).

The reference's CUDA path is rebuilt for sm_103a by oracle/ref_build.py and
driven by oracle/ref_golden.cpp's timing mode.  The reference ships no FIRE
or SHAKE source, so the comparison covers the evaluation it does have, stage
by stage through each side's public Model methods: updatePolygonGeometry,
updateNeighborCells, updateNeighbors, updateOutersections, updateForceEnergy
and projectForce (model.cpp:252-395, model.cu:113-206).  Both sides are
timed on the host around each call and a device synchronisation, after one
warm-up evaluation, as the mean over `reps` evaluations (the reference's
methods allocate, copy and synchronise inside, so a device-event time would
not be their cost).  The workload is the benchmark's system: 4096 polygons x
32 vertices at packing fraction 0.88, cell size from the longest edge,
positions as generated.

The reference's exterior kernel returns early for a crossing record without
an exit partner, before a block barrier (src/kernels.cuh:1067-1273), and such
records occur (one to five in most 4096 x 32 systems).  So the seed is the
first from 2024 on whose records the CPU oracle finds all paired, and if none
of twenty is, only the contact stages are timed.

Usage (on a machine with a GPU, sources staged by `ref_build.py stage`):
    python oracle/ref_time.py [reps]      # one JSON object on stdout
"""
import json
import os
import struct
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from oracle import ref_build  # noqa: E402
from pycudapolygon_gb300.systems import load_into, make_system  # noqa: E402

N_POLY, N_VERT, PHI, SEED = 4096, 32, 0.88, 2024
STAGES = ["updatePolygonGeometry", "updateNeighborCells", "updateNeighbors",
          "updateOutersections", "updateForceEnergy", "projectForce"]
F_FORCE, F_PROJECT = 1, 2


def write_input(path, system, flags):
    """The driver's input file (format in oracle/ref_golden.cpp)."""
    V, P = system.num_vertices, system.num_polygons
    with open(path, "wb") as f:
        f.write(struct.pack("<6i", 0x47504350, 1, V, P, flags, 0))
        f.write(struct.pack("<3d", system.max_edge_length, 0.0, 0.0))
        f.write(np.asarray(system.start_indices, dtype="<i4").tobytes())
        f.write(np.asarray(system.positions, dtype="<f8").tobytes())
        f.write(np.asarray(system.target_areas, dtype="<f8").tobytes())
        f.write(np.asarray(system.target_edge_lengths, dtype="<f8").tobytes())


def oracle_records(system):
    """(every record has an exit partner, number of records) by the oracle."""
    o = load_into(orc.OracleModel(system.num_vertices), system)
    o.updatePolygonGeometry()
    o.updateNeighborCells()
    o.updateNeighbors()
    o.updateOutersections()
    keys, outs = o.getIntersections(), o.getOutersections()
    return bool(np.all(keys != outs)), int(keys.size)


def time_ours(system, reps, stages):
    import torch

    import pycudapolygon_gb300 as pg
    lib = pg.load_module()
    m = load_into(lib.Model(system.num_vertices), system)
    for st in stages:
        getattr(m, st)()
    torch.cuda.synchronize()
    total = dict.fromkeys(stages, 0.0)
    for _ in range(reps):
        for st in stages:
            t0 = time.perf_counter()
            getattr(m, st)()
            torch.cuda.synchronize()
            total[st] += time.perf_counter() - t0
    return {"reps": reps, "records": int(m.getNumIntersections()),
            "energy": float(m.getEnergy()) if "updateForceEnergy" in stages else 0.0,
            "stage_ms": {k: 1e3 * v / reps for k, v in total.items()}}


def main():
    reps = int(sys.argv[1]) if len(sys.argv) > 1 else 10
    for seed in range(SEED, SEED + 20):
        s = make_system(N_POLY, N_VERT, PHI, seed=seed)
        paired, records = oracle_records(s)
        if paired:
            break
    flags = F_FORCE | F_PROJECT if paired else 0
    stages = STAGES if paired else STAGES[:4]
    binary = ref_build.build()
    with tempfile.TemporaryDirectory() as td:
        inp, out = os.path.join(td, "in.bin"), os.path.join(td, "out.json")
        write_input(inp, s, flags)
        subprocess.run([binary, "--time", inp, str(reps), out], check=True, timeout=900)
        with open(out) as f:
            ref = json.load(f)
    ours = time_ours(s, reps, stages)
    ref_total = sum(ref["stage_ms"].values())
    our_total = sum(ours["stage_ms"].values())
    print(json.dumps({
        "workload": "%d polygons x %d vertices, phi %.2f, seed %d, %d vertices; cell size "
                    "%.6g (box size %d)" % (N_POLY, N_VERT, PHI, seed, s.num_vertices,
                                            s.max_edge_length, int(1.0 / s.max_edge_length)),
        "oracle_records": records, "all_records_paired": paired,
        "timing": "host clock around each Model method and a device synchronisation, mean "
                  "over %d evaluations after one warm-up" % reps,
        "reference_kernels_sm103a": ref, "this_repository": ours,
        "evaluation_ms": {"reference": ref_total, "this_repository": our_total},
        "speedup": ref_total / our_total if our_total > 0 else None,
    }))


if __name__ == "__main__":
    main()
