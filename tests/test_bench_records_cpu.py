"""The committed measurement records bench.py copies into its line: the
reference's own kernels against this repository's (oracle/ref_time.py's
output) and the FP64-pipe and DRAM figures of the ncu captures."""
import json
import os

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_kernels_record_is_consistent():
    r = bench.reference_kernels_record()
    assert r is not None
    ref, ours = r["stage_ms"]["reference"], r["stage_ms"]["this_repository"]
    assert set(ref) == set(ours) and "updateForceEnergy" in ref
    assert abs(sum(ref.values()) - r["evaluation_ms"]["reference"]) < 1e-9
    assert abs(sum(ours.values()) - r["evaluation_ms"]["this_repository"]) < 1e-9
    assert abs(r["speedup"] - sum(ref.values()) / sum(ours.values())) < 1e-9
    raw = json.load(open(os.path.join(ROOT, "profiles", "reference_kernels_4096x32.json")))
    # both sides evaluated the same system: same records, same energy
    a, b = raw["reference_kernels_sm103a"], raw["this_repository"]
    assert a["records"] == b["records"] == raw["oracle_records"] > 0
    assert abs(a["energy"] - b["energy"]) <= 1e-12 * abs(a["energy"])
    assert raw["all_records_paired"]


def test_profile_records_load():
    for name in ["narrow_phase_traffic.json", "fp64_pipe_4096x32.json"]:
        d = json.load(open(os.path.join(ROOT, "profiles", name)))
        assert d
