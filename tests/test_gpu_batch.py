"""Many independent systems minimised together (pcp_batch_*, libpyCudaPolygon.Batch).

Systems of uneven size (polygon counts 64..256, 12..48 vertices per polygon,
packing fraction 0.80..0.92, seeded) run on a pool of streams with several
FIRE steps per graph launch.  The checks:

  * ten steps of Model::minimizeFIRE (model.cpp:488-504) per system in the
    batch match the same ten steps run by the CPU oracle on that system alone:
    energy after the last step 1e-9 relative (the per-step bound of the FIRE
    tests), dt exact, positions 1e-9;
  * the same ten steps with other launch shapes (grids of the narrow phase
    and the force pass) give the same energy and positions within 1e-12 /
    1e-12 (the grids only change the order of the FP64 sums);
  * a full run with the reference Python driver's rule stops every system
    (stagnation or |F|max <= threshold) before the step limit, with a
    finite energy, and reports the same stop as the system's control block;
  * the autotuner returns one of its candidate grids per system and a
    timing table with a row per size class.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pycudapolygon_gb300 as pg  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from pycudapolygon_gb300.systems import batched_specs, load_into, make_system  # noqa: E402

pg.build()
lib = pg.load_module()
FIRE = dict(dtMax=0.1, alphaStart=0.1, fAlpha=0.99, fInc=1.1, fDec=0.5, nMin=5, shakeIter=5)


def _systems(n=16, seed=5):
    specs = batched_specs(n, seed, p_range=(64, 256))
    return [make_system(P, nv, phi, seed=sd) for P, nv, phi, sd in specs]


def _models(systems):
    ms = []
    for s in systems:
        m = load_into(lib.Model(s.num_vertices), s)
        m.shakeProject(100, 1e-15)
        ms.append(m)
    return ms


def _wrapdiff(a, b):
    return (np.asarray(a) - np.asarray(b) + 0.5) % 1.0 - 0.5


def test_ten_steps_per_system_match_oracle_and_other_launch_shapes():
    systems = _systems()
    models = _models(systems)
    batch = lib.Batch()
    for m in models:
        batch.add(m)
    batch.setStreams(4, 4)
    out = batch.minimizeFIRE(0, -1.0, 1e-3, 10, **FIRE)
    assert np.all(out[:, 2] == 10) and np.all(out[:, 3] == 0)
    for k, s in enumerate(systems):
        o = load_into(orc.OracleModel(s.num_vertices), s)
        o.shakeProject(100, 1e-15)
        ro = o.minimizeFIRE(-1.0, 1e-3, 10)   # returns getEnergy() after the last step
        assert models[k].getEnergy() == pytest.approx(ro[0], rel=1e-9), k
        assert out[k, 1] == ro[1], k
        assert np.abs(_wrapdiff(models[k].getPositions(), o.getPositions())).max() < 1e-9, k
    # the same run with other grids (a fresh batch of fresh models)
    models2 = _models(systems)
    batch2 = lib.Batch()
    for m in models2:
        m.setLaunchShape(7, 3)
        batch2.add(m)
    batch2.setStreams(3, 5)
    out2 = batch2.minimizeFIRE(0, -1.0, 1e-3, 10, **FIRE)
    np.testing.assert_allclose(out2[:, 0], out[:, 0], rtol=1e-12)
    np.testing.assert_array_equal(out2[:, 1], out[:, 1])
    for a, b in zip(models, models2):
        assert np.abs(_wrapdiff(a.getPositions(), b.getPositions())).max() < 1e-12


def test_full_run_stops_every_system():
    systems = _systems(12, seed=9)
    models = _models(systems)
    batch = lib.Batch()
    for m in models:
        batch.add(m)
    out = batch.minimizeFIRE(1, 1e-10, 1e-3, 20000, **FIRE)
    assert np.all(np.isfinite(out[:, 0]))
    assert np.all(out[:, 2] < 20000)
    assert np.all(out[:, 3] > 0)                    # |F|max or the stagnation rule
    for k, m in enumerate(models):
        stag = m.fireRunStats()[0]
        assert (out[k, 3] == 2) == (stag == 1)
        if out[k, 3] == 1:
            assert m.getMaxUnbalancedForce() <= 1e-10


def test_autotune_picks_candidate_grids():
    systems = _systems(8, seed=3)
    models = _models(systems)
    batch = lib.Batch()
    for m in models:
        batch.add(m)
    shapes = batch.autotune(4)
    rep = json.loads(batch.report())
    cand = set(rep["candidates_blocks"])
    assert shapes.shape == (8, 2)
    assert all(int(a) in cand and int(a) == int(b) for a, b in shapes)
    assert len(rep["classes"]) >= 1 and all(len(c["ms"]) == 5 for c in rep["classes"])
    for m, (a, b) in zip(models, shapes):
        assert m.getLaunchShape() == (int(a), int(b))
    out = batch.minimizeFIRE(1, 1e-10, 1e-3, 20000, **FIRE)
    assert np.all(out[:, 3] > 0)
