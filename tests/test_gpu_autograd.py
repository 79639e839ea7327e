"""The overlap energy as a torch.autograd.Function (pycudapolygon_gb300/autograd.py).

Workload of the checks: 1024 polygons of 24 vertices at packing fraction
0.87, a batch of 64 configurations (seeded), FP64.

  * mode 0 of the energy kernel (a plain record-by-record restatement of the
    reference's exterior and interior terms, kernels.cuh:1067-1424) gives the
    same force and energy as the FIRE path's overlap-force kernel:
    forces 1e-10 of the largest component, energy 1e-12 relative;
  * the exact-crossing energy differs from the reference's (float-rounded
    crossing parameters, kernels.cuh:857-858) by less than 1e-6 relative;
  * the backward pass equals the kernel's gradient, and the gradient matches
    central finite differences (h = 1e-6) on 256 random coordinates per
    configuration: |FD - grad| <= 1e-6 max|grad| + 1e-6 |grad|.  A
    coordinate whose +-h moves change the set of crossing records (the energy
    is not smooth there) is skipped and counted; at most 1% may be.  Beside
    a nearly parallel crossing the O(h^2) truncation error of the central
    difference alone exceeds that bound (seed 101, coordinate 38432: FD error
    5.2e-6 at h = 1e-6, 1.3e-6 at h/2, 3.2e-7 at h/4); there the difference
    at h/2 must show the h^2 decay and the Richardson extrapolation from h
    and h/2 must meet the bound; at most 1% of coordinates may need it;
  * against the reference force: at every vertex that is not one of the four
    vertices of a record's entry edges (where the chain's start point moves)
    the gradient is -1/2 of the reference force within 1e-6 of its largest
    component (the 1/2 of the energy, and the exact versus float-rounded
    crossing points); at the others they differ by the start-point term.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pycudapolygon_gb300 as pg  # noqa: E402
from pycudapolygon_gb300.autograd import OverlapSystem, overlap_energy  # noqa: E402
from pycudapolygon_gb300.systems import load_into, make_system  # noqa: E402

pg.build()
lib = pg.load_module()
DEV = torch.device("cuda:0")
P, N, PHI, BATCH = 1024, 24, 0.87, 64


@pytest.fixture(scope="module")
def batch():
    systems = [make_system(P, N, PHI, seed=100 + b) for b in range(BATCH)]
    x = torch.tensor(np.stack([s.positions for s in systems]), dtype=torch.float64, device=DEV)
    return systems, x


@pytest.fixture(scope="module")
def osys(batch):
    systems, _ = batch
    return OverlapSystem(systems[0].start_indices)


def test_reference_mode_matches_fire_path_force(batch, osys):
    systems, x = batch
    for b in (0, 1, 2):
        s = systems[b]
        m = load_into(lib.Model(s.num_vertices), s)
        m.setMaxEdgeLength(0.5)
        m.updatePolygonGeometry()
        m.updateNeighborCells()
        m.updateNeighbors()
        m.updateOutersections()
        m.updateForceEnergy()
        f_ref = np.asarray(m.getForces())
        e, out = osys.evaluate(x[b:b + 1], mode=0)
        assert float(e[0]) == pytest.approx(m.getEnergy(), rel=1e-12)
        err = np.abs(out[0].cpu().numpy() - f_ref).max() / np.abs(f_ref).max()
        assert err <= 1e-10, err


def test_backward_is_the_kernel_gradient(batch, osys):
    _, x = batch
    xb = x[:8].clone().requires_grad_(True)
    e = overlap_energy(xb, osys)
    w = torch.linspace(0.5, 1.5, 8, dtype=torch.float64, device=DEV)
    (g,) = torch.autograd.grad((w * e).sum(), xb)
    e2, grad = osys.evaluate(x[:8], mode=1)
    # a second evaluation adds the same terms in another order (FP64 atomics)
    torch.testing.assert_close(e.detach(), e2, rtol=1e-13, atol=0)
    gmax = float(torch.abs(grad).max())
    torch.testing.assert_close(g, w[:, None] * grad, rtol=0, atol=1e-13 * gmax)
    e0, _ = osys.evaluate(x[:8], mode=0)
    assert torch.all(torch.abs(e2 - e0) <= 1e-6 * torch.abs(e0))


def _records(osys):
    k = np.asarray(osys.model.getIntersections(), dtype=np.uint64)
    o = np.asarray(osys.model.getOutersections(), dtype=np.uint64)
    return k.tobytes() + o.tobytes()


def _central_difference(osys, xb, c, h):
    xp = xb.clone()
    xp[0, c] += h
    ep, _ = osys.evaluate(xp, mode=1)
    xm = xb.clone()
    xm[0, c] -= h
    em, _ = osys.evaluate(xm, mode=1)
    return float(ep[0] - em[0]) / (2 * h)


def test_gradient_matches_central_differences(batch, osys):
    _, x = batch
    h = 1e-6
    rng = np.random.default_rng(7)
    checked = skipped = extrapolated = 0
    for b in range(BATCH):
        xb = x[b:b + 1].clone()
        _, grad = osys.evaluate(xb, mode=1)
        g = grad[0].cpu().numpy()
        gmax = np.abs(g).max()
        # half the coordinates where the gradient is non-zero, half anywhere
        nz = np.nonzero(g)[0]
        coords = np.concatenate([rng.choice(nz, 128, replace=False),
                                 rng.choice(g.size, 128, replace=False)])
        for c in coords:
            xp = xb.clone()
            xp[0, c] += h
            ep, _ = osys.evaluate(xp, mode=1)
            rp = _records(osys)
            xm = xb.clone()
            xm[0, c] -= h
            em, _ = osys.evaluate(xm, mode=1)
            rm = _records(osys)
            if rp != rm:
                skipped += 1
                continue
            fd = float(ep[0] - em[0]) / (2 * h)
            tol = 1e-6 * gmax + 1e-6 * abs(g[c])
            err = abs(fd - g[c])
            if err > tol:
                # Truncation error of the central difference: next to a
                # nearly parallel crossing (cross product of the two edges
                # ~1e-6) the crossing point's third derivative is large, and
                # the O(h^2) term alone exceeds the tolerance.  Then the
                # difference at h/2 must show the h^2 decay, and the
                # Richardson extrapolation (4 fd(h/2) - fd(h)) / 3, whose
                # error is O(h^4), must match the gradient.
                fd2 = _central_difference(osys, xb, c, h / 2)
                rich = (4.0 * fd2 - fd) / 3.0
                assert abs(rich - g[c]) <= tol, (b, c, fd, fd2, rich, g[c], gmax)
                assert abs(fd2 - g[c]) < 0.5 * err, (b, c, fd, fd2, g[c])
                extrapolated += 1
            checked += 1
    assert skipped <= 0.01 * (checked + skipped), (skipped, checked)
    assert extrapolated <= 0.01 * checked, (extrapolated, checked)


def test_gradient_against_reference_force(batch, osys):
    _, x = batch
    for b in range(4):
        _, grad = osys.evaluate(x[b:b + 1], mode=1)
        _, force = osys.evaluate(x[b:b + 1], mode=0)
        g = grad[0].cpu().numpy().reshape(-1, 2)
        f = force[0].cpu().numpy().reshape(-1, 2)
        keys = np.asarray(osys.model.getIntersections(), dtype=np.uint64)
        outs = np.asarray(osys.model.getOutersections(), dtype=np.uint64)
        start = np.asarray(osys.model.getStartIndices())
        touched = np.zeros(g.shape[0], dtype=bool)
        for kk, oo in zip(keys, outs):
            if kk == oo:
                continue
            s1, s2 = int((kk >> np.uint64(32)) & np.uint64(0xFFFF)), int(kk >> np.uint64(48))
            i, j = int((kk >> np.uint64(16)) & np.uint64(0xFFFF)), int(kk & np.uint64(0xFFFF))
            for s, loc in ((s1, i), (s2, j)):
                n = start[s + 1] - start[s]
                touched[start[s] + loc] = True
                touched[start[s] + (loc + 1) % n] = True
        fmax = np.abs(f).max()
        free = ~touched
        assert free.sum() > 0 and touched.sum() > 0
        assert np.abs(g[free] + 0.5 * f[free]).max() <= 1e-6 * fmax
        # at the entry-edge vertices the start-point term is visible
        assert np.abs(g[touched] + 0.5 * f[touched]).max() > 1e-6 * fmax


def _exact_energy_restated(x, start, keys, outs):
    """The exact-crossing overlap energy written with torch operations on the
    CPU (FP64), for differentiation by torch's autograd: for every record
    with an exit partner, half the sum of h(a, b, f1) over the chain
    f1 -> p(i+1) -> ... -> p(l) -> f2 (or f1 -> f2 when i == l), with f1, f2
    the exact crossing points (kernels.cuh:1067-1424 for the chain and the
    records, kernels.cuh:161-222 for the crossing parameter)."""
    def wrap(d):
        return d - torch.floor(d + 0.5)

    def cross_point(pa, pza, pb, pzb):
        da, db, g = wrap(pza - pa), wrap(pzb - pb), wrap(pb - pa)
        t = (db[:, 0] * g[:, 1] - db[:, 1] * g[:, 0]) / (db[:, 0] * da[:, 1] - db[:, 1] * da[:, 0])
        return wrap(pa + t[:, None] * da)

    def h(a, b, s):
        r1, r2 = wrap(a - s), wrap(b - s)
        return (r1[:, 0] + r2[:, 0]) * wrap(r2[:, 1] - r1[:, 1])

    idx = {k: [] for k in ("i", "zi", "j", "zj", "k", "zk", "m", "zm", "same")}
    inner_rec, inner_a, inner_za = [], [], []
    for kk, oo in zip(keys, outs):
        if kk == oo:
            continue
        s1, s2 = int((kk >> np.uint64(32)) & np.uint64(0xFFFF)), int(kk >> np.uint64(48))
        i, j = int((kk >> np.uint64(16)) & np.uint64(0xFFFF)), int(kk & np.uint64(0xFFFF))
        k, l = int((oo >> np.uint64(16)) & np.uint64(0xFFFF)), int(oo & np.uint64(0xFFFF))
        b1, n1 = int(start[s1]), int(start[s1 + 1] - start[s1])
        b2, n2 = int(start[s2]), int(start[s2 + 1] - start[s2])
        r = len(idx["i"])
        for name, v in (("i", b1 + i), ("zi", b1 + (i + 1) % n1), ("j", b2 + j),
                        ("zj", b2 + (j + 1) % n2), ("k", b2 + k), ("zk", b2 + (k + 1) % n2),
                        ("m", b1 + l), ("zm", b1 + (l + 1) % n1), ("same", i == l)):
            idx[name].append(v)
        a = (i + 1) % n1
        while i != l and a != l:
            inner_rec.append(r)
            inner_a.append(b1 + a)
            inner_za.append(b1 + (a + 1) % n1)
            a = (a + 1) % n1
    p = x.view(-1, 2)
    t = {k: torch.tensor(v) for k, v in idx.items()}
    f1 = cross_point(p[t["i"]], p[t["zi"]], p[t["j"]], p[t["zj"]])
    f2 = cross_point(p[t["k"]], p[t["zk"]], p[t["m"]], p[t["zm"]])
    same = t["same"]
    e = torch.where(same, h(f1, f2, f1), h(f1, p[t["zi"]], f1) + h(p[t["m"]], f2, f1)).sum()
    if inner_rec:
        ir = torch.tensor(inner_rec)
        e = e + h(p[torch.tensor(inner_a)], p[torch.tensor(inner_za)], f1[ir]).sum()
    return 0.5 * e


def test_gradient_matches_autodiff_of_restated_energy(batch, osys):
    """The kernel's energy and gradient (mode 1) against torch's autograd of
    the restated energy, on the oracle's contact records: energy 1e-12
    relative, gradient 1e-10 of its largest component (FP64 atomics add the
    terms in another order)."""
    from oracle import oracle as orc

    systems, x = batch
    for b in (0, 1):
        s = systems[b]
        o = load_into(orc.OracleModel(s.num_vertices), s)
        o.updatePolygonGeometry()
        o.updateNeighborCells()
        o.updateNeighbors()
        o.updateOutersections()
        keys, outs = o.getIntersections(), o.getOutersections()
        e, grad = osys.evaluate(x[b:b + 1], mode=1)
        # the same records (the model lists them in its slot order here)
        gk = np.asarray(osys.model.getIntersections(), dtype=np.uint64)
        go = np.asarray(osys.model.getOutersections(), dtype=np.uint64)
        ok, oo = np.asarray(keys, dtype=np.uint64), np.asarray(outs, dtype=np.uint64)
        ig, io = np.lexsort((go, gk)), np.lexsort((oo, ok))
        assert np.array_equal(gk[ig], ok[io]) and np.array_equal(go[ig], oo[io])
        xc = torch.tensor(s.positions, dtype=torch.float64, requires_grad=True)
        er = _exact_energy_restated(xc, s.start_indices, keys, outs)
        (gr,) = torch.autograd.grad(er, xc)
        assert float(e[0]) == pytest.approx(float(er.detach()), rel=1e-12)
        g = grad[0].cpu()
        assert float(torch.abs(g - gr).max()) <= 1e-10 * float(torch.abs(gr).max())
