"""Learned FIRE warm start: a message-passing network over the contact graph.

The reference has no counterpart.  A system compressed to a higher packing
fraction is minimised by plain FIRE from a starting point the network
proposes (per-vertex displacements), instead of from the compressed state
itself.  FIRE with the reference's rules still runs to the same stop, so
the network can only move the starting point; the result is always FIRE's.

Graph: one node per polygon vertex; edges join each vertex to its two ring
neighbours and the end vertices of every pair of crossing edges (the contact
records of the contact search), in both directions.  Node features
(pycudapolygon_gb300.warmstart.node_features): the vertex relative to its
polygon's centroid, its two edge vectors, the reference's projected force,
the area gradient, the polygon's area deficit and the number of crossings
on its edges, scaled to order one and padded to 16 columns.

Network (hidden width 128, three message-passing layers):
    h0 = relu(x W0^T + b0)
    h_l = relu([h_{l-1}, s * sum_{j ~ i} h_{l-1, j}] W_l^T + b_l),  l = 1..3
    d  = h3 Wout^T + bout  (first two columns: the displacement / scale)
Every product runs in the hand-written tensor-core GEMM of this library
(pcp_gemm_bf16: BF16 operands, FP32 accumulation) and every neighbour sum in
pcp_graph_sum_bf16, forward and backward; PyTorch holds the buffers and runs
the elementwise glue (ReLU masks, bias sums, the Adam update).
"""
import ctypes
import time

import numpy as np
import torch

from . import cabi

HIDDEN = 128
FEATURES = 16
LAYERS = 3


def _lib():
    return cabi.lib()


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check(rc):
    if rc != 0:
        raise RuntimeError("pcp status %d: %s" % (rc, _lib().pcp_last_error().decode()))


def gemm(a, b, bias=None, relu=False, splits=1, out=None):
    """a [m, k] and b [n, k] (BF16, contiguous, k a multiple of 8) ->
    a b^T [m, n] FP32 (+ bias, ReLU) on the tensor cores."""
    if a.dtype != torch.bfloat16 or b.dtype != torch.bfloat16:
        raise TypeError("gemm takes BF16 operands")
    a, b = a.contiguous(), b.contiguous()
    m, k = a.shape
    n, k2 = b.shape
    if k != k2:
        raise ValueError("inner sizes differ")
    if out is None:
        out = (torch.zeros if splits > 1 else torch.empty)(m, n, dtype=torch.float32,
                                                           device=a.device)
    bp = ctypes.c_void_p(bias.data_ptr()) if bias is not None else None
    _check(_lib().pcp_gemm_bf16(ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                                ctypes.c_void_p(out.data_ptr()), m, n, k, bp, int(relu),
                                int(splits), _stream()))
    return out


def gemm_status():
    """True when no wait inside a GEMM ran out since the last call."""
    v = ctypes.c_int(0)
    _check(_lib().pcp_gemm_status(ctypes.byref(v)))
    return v.value == 0


def graph_sum(rowptr, col, h, scale=1.0):
    """scale * sum of the neighbours' rows of h (BF16 [v, f]) -> BF16 [v, f]."""
    h = h.contiguous()
    out = torch.empty_like(h)
    v, f = h.shape
    _check(_lib().pcp_graph_sum_bf16(ctypes.c_void_p(rowptr.data_ptr()),
                                     ctypes.c_void_p(col.data_ptr()),
                                     ctypes.c_void_p(h.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                     v, f, ctypes.c_float(scale), _stream()))
    return out


# ---------------------------------------------------------------- graph ----
def _pad_rows(v, mult=128):
    return (v + mult - 1) // mult * mult


def contact_graph(start, keys, num_vertices):
    """CSR (rowptr, col) over the vertices, padded to a multiple of 128 rows:
    ring neighbours, and for every crossing record (sj, si, i, j) the start
    vertices of the two crossing edges and their end vertices, joined both
    ways (so the neighbour sum is its own transpose)."""
    start = np.asarray(start, dtype=np.int64)
    V = int(num_vertices)
    n = np.diff(start)
    poly = np.repeat(np.arange(len(n)), n)
    loc = np.arange(V) - start[poly]
    nxt = start[poly] + (loc + 1) % n[poly]
    prv = start[poly] + (loc - 1) % n[poly]
    src = [np.arange(V), np.arange(V)]
    dst = [nxt, prv]
    k = np.asarray(keys, dtype=np.uint64)
    if k.size:
        sj = (k >> np.uint64(48)).astype(np.int64)
        si = ((k >> np.uint64(32)) & np.uint64(0xFFFF)).astype(np.int64)
        i = ((k >> np.uint64(16)) & np.uint64(0xFFFF)).astype(np.int64)
        j = (k & np.uint64(0xFFFF)).astype(np.int64)
        a0, b0 = start[si] + i, start[sj] + j
        a1 = start[si] + (i + 1) % n[si]
        b1 = start[sj] + (j + 1) % n[sj]
        src += [a0, b0, a1, b1]
        dst += [b0, a0, b1, a1]
    src, dst = np.concatenate(src), np.concatenate(dst)
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    Vp = _pad_rows(V)
    rowptr = np.zeros(Vp + 1, dtype=np.int32)
    np.add.at(rowptr, src + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return rowptr, dst.astype(np.int32)


def node_features(x, start, forces, areas, target_areas, keys, num_vertices):
    """Node features [Vp, 16] (BF16 on the GPU) of a state, and the length
    scale s that makes them order one (the square root of the mean polygon
    area)."""
    start = np.asarray(start, dtype=np.int64)
    V = int(num_vertices)
    n = np.diff(start)
    P = len(n)
    poly = np.repeat(np.arange(P), n)
    loc = np.arange(V) - start[poly]
    xy = np.asarray(x, dtype=np.float64).reshape(-1, 2)
    wrap = lambda d: d - np.floor(d + 0.5)   # noqa: E731
    first = xy[start[:-1]]
    rel0 = wrap(xy - first[poly])
    cen = np.zeros((P, 2))
    np.add.at(cen, poly, rel0)
    cen /= n[:, None]
    rel = rel0 - cen[poly]
    nxt = start[poly] + (loc + 1) % n[poly]
    prv = start[poly] + (loc - 1) % n[poly]
    e_next = wrap(xy[nxt] - xy)
    e_prev = wrap(xy - xy[prv])
    s = float(np.sqrt(np.mean(np.asarray(target_areas))))
    f = np.asarray(forces, dtype=np.float64).reshape(-1, 2)
    fs = f / (np.abs(f).max() + 1e-30)
    ag = 0.5 * np.stack([wrap(xy[nxt, 1] - xy[prv, 1]), wrap(xy[prv, 0] - xy[nxt, 0])], axis=1)
    deficit = (np.asarray(areas) / np.asarray(target_areas) - 1.0)[poly]
    cross = np.zeros(V)
    k = np.asarray(keys, dtype=np.uint64)
    if k.size:
        sj = (k >> np.uint64(48)).astype(np.int64)
        si = ((k >> np.uint64(32)) & np.uint64(0xFFFF)).astype(np.int64)
        i = ((k >> np.uint64(16)) & np.uint64(0xFFFF)).astype(np.int64)
        j = (k & np.uint64(0xFFFF)).astype(np.int64)
        for v in (start[si] + i, start[sj] + j, start[si] + (i + 1) % n[si],
                  start[sj] + (j + 1) % n[sj]):
            np.add.at(cross, v, 1.0)
    feats = np.zeros((_pad_rows(V), FEATURES), dtype=np.float32)
    feats[:V, 0:2] = rel / s
    feats[:V, 2:4] = e_next / s
    feats[:V, 4:6] = e_prev / s
    feats[:V, 6:8] = fs
    feats[:V, 8:10] = ag / s
    feats[:V, 10] = 10.0 * deficit
    feats[:V, 11] = 0.25 * cross
    feats[:V, 12] = 1.0
    return feats, s


# -------------------------------------------------------------- network ----
class WarmStartNet:
    """The network's FP32 master weights and an Adam state; forward and
    backward run through gemm() and graph_sum()."""

    def __init__(self, seed=0, device="cuda", agg_scale=0.25):
        g = torch.Generator(device="cpu").manual_seed(seed)

        def init(n, k, gain=2.0):
            return (torch.randn(n, k, generator=g) * np.sqrt(gain / k)).to(device)
        self.agg = agg_scale
        self.W = [init(HIDDEN, FEATURES)] + [init(HIDDEN, 2 * HIDDEN) for _ in range(LAYERS)]
        wout = torch.zeros(FEATURES, HIDDEN)
        wout[:2] = torch.randn(2, HIDDEN, generator=g) * 1e-2
        self.W.append(wout.to(device))
        self.b = [torch.zeros(HIDDEN, device=device) for _ in range(LAYERS + 1)] + \
                 [torch.zeros(FEATURES, device=device)]
        self.m = [torch.zeros_like(p) for p in self.W + self.b]
        self.v = [torch.zeros_like(p) for p in self.W + self.b]
        self.t = 0

    def forward(self, x, rowptr, col, keep=False):
        """x: BF16 [Vp, 16] -> FP32 [Vp, 2] (displacement / scale)."""
        acts = []
        z = gemm(x, self.W[0].to(torch.bfloat16), self.b[0], relu=True)
        h = z.to(torch.bfloat16)
        acts.append((x, z))
        for li in range(1, LAYERS + 1):
            msg = graph_sum(rowptr, col, h, self.agg)
            hc = torch.cat([h, msg], dim=1)
            z = gemm(hc, self.W[li].to(torch.bfloat16), self.b[li], relu=True)
            acts.append((hc, z))
            h = z.to(torch.bfloat16)
        y = gemm(h, self.W[-1].to(torch.bfloat16), self.b[-1])
        if keep:
            self._acts, self._h = acts, h
        return y[:, :2]

    def backward(self, dy, rowptr, col):
        """dL/dy [Vp, 2] FP32 -> gradients of every weight and bias."""
        Vp = dy.shape[0]
        splits = max(1, min(64, Vp // 512))
        dy16 = torch.zeros(Vp, FEATURES, device=dy.device, dtype=torch.bfloat16)
        dy16[:, :2] = dy.to(torch.bfloat16)
        gW = [None] * len(self.W)
        gb = [None] * len(self.b)
        gW[-1] = gemm(dy16.T.contiguous(), self._h.T.contiguous(), splits=splits)
        gb[-1] = torch.zeros(FEATURES, device=dy.device)
        gb[-1][:2] = dy.sum(0)
        dh = gemm(dy16, self.W[-1].to(torch.bfloat16).T.contiguous())
        for li in range(LAYERS, -1, -1):
            inp, z = self._acts[li]
            dz = dh * (z > 0)
            dzb = dz.to(torch.bfloat16)
            gW[li] = gemm(dzb.T.contiguous(), inp.T.contiguous(), splits=splits)
            gb[li] = dz.sum(0)
            if li == 0:
                break
            dhc = gemm(dzb, self.W[li].to(torch.bfloat16).T.contiguous())
            back = graph_sum(rowptr, col, dhc[:, HIDDEN:].to(torch.bfloat16).contiguous(),
                             self.agg)
            dh = dhc[:, :HIDDEN] + back.float()
        return gW, gb

    def adam(self, gW, gb, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.t += 1
        for p, g, m, v in zip(self.W + self.b, gW + gb, self.m, self.v):
            m.mul_(b1).add_(g, alpha=1 - b1)
            v.mul_(b2).addcmul_(g, g, value=1 - b2)
            mh = m / (1 - b1 ** self.t)
            vh = v / (1 - b2 ** self.t)
            p.add_(-lr * mh / (vh.sqrt() + eps))
        self.W[-1][2:].zero_()
        self.b[-1][2:].zero_()


# ------------------------------------------------------- data and runs ----
def _wrap(d):
    return d - np.floor(d + 0.5)


def _longest_edge(x, start):
    xy = np.asarray(x).reshape(-1, 2)
    start = np.asarray(start)
    n = np.diff(start)
    poly = np.repeat(np.arange(len(n)), n)
    nxt = start[poly] + (np.arange(xy.shape[0]) - start[poly] + 1) % n[poly]
    e = _wrap(xy[nxt] - xy)
    return float(np.sqrt((e * e).sum(axis=1)).max())


def compressed_state(lib, system, phi):
    """The system compressed to packing fraction phi as the reference's
    setPhi does it (pyCudaPolygon.py:223-234: targets scaled, every polygon
    rescaled about its centre of mass by resetAreas), then put on the
    constraint manifold by SHAKE.  Returns (positions, target areas, target
    edge lengths)."""
    from .systems import load_into
    m = load_into(lib.Model(system.num_vertices), system)
    m.shakeProject(100, 1e-15)
    ta = np.asarray(m.getTargetAreas(), dtype=np.float64)
    ratio = phi / ta.sum()
    m.setTargetAreas(ta * ratio)
    m.setTargetEdgeLengths(np.asarray(m.getTargetEdgeLengths()) * np.sqrt(ratio))
    m.updatePolygonGeometry()
    m.resetAreas()
    m.updatePolygonGeometry()
    m.shakeProject(100, 1e-15)
    return (np.asarray(m.getPositions()).copy(), np.asarray(m.getTargetAreas()).copy(),
            np.asarray(m.getTargetEdgeLengths()).copy())


def model_at(lib, system, x, ta, tl):
    m = lib.Model(system.num_vertices)
    m.setNumVertices(system.num_vertices)
    m.setStartIndices(system.start_indices)
    m.setPositions(x)
    m.setTargetAreas(ta)
    m.setTargetEdgeLengths(tl)
    m.initializeNeighborCells()
    m.setMaxEdgeLength(max(_longest_edge(x, system.start_indices), 1e-3))
    return m


def state_inputs(m, system, device="cuda"):
    """Features and graph of the model's current state (one contact search,
    the reference's force and its projection)."""
    m.updatePolygonGeometry()
    m.updateNeighborCells()
    m.updateNeighbors()
    m.updateOutersections()
    m.updateForceEnergy()
    m.projectForce()
    keys = np.asarray(m.getIntersections(), dtype=np.uint64)
    feats, s = node_features(m.getPositions(), system.start_indices, m.getForces(),
                             m.getAreas(), m.getTargetAreas(), keys, system.num_vertices)
    rowptr, col = contact_graph(system.start_indices, keys, system.num_vertices)
    return (torch.tensor(feats, device=device).to(torch.bfloat16),
            torch.tensor(rowptr, device=device), torch.tensor(col, device=device), s)


FIRE_DEFAULTS = (0.1, 0.1, 0.99, 1.1, 0.5, 5, 5)


def minimise(m, max_steps):
    """The reference Python driver's minimizeFIRE (device loop): returns
    (seconds, energy, steps, |F|max)."""
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = m.minimizeFIREDevice(1e-10, 1e-3, max_steps, *FIRE_DEFAULTS)
    torch.cuda.synchronize()
    return time.perf_counter() - t0, float(r[0]), int(r[2]), float(m.getMaxUnbalancedForce())


def make_sample(lib, seed, P, n, phi0, phi1, max_steps):
    """A (compressed, FIRE-minimised) pair generated by the plain method."""
    from .systems import make_system
    system = make_system(P, n, phi0, seed=seed)
    x, ta, tl = compressed_state(lib, system, phi1)
    m = model_at(lib, system, x, ta, tl)
    feats, rowptr, col, s = state_inputs(m, system)
    m = model_at(lib, system, x, ta, tl)
    secs, e, steps, fmax = minimise(m, max_steps)
    return dict(system=system, x=x, ta=ta, tl=tl, feats=feats, rowptr=rowptr, col=col, s=s,
                target=_wrap(np.asarray(m.getPositions()) - x), cold=(secs, e, steps, fmax))


def train(net, samples, epochs, dscale, lr=1e-3, physics=0.0, seed=0, mse=1.0):
    """Adam on mse times the mean squared error of the displacement (in
    units of dscale) over every vertex; with physics > 0, plus physics *
    E(x + d) / E(x) from the overlap energy's autograd Function (its
    backward is the exact-gradient kernel).  Returns the loss per epoch."""
    from .autograd import OverlapSystem, overlap_energy
    rng = np.random.default_rng(seed)
    osys = {}
    history = []
    for _ in range(epochs):
        tot = 0.0
        for k in rng.permutation(len(samples)):
            smp = samples[k]
            V = smp["system"].num_vertices
            Vp = smp["feats"].shape[0]
            t = torch.zeros(Vp, 2, device="cuda")
            t[:V] = torch.tensor(smp["target"].reshape(-1, 2) / dscale, device="cuda",
                                 dtype=torch.float32)
            y = net.forward(smp["feats"], smp["rowptr"], smp["col"], keep=True)
            diff = (y - t)
            diff[V:] = 0.0
            loss = mse * float((diff[:V] ** 2).sum()) / V
            dy = (2.0 * mse / V) * diff
            if physics > 0.0:
                key = id(smp["system"])
                if key not in osys:
                    osys[key] = OverlapSystem(smp["system"].start_indices)
                x0 = torch.tensor(smp["x"], device="cuda", dtype=torch.float64)
                d = (y[:V].detach().double() * dscale).reshape(-1)
                xn = (x0 + d).remainder(1.0).requires_grad_(True)
                e0 = float(osys[key].evaluate(x0[None], mode=1)[0][0]) + 1e-30
                e = overlap_energy(xn, osys[key])
                e.backward()
                dy[:V] += (physics / e0 * dscale) * xn.grad.reshape(-1, 2).float()
                loss += physics * float(e.detach()) / e0
            gW, gb = net.backward(dy, smp["rowptr"], smp["col"])
            net.adam(gW, gb, lr=lr)
            tot += loss
        history.append(tot / len(samples))
    return history


def warm_minimise(lib, net, smp, dscale, max_steps):
    """Warm start: features of the compressed state, the network's
    displacement, SHAKE onto the constraints, then the same FIRE run as the
    cold start.  The time includes everything after the compressed state."""
    system = smp["system"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m = model_at(lib, system, smp["x"], smp["ta"], smp["tl"])
    feats, rowptr, col, _ = state_inputs(m, system)
    y = net.forward(feats, rowptr, col)[:system.num_vertices]
    x1 = np.mod(smp["x"] + (y.double().cpu().numpy() * dscale).reshape(-1), 1.0)
    m.setPositions(x1)
    m.shakeProject(100, 1e-15)
    torch.cuda.synchronize()
    t_pre = time.perf_counter() - t0
    secs, e, steps, fmax = minimise(m, max_steps)
    return t_pre + secs, e, steps, fmax, t_pre


def experiment(n_train=32, n_test=8, P=1024, n=24, phi0=0.84, phi1=0.86, epochs=8,
               max_steps=100000, seed=9000, physics=0.1, mse=1.0, lr=1e-3):
    """Generate pairs with the plain method, train, and compare warm-started
    with cold FIRE on held-out seeds.  Returns a JSON-ready dict."""
    from . import load_module
    lib = load_module()
    t0 = time.perf_counter()
    train_s = [make_sample(lib, seed + i, P, n, phi0, phi1, max_steps) for i in range(n_train)]
    test_s = [make_sample(lib, seed + 100000 + i, P, n, phi0, phi1, max_steps)
              for i in range(n_test)]
    t_data = time.perf_counter() - t0
    dscale = float(np.sqrt(np.mean([np.mean(s["target"] ** 2) for s in train_s])))
    net = WarmStartNet(seed=seed)
    t0 = time.perf_counter()
    hist = train(net, train_s, epochs, dscale, lr=lr, physics=physics, seed=seed, mse=mse)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    ok = gemm_status()
    cold, warm = [], []
    for smp in test_s:
        cold.append(smp["cold"])
        warm.append(warm_minimise(lib, net, smp, dscale, max_steps))
    ct = np.array([c[0] for c in cold])
    wt = np.array([w[0] for w in warm])
    ce = np.array([c[1] for c in cold])
    we = np.array([w[1] for w in warm])
    return {
        "workload": "%d polygons x %d vertices compressed from phi %.2f to %.2f; %d training "
                    "pairs (compressed -> FIRE-minimised by the plain method), %d held-out "
                    "seeds" % (P, n, phi0, phi1, n_train, n_test),
        "network": "3 message-passing layers, hidden 128, BF16 operands with FP32 "
                   "accumulation (tcgen05 GEMM), neighbour sums over ring and contact edges",
        "loss": "%.2g x displacement MSE + %.2g x overlap energy (autograd Function)" % (
            mse, physics),
        "train_loss_per_epoch": [float(h) for h in hist],
        "gemm_waits_ok": bool(ok),
        "data_generation_s": t_data, "training_s": t_train,
        "cold_s_per_system": float(ct.mean()), "warm_s_per_system": float(wt.mean()),
        "warm_over_cold_time": float(wt.mean() / ct.mean()),
        "warm_inference_s_per_system": float(np.mean([w[4] for w in warm])),
        "cold_steps": [c[2] for c in cold], "warm_steps": [w[2] for w in warm],
        "cold_energy": [float(e) for e in ce], "warm_energy": [float(e) for e in we],
        "cold_max_force": [c[3] for c in cold], "warm_max_force": [w[3] for w in warm],
        "stop_rule": "reference Python driver: |F|max <= 1e-10 or six steps with |dE| < 1e-15",
    }


if __name__ == "__main__":
    import json
    import sys
    args = [int(a) for a in sys.argv[1:3]] if len(sys.argv) > 2 else [32, 8]
    print(json.dumps(experiment(n_train=args[0], n_test=args[1])))
