"""Tensor-core kernels of the learned warm start (csrc/warmstart.cu).

  * pcp_gemm_bf16 against the FP64 product of the same BF16 operands: every
    entry within 1e-5 of sum_k |a_ik b_jk| (+ |bias|) -- FP32 accumulation
    of the exact BF16 products -- for tile edges in M and N, N from 2 to
    256, K from 16 to 24576 (split over blocks that add into C), bias and
    ReLU; no wait ran out;
  * pcp_graph_sum_bf16 against a sum in FP64: within the BF16 rounding of
    the result (2^-8 relative);
  * the warm-start network's hand-written backward against torch autograd.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import pycudapolygon_gb300 as pg  # noqa: E402
from pycudapolygon_gb300 import warmstart as ws  # noqa: E402

pg.build()
DEV = torch.device("cuda:0")


@pytest.mark.parametrize("m,n,k,splits,relu,bias", [
    (300, 128, 256, 1, True, True),
    (24576, 128, 16, 1, False, True),
    (1000, 2, 128, 1, False, True),
    (16, 128, 24576, 8, False, False),
    (257, 256, 512, 1, True, False),
    (128, 48, 64, 3, False, True),
    (5000, 64, 200, 1, True, True),
])
def test_gemm_matches_fp64_product(m, n, k, splits, relu, bias):
    g = torch.Generator(device=DEV).manual_seed(m * 7 + n * 3 + k)
    a = torch.randn(m, k, device=DEV, generator=g).to(torch.bfloat16)
    b = torch.randn(n, k, device=DEV, generator=g).to(torch.bfloat16)
    bv = torch.randn(n, device=DEV, generator=g) if bias else None
    c = ws.gemm(a, b, bias=bv, relu=relu, splits=splits)
    torch.cuda.synchronize()
    assert ws.gemm_status()
    ref = a.double() @ b.double().T
    scale = a.double().abs() @ b.double().abs().T
    if bv is not None:
        ref = ref + bv.double()
        scale = scale + bv.double().abs()
    if relu:
        ref = ref.clamp_min(0.0)
    err = (c.double() - ref).abs()
    assert torch.all(err <= 1e-5 * scale + 1e-30), float((err / (scale + 1e-30)).max())


def test_graph_sum_matches_fp64():
    rng = np.random.default_rng(4)
    V = 3000
    deg = rng.integers(0, 7, V)
    rowptr = np.concatenate(([0], np.cumsum(deg))).astype(np.int32)
    col = rng.integers(0, V, int(rowptr[-1])).astype(np.int32)
    for F in (128, 256):
        h = torch.randn(V, F, device=DEV).to(torch.bfloat16)
        rp = torch.tensor(rowptr, device=DEV)
        cl = torch.tensor(col, device=DEV)
        out = ws.graph_sum(rp, cl, h, scale=0.25)
        hd = h.double().cpu().numpy()
        ref = np.zeros((V, F))
        for i in range(V):
            ref[i] = 0.25 * hd[col[rowptr[i]:rowptr[i + 1]]].sum(axis=0)
        got = out.double().cpu().numpy()
        assert np.all(np.abs(got - ref) <= 2.0 ** -8 * np.abs(ref) + 1e-30)


def test_network_backward_matches_autograd():
    """The network's hand-written backward (products on the tensor cores,
    the neighbour sum as its own transpose) against torch autograd of the
    same network in FP32 with the same BF16 roundings of weights and
    activations: every gradient within 2% of its norm (the backward rounds
    its intermediate gradients to BF16 as well)."""
    from pycudapolygon_gb300.systems import load_into, make_system
    lib = pg.load_module()
    s = make_system(32, 16, 0.85, seed=3)
    m = load_into(lib.Model(s.num_vertices), s)
    feats, rowptr, col, _ = ws.state_inputs(m, s)
    V = s.num_vertices
    Vp = feats.shape[0]
    net = ws.WarmStartNet(seed=1)
    for w in net.W:
        w.mul_(1.0)
    net.W[-1][:2] = torch.randn(2, ws.HIDDEN, device=DEV) * 0.1
    g = torch.Generator(device=DEV).manual_seed(0)
    t = torch.randn(Vp, 2, device=DEV, generator=g)
    t[V:] = 0
    y = net.forward(feats, rowptr, col, keep=True)
    diff = y - t
    diff[V:] = 0
    gW, gb = net.backward(2.0 * diff / V, rowptr, col)
    # the same network with torch autograd
    A = torch.zeros(Vp, Vp, device=DEV)
    rp, cl = rowptr.cpu().numpy(), col.cpu().numpy()
    for i in range(Vp):
        for j in cl[rp[i]:rp[i + 1]]:
            A[i, j] += 1.0
    Ws = [w.clone().requires_grad_(True) for w in net.W]
    bs = [b.clone().requires_grad_(True) for b in net.b]
    bf = lambda a: a.to(torch.bfloat16).float()   # noqa: E731
    h = bf(torch.relu(feats.float() @ bf(Ws[0]).T + bs[0]))
    for li in range(1, ws.LAYERS + 1):
        msg = bf(net.agg * (A @ h))
        h = bf(torch.relu(torch.cat([h, msg], 1) @ bf(Ws[li]).T + bs[li]))
    yr = (h @ bf(Ws[-1]).T + bs[-1])[:, :2]
    assert torch.allclose(yr.detach(), y, rtol=2e-2, atol=2e-2 * float(yr.detach().abs().max()))
    loss = ((yr[:V] - t[:V]) ** 2).sum() / V
    loss.backward()
    for mine, ref in zip(gW + gb, [w.grad for w in Ws] + [b.grad for b in bs]):
        n = float(ref.norm())
        assert float((mine - ref).norm()) <= 2e-2 * n + 1e-12, (float((mine - ref).norm()), n)
    assert ws.gemm_status()
