"""Learned FIRE warm start: a message-passing network over the contact graph.

The reference has no counterpart: this is the benchmark spec's learned warm
start.  A system compressed to a higher packing fraction is minimised by
plain FIRE from a starting point the network proposes (per-vertex
displacements), instead of from the compressed state itself.  FIRE with the
reference's rules still runs to the same stop, so the network can only move
the starting point; the result is always FIRE's.

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
