"""PyTorch edge: the total overlap energy as a torch.autograd.Function.

`OverlapEnergy.apply(positions, system)` returns the overlap energy of the
polygons of `system` at `positions` (a CUDA float64 tensor of 2V interleaved
coordinates, or [B, 2V] for B configurations of the same polygons, giving B
energies).  The forward pass runs the contact search and the energy kernel of
the C ABI (pcp_model_overlap_energy_gradient, mode 1) on the GPU; that kernel
also writes dE/dx, which the backward pass returns scaled by the incoming
gradient.  No PyTorch operation computes the energy or its gradient: torch
holds the buffers and the graph.

The energy is the reference's (kernels.cuh:1067-1424: half the sum of h over
each crossing chain, with the chain's entry point as start point) with the
crossing points taken exactly instead of from float-rounded parameters
(kernels.cuh:857-858), which would make it a staircase at the 1e-8 level.
Its gradient includes the dependence of each chain's start point; the
reference's force leaves that out and is not this gradient.  Between changes
of the crossing topology the energy is smooth and the gradient matches
central finite differences.
"""
import numpy as np
import torch

from . import load_module


class OverlapSystem:
    """The polygons (CSR offsets) of a system, held by one GPU model.

    `max_edge_length` sets the edge-midpoint cell size of the contact search
    (0.5, the reference's default, searches every pair); it must not be
    smaller than the longest edge, or crossings of edges in cells more than
    one apart are not found (kernels.cuh:709-812)."""

    def __init__(self, start_indices, max_edge_length=0.5):
        lib = load_module()
        start = np.ascontiguousarray(start_indices, dtype=np.int32)
        self.num_vertices = int(start[-1])
        self.model = lib.Model(self.num_vertices)
        self.model.setNumVertices(self.num_vertices)
        self.model.setStartIndices(start)
        self.model.setPositions(np.full(2 * self.num_vertices, 0.5))
        self.model.initializeNeighborCells()
        self.model.setMaxEdgeLength(max_edge_length)

    def evaluate(self, positions, mode=1):
        """Energies [B] and per-vertex outputs [B, 2V] for positions [B, 2V]:
        mode 1 the exact energy and its gradient, mode 0 the reference's
        energy and force."""
        x = positions.detach().to(dtype=torch.float64).contiguous()
        if x.dim() != 2 or x.shape[1] != 2 * self.num_vertices or not x.is_cuda:
            raise ValueError("positions must be a CUDA tensor [B, 2*numVertices]")
        out = torch.empty_like(x)
        energies = torch.empty(x.shape[0], dtype=torch.float64)
        self.model.setStream(torch.cuda.current_stream(x.device).cuda_stream)
        for b in range(x.shape[0]):
            self.model.setPositionsDevice(x[b].data_ptr(), x.shape[1])
            energies[b] = self.model.overlapEnergyGradient(mode, True, out[b].data_ptr())
        return energies.to(x.device), out


class OverlapEnergy(torch.autograd.Function):
    """E(x) with dE/dx from the hand-written CUDA kernel."""

    @staticmethod
    def forward(ctx, positions, system):
        single = positions.dim() == 1
        x = positions.unsqueeze(0) if single else positions
        energies, grad = system.evaluate(x, mode=1)
        ctx.save_for_backward(grad)
        ctx.single = single
        return energies[0] if single else energies

    @staticmethod
    def backward(ctx, grad_out):
        (grad,) = ctx.saved_tensors
        if ctx.single:
            return grad_out * grad[0], None
        return grad_out[:, None] * grad, None


def overlap_energy(positions, system):
    return OverlapEnergy.apply(positions, system)
