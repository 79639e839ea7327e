// geometry.cu -- per-polygon geometry, topology, edge-midpoint cells and the
// element-wise / reduction kernels of the hot path (sm_103a).
//
// Restates, with GB300-first launch shapes (one warp per polygon, reductions
// in registers and shuffles instead of CUB segmented reductions and FP64
// atomics), the reference kernels named beside each function
// (camdennis/pyCudaPolygon src/kernels.cuh, src/model.cu).
#include <cuda_runtime.h>
#include <math.h>

#include "pcp_common.cuh"
#include "pcp_internal.h"

namespace pcp {

static int g_sm_count = 0;
int sm_count() {
    if (g_sm_count == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess
            || g_sm_count <= 0)
            g_sm_count = 152;
    }
    return g_sm_count;
}

static inline int blocks_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 2147483647LL) b = 2147483647LL;
    return (int)b;
}

// ------------------------------------------------------------- topology ----
// updateShapeIdKernel (kernels.cuh:652-659) + computeNextPrevKernel (:127-135)
__global__ void k_topology(const int* __restrict__ start, int P, int V, int* __restrict__ shapeId,
                           int* __restrict__ next, int* __restrict__ prev) {
    pdl_enter();
    int p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (p >= P) return;
    int st = start[p], en = start[p + 1];
    for (int i = st + lane; i < en; i += 32) {
        if (i < 0 || i >= V) continue;
        shapeId[i] = p;
        next[i] = (i + 1 == en) ? st : i + 1;
        prev[i] = (i == st) ? en - 1 : i - 1;
    }
}

cudaError_t launch_topology(const int* start, int P, int V, int* shapeId, int* next, int* prev,
                            cudaStream_t st) {
    if (P <= 0) return cudaSuccess;
    launch_k(k_topology, dim3(blocks_for(P, 8)), dim3(256), 0, st, start, P, V, shapeId, next, prev);
    return cudaGetLastError();
}

__global__ void k_zero_scalar(double* x, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    *x = 0.0;
}

// ------------------------------------------------------------- geometry ----
// k_geometry's form for polygons of at most 32 vertices: one vertex per lane, the
// neighbours' positions, the previous edge and its length taken from the
// neighbouring lane instead of recomputed, one reciprocal square root per
// edge (tangent and length), the seven sums reduced four and three at a time
// (warp_sum4), and the normalised constraints written once.  About half the
// FP64 instructions of the general form; the values agree with it to a few ulps
// (the reference's divisions by lengths and norms become multiplications by
// reciprocal square roots, and wrap(x_k - x_k+1) is taken as -wrap(x_k+1 - x_k)).
__device__ __forceinline__ void geometry_lanes(const double2* __restrict__ pos, int p, int st, int n,
                                               double* __restrict__ edgeLengths,
                                               double* __restrict__ areas,
                                               double* __restrict__ comX, double* __restrict__ comY,
                                               double* __restrict__ perimeters,
                                               double* __restrict__ constraints,
                                               double* __restrict__ maxEdge) {
    const int lane = threadIdx.x & 31;
    const bool live = lane < n;
    const int kn = (lane + 1 >= n) ? 0 : lane + 1;
    const int kp = (lane == 0) ? n - 1 : lane - 1;
    const double2 x = live ? pos[st + lane] : make_double2(0.0, 0.0);
    const double2 xn = make_double2(__shfl_sync(PCP_FULL, x.x, kn), __shfl_sync(PCP_FULL, x.y, kn));
    const double2 xp = make_double2(__shfl_sync(PCP_FULL, x.x, kp), __shfl_sync(PCP_FULL, x.y, kp));
    const double p0x = __shfl_sync(PCP_FULL, x.x, 0), p0y = __shfl_sync(PCP_FULL, x.y, 0);
    // edge k -> k+1
    const double dx = wrap(xn.x - x.x), dy = wrap(xn.y - x.y);
    const double len2 = dx * dx + dy * dy;
    // 1 / |e| (inf for a zero-length edge, whose unit tangent is then NaN
    // as the reference's 0/0 is) and |e| (0 for it)
    const double il = rsqrt(len2);
    const double el = __double_as_longlong(len2) != 0 ? len2 * il : 0.0;
    // edge k-1 -> k from the previous lane
    const double dpx = __shfl_sync(PCP_FULL, dx, kp), dpy = __shfl_sync(PCP_FULL, dy, kp);
    const double ilp = __shfl_sync(PCP_FULL, il, kp);
    // constraint gradients (updatePolygonGeometryKernel, kernels.cuh:303-318):
    // area (x_k-1 - x_k+1 rotated), edge (x_k - x_k+1) + (x_k - x_k-1), unit-edge sum
    const double a0 = -wrap(xp.y - xn.y), a1 = wrap(xp.x - xn.x);
    const double e20 = -dx + dpx, e21 = -dy + dpy;
    const double u0 = -dx * il + dpx * ilp, u1 = -dy * il + dpy * ilp;
    const double x1x = wrap(x.x - p0x), x1y = wrap(x.y - p0y);
    const double x2 = __shfl_sync(PCP_FULL, x1x, kn);
    double sA = 0.0, sX = 0.0, sY = 0.0, sPer = 0.0, n0 = 0.0, n1 = 0.0, n2 = 0.0;
    if (live) {
        sA = dy * (x2 + x1x);          // halved after the sum (exact)
        sX = x1x; sY = x1y; sPer = el;
        n0 = a0 * a0 + a1 * a1;
        n1 = e20 * e20 + e21 * e21;
        n2 = u0 * u0 + u1 * u1;
    }
    const Sum4 s4 = warp_sum4(sA, sX, sY, sPer);
    const Sum4 t4 = warp_sum4(n0, n1, n2, 0.0);
    unsigned long long em = live ? (unsigned long long)__double_as_longlong(el) : 0ull;
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long t = __shfl_xor_sync(PCP_FULL, em, o);
        em = t > em ? t : em;
    }
    const double r0 = t4.x > 0.0 ? rsqrt(t4.x) : 1.0;
    const double r1 = t4.y > 0.0 ? rsqrt(t4.y) : 1.0;
    const double r2 = t4.z > 0.0 ? rsqrt(t4.z) : 1.0;
    if (live) {
        edgeLengths[st + lane] = el;
        double* c = constraints + 6 * (size_t)(st + lane);
        c[0] = a0 * r0; c[1] = a1 * r0; c[2] = e20 * r1; c[3] = e21 * r1; c[4] = u0 * r2; c[5] = u1 * r2;
    }
    if (lane == 0) {
        areas[p] = s4.x * 0.5;
        perimeters[p] = s4.w;
        double cx = s4.y / (double)n + p0x;
        cx -= floor(cx);
        double cy = s4.z / (double)n + p0y;
        cy -= floor(cy);
        comX[p] = cx;
        comY[p] = cy;
        atomic_max_nonneg(maxEdge, __longlong_as_double((long long)em));
    }
}


// updatePolygonGeometryKernel (kernels.cuh:295-333), the segmented sums and
// max of updatePolygonGeometryCUDA (model.cu:113-152), normalizeKernel
// (kernels.cuh:635-650) and normalizeConstraintsKernel (kernels.cuh:335-345)
// fused into one warp per polygon.
__global__ void __launch_bounds__(256)
k_geometry(const double2* __restrict__ pos, const int* __restrict__ start, int P,
           double* __restrict__ edgeLengths, double* __restrict__ areas,
           double* __restrict__ comX, double* __restrict__ comY, double* __restrict__ perimeters,
           double* __restrict__ constraints, double* __restrict__ maxEdge, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    int lane = threadIdx.x & 31;
    if (p >= P) return;
    int st = start[p], en = start[p + 1];
    int n = en - st;
    if (n <= 0) return;
    if (n <= 32) {
        geometry_lanes(pos, p, st, n, edgeLengths, areas, comX, comY, perimeters, constraints,
                       maxEdge);
        return;
    }
    double2 p0 = pos[st];
    double sA = 0.0, sX = 0.0, sY = 0.0, sPer = 0.0, n0 = 0.0, n1 = 0.0, n2 = 0.0, emax = 0.0;
    for (int kl = lane; kl < n; kl += 32) {
        int k = st + kl;
        int nx = (kl + 1 == n) ? st : k + 1;
        int pv = (kl == 0) ? en - 1 : k - 1;
        double2 pk = pos[k], pn = pos[nx], pp = pos[pv];
        double x1x = wrap(pk.x - p0.x), x1y = wrap(pk.y - p0.y);
        double dxPrev = wrap(pk.x - pp.x), dyPrev = wrap(pk.y - pp.y);
        double dxNext = wrap(pk.x - pn.x), dyNext = wrap(pk.y - pn.y);
        double lenPrev = sqrt(dxPrev * dxPrev + dyPrev * dyPrev);
        double lenNext = sqrt(dxNext * dxNext + dyNext * dyNext);
        // alpha = 0: x4 = wrap(y_prev - y_next), areaComp = -x4
        // alpha = 1: x4 = wrap(x_prev - x_next), areaComp = +x4
        double a0 = -wrap(pp.y - pn.y);
        double a1 = wrap(pp.x - pn.x);
        double e20 = dxNext + dxPrev, e21 = dyNext + dyPrev;
        double u0 = (dxNext / lenNext) + (dxPrev / lenPrev);
        double u1 = (dyNext / lenNext) + (dyPrev / lenPrev);
        double* c = constraints + 6 * (size_t)k;
        c[0] = a0; c[1] = a1; c[2] = e20; c[3] = e21; c[4] = u0; c[5] = u1;
        n0 += a0 * a0 + a1 * a1;
        n1 += e20 * e20 + e21 * e21;
        n2 += u0 * u0 + u1 * u1;
        double dx = wrap(pn.x - pk.x), dy = wrap(pn.y - pk.y);
        double el = sqrt(dx * dx + dy * dy);
        edgeLengths[k] = el;
        double x2 = wrap(pn.x - p0.x);
        sA += dy * (x2 + x1x) / 2.0;
        sX += x1x;
        sY += x1y;
        sPer += el;
        emax = fmax(emax, el);
    }
    {
        const Sum4 s4 = warp_sum4(sA, sX, sY, sPer), t4 = warp_sum4(n0, n1, n2, 0.0);
        sA = s4.x; sX = s4.y; sY = s4.z; sPer = s4.w; n0 = t4.x; n1 = t4.y; n2 = t4.z;
    }
    emax = warp_maxd(emax);
    if (lane == 0) {
        areas[p] = sA;
        perimeters[p] = sPer;
        double cx = sX / (double)n + p0.x;
        cx -= floor(cx);
        double cy = sY / (double)n + p0.y;
        cy -= floor(cy);
        comX[p] = cx;
        comY[p] = cy;
        atomic_max_nonneg(maxEdge, emax);
    }
    double r0 = n0 > 0.0 ? sqrt(n0) : 1.0;
    double r1 = n1 > 0.0 ? sqrt(n1) : 1.0;
    double r2 = n2 > 0.0 ? sqrt(n2) : 1.0;
    for (int kl = lane; kl < n; kl += 32) {
        double* c = constraints + 6 * (size_t)(st + kl);
        c[0] /= r0; c[1] /= r0; c[2] /= r1; c[3] /= r1; c[4] /= r2; c[5] /= r2;
    }
}

cudaError_t launch_geometry(const double2* pos, const int* start, int P, int V,
                            double* edgeLengths, double* areas, double* comX, double* comY,
                            double* perimeters, double* constraints, double* maxEdge,
                            const int* gate, cudaStream_t st) {
    (void)V;
    if (P <= 0) return cudaSuccess;
    launch_k(k_zero_scalar, dim3(1), dim3(1), 0, st, maxEdge, gate);
    launch_k(k_geometry, dim3(blocks_for(P, 8)), dim3(256), 0, st, pos, start, P, edgeLengths, areas, comX, comY,
                                                 perimeters, constraints, maxEdge, gate);
    return cudaGetLastError();
}

// ------------------------------------------------------- midpoint cells ----
__global__ void k_neighbor_cells(const double2* __restrict__ pos, const int* __restrict__ start,
                                 const int* __restrict__ shapeId, int V, int B,
                                 int* __restrict__ cell, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    int v2 = i + 1;
    if (i == V - 1 || shapeId[i] != shapeId[i + 1]) v2 = start[shapeId[i]];
    double2 a = pos[i], b = pos[v2];
    cell[i] = midpoint_cell_fast(a, b, make_float2((float)a.x, (float)a.y),
                                 make_float2((float)b.x, (float)b.y), B);
}

cudaError_t launch_neighbor_cells(const double2* pos, const int* start, const int* shapeId,
                                  int V, int B, int* cellLocation, const int* gate,
                                  cudaStream_t st) {
    if (V <= 0) return cudaSuccess;
    if (B < 1) B = 1;
    launch_k(k_neighbor_cells, dim3(blocks_for(V, 256)), dim3(256), 0, st, pos, start, shapeId, V, B, cellLocation,
                                                         gate);
    return cudaGetLastError();
}

// ------------------------------------------------------- element-wise ----
// updatePositionsKernel (kernels.cuh:1433-1438)
__global__ void k_update_positions(double* __restrict__ pos, const double* __restrict__ force,
                                   int n2, double dt) {
    pdl_enter();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2) return;
    double p = pos[i] + force[i] * dt;
    pos[i] = p - floor(p);
}

cudaError_t launch_update_positions(double* pos, const double* force, int V, double dt,
                                    cudaStream_t st) {
    if (V <= 0) return cudaSuccess;
    launch_k(k_update_positions, dim3(blocks_for(2LL * V, 256)), dim3(256), 0, st, pos, force, 2 * V, dt);
    return cudaGetLastError();
}

// resetAreasKernel (kernels.cuh:1440-1455)
__global__ void k_reset_areas(double* __restrict__ pos, const int* __restrict__ shapeId,
                              const double* __restrict__ areas, const double* __restrict__ tgt,
                              const double* __restrict__ comX, const double* __restrict__ comY,
                              int n2) {
    pdl_enter();
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n2) return;
    double x = pos[idx];
    int s = shapeId[idx / 2];
    double cur = areas[s], target = tgt[s];
    if (!(cur > 0.0)) return;
    double rescale = sqrt(target / cur);
    double u = (idx % 2) ? wrap(x - comY[s]) : wrap(x - comX[s]);
    u *= rescale;
    double p = (idx % 2) ? u + comY[s] : u + comX[s];
    pos[idx] = p - floor(p);
}

cudaError_t launch_reset_areas(double* pos, const int* shapeId, const double* areas,
                               const double* targetAreas, const double* comX,
                               const double* comY, int V, cudaStream_t st) {
    if (V <= 0) return cudaSuccess;
    launch_k(k_reset_areas, dim3(blocks_for(2LL * V, 256)), dim3(256), 0, st, pos, shapeId, areas, targetAreas,
                                                            comX, comY, 2 * V);
    return cudaGetLastError();
}

// max |x| (getMaxUnbalancedForceCUDA, model.cu:91-109); out must be zeroed.
__global__ void k_max_abs(const double* __restrict__ x, int n, double* __restrict__ out) {
    pdl_enter();
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        m = fmax(m, fabs(x[i]));
    m = warp_maxd(m);
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(out, m);
}

cudaError_t launch_max_abs(const double* x, int n, double* out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
    if (e != cudaSuccess || n <= 0) return e;
    int b = blocks_for(n, 256);
    if (b > 4 * sm_count()) b = 4 * sm_count();
    launch_k(k_max_abs, dim3(b), dim3(256), 0, st, x, n, out);
    return cudaGetLastError();
}

// effectiveForceMagKernel (kernels.cuh:625-633) + max (model.cu:284-306)
__global__ void k_max_eff(const double* __restrict__ pos, const double* __restrict__ tent,
                          const double* __restrict__ f, int V, double scale,
                          double* __restrict__ out) {
    pdl_enter();
    double m = 0.0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < V; k += gridDim.x * blockDim.x) {
        double fx = f[2 * k] + scale * (pos[2 * k] - tent[2 * k]);
        double fy = f[2 * k + 1] + scale * (pos[2 * k + 1] - tent[2 * k + 1]);
        m = fmax(m, sqrt(fx * fx + fy * fy));
    }
    m = warp_maxd(m);
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(out, m);
}

cudaError_t launch_max_effective_force(const double* pos, const double* posTent,
                                       const double* force, int V, double scale,
                                       double* out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
    if (e != cudaSuccess || V <= 0) return e;
    int b = blocks_for(V, 256);
    if (b > 4 * sm_count()) b = 4 * sm_count();
    launch_k(k_max_eff, dim3(b), dim3(256), 0, st, pos, posTent, force, V, scale, out);
    return cudaGetLastError();
}

// ------------------------------------------------------ soft-body terms ----
__device__ __forceinline__ double loop_wrap_below_one(double x) {
    int it = 0;
    while (x >= 1.0 && it < 64) { x -= 1.0; ++it; }
    return x;
}

// updateForceEnergyEdgeKernel (kernels.cuh:1284-1335)
__global__ void k_soft_edge(const double2* __restrict__ pos, const double* __restrict__ tl,
                            const double* __restrict__ el, const int* __restrict__ next,
                            const int* __restrict__ prev, const int* __restrict__ shapeId, int V,
                            double stiffness, double* __restrict__ force,
                            double* __restrict__ energy, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    double le = 0.0;
    if (m < V) {
        int prv = prev[m], nxt = next[m];
        double l0 = tl[shapeId[m]], l0prv = tl[shapeId[prv]];
        double l = el[m], prvl = el[prv];
        double2 pm = pos[m], pn = pos[nxt], pp = pos[prv];
        double ax = loop_wrap_below_one(pm.x - pn.x + 1.5) - 0.5;
        double ay = loop_wrap_below_one(pm.y - pn.y + 1.5) - 0.5;
        double bx = loop_wrap_below_one(pp.x - pm.x + 1.5) - 0.5;
        double by = loop_wrap_below_one(pp.y - pm.y + 1.5) - 0.5;
        double c1 = (l > 1e-14) ? (1.0 - l0 / l) : 0.0;
        double c2 = (prvl > 1e-14) ? (1.0 - l0prv / prvl) : 0.0;
        le = stiffness * (l - l0) * (l - l0) / 2.0;
        double fx = -(c1 * ax - c2 * bx) * stiffness;
        double fy = -(c1 * ay - c2 * by) * stiffness;
        if (fx != 0.0 || fy != 0.0) {
            atomicAdd(&force[2 * m], fx);
            atomicAdd(&force[2 * m + 1], fy);
        }
    }
    le = warp_sum(le);
    if ((threadIdx.x & 31) == 0 && le != 0.0) atomicAdd(energy, le);
}

cudaError_t launch_soft_edge(const double2* pos, const double* targetEdgeLengths,
                             const double* edgeLengths, const int* next, const int* prev,
                             const int* shapeId, int V, double stiffness, double* force,
                             double* energy, const int* gate, cudaStream_t st) {
    if (V <= 0) return cudaSuccess;
    launch_k(k_soft_edge, dim3(blocks_for(V, 256)), dim3(256), 0, st, pos, targetEdgeLengths, edgeLengths, next,
                                                     prev, shapeId, V, stiffness, force, energy,
                                                     gate);
    return cudaGetLastError();
}

// updateForceEnergyAreaKernel (kernels.cuh:1337-1352)
__global__ void k_soft_area(const double2* __restrict__ pos, const int* __restrict__ shapeId,
                            const int* __restrict__ next, const int* __restrict__ prev,
                            const double* __restrict__ areas, const double* __restrict__ tgt,
                            const int* __restrict__ start, int V, double comp,
                            double* __restrict__ force, double* __restrict__ energy,
                            const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    double le = 0.0;
    if (m < V) {
        int s = shapeId[m];
        double A = areas[s], A0 = tgt[s];
        if (!(A0 < 1e-14)) {
            double coeff = 0.5 * comp * (A - A0);
            double2 pn = pos[next[m]], pp = pos[prev[m]];
            double fx = -coeff * wrap(pn.y - pp.y);
            double fy = -coeff * wrap(pp.x - pn.x);
            atomicAdd(&force[2 * m], fx);
            atomicAdd(&force[2 * m + 1], fy);
            if (start[s] == m) le = comp * (A - A0) * (A - A0) / 2.0;
        }
    }
    le = warp_sum(le);
    if ((threadIdx.x & 31) == 0 && le != 0.0) atomicAdd(energy, le);
}

cudaError_t launch_soft_area(const double2* pos, const int* shapeId, const int* next,
                             const int* prev, const double* areas, const double* targetAreas,
                             const int* start, int V, double compressibility, double* force,
                             double* energy, const int* gate, cudaStream_t st) {
    if (V <= 0) return cudaSuccess;
    launch_k(k_soft_area, dim3(blocks_for(V, 256)), dim3(256), 0, st, pos, shapeId, next, prev, areas, targetAreas,
                                                     start, V, compressibility, force, energy, gate);
    return cudaGetLastError();
}

// ------------------------------------------------- Monte-Carlo overlap ----
// updateOverlapAreaKernel (kernels.cuh:879-979) + the CUB sum
// (model.cu:466-507).  Grid point (ix + 0.5, iy + 0.5) / d; polygons owning
// vertices in the 3x3 cells around it; angle-sum inside test; c(c-1)/2.
__device__ __forceinline__ double wrap_periodic(double x) {
    x += 1.5;
    int it = 0;
    while (x > 1.0 && it < 64) { x -= 1.0; ++it; }
    return x - 0.5;
}

__global__ void k_overlap_mc(const double2* __restrict__ pos, const int* __restrict__ start,
                             const int* __restrict__ shapeId, const int* __restrict__ nbIdx,
                             const int* __restrict__ boxStarts, int V, int B, int d,
                             int* __restrict__ counter, unsigned long long* __restrict__ sum) {
    pdl_enter();
    const double eps = 1e-12;
    const double pi = 3.141592653589793238462643383279;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    long long total = (long long)d * d;
    int val = 0;
    if (idx < total) {
        int ix = idx % d, iy = idx / d;
        double px = (ix + 0.5) / d, py = (iy + 0.5) / d;
        int cellX = (int)(px * B), cellY = (int)(py * B);
        int boxCount = B * B;
        int tracked[512];
        int nt = 0, hits = 0;
        bool full = false;
        for (int dx = -1; dx <= 1 && !full; dx++) {
            int nx = cellX + dx;
            if (nx < 0) nx += B; else if (nx >= B) nx -= B;
            for (int dy = -1; dy <= 1 && !full; dy++) {
                int ny = cellY + dy;
                if (ny < 0) ny += B; else if (ny >= B) ny -= B;
                int box = ny * B + nx;
                int si = boxStarts[box];
                int sf = (box + 1 < boxCount) ? boxStarts[box + 1] : V;
                for (int q = si; q < sf; q++) {
                    int poly = shapeId[nbIdx[q]];
                    bool seen = false;
                    for (int t = 0; t < nt; t++) if (tracked[t] == poly) { seen = true; break; }
                    if (seen) continue;
                    int s0 = start[poly], s1 = start[poly + 1];
                    if (s1 - s0 >= 3) {
                        double ang = 0.0;
                        double vxp = wrap_periodic(pos[s0].x - px);
                        double vyp = wrap_periodic(pos[s0].y - py);
                        double vx0 = vxp, vy0 = vyp;
                        for (int e = s0 + 1; e < s1; e++) {
                            double vx = vxp + wrap_periodic(pos[e].x - pos[e - 1].x);
                            double vy = vyp + wrap_periodic(pos[e].y - pos[e - 1].y);
                            // the reference's contracted products, rounded
                            // as its build rounds them (a grid point on an
                            // edge takes its count from the cross's sign)
                            ang += atan2(__fma_rn(vxp, vy, -__dmul_rn(vyp, vx)),
                                         __fma_rn(vxp, vx, __dmul_rn(vyp, vy)));
                            vxp = vx; vyp = vy;
                        }
                        ang += atan2(__fma_rn(vxp, vy0, -__dmul_rn(vyp, vx0)),
                                     __fma_rn(vxp, vx0, __dmul_rn(vyp, vy0)));
                        if (fabs(ang - 2.0 * pi) < eps) hits++;
                    }
                    if (nt < 512) tracked[nt++] = poly;
                    else { full = true; break; }
                }
            }
        }
        val = hits * (hits - 1) / 2;
        counter[idx] = val;
    }
    unsigned long long v = (unsigned long long)val;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(PCP_FULL, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(sum, v);
}

cudaError_t launch_overlap_area_mc(const double2* pos, const int* start, const int* shapeId,
                                   const int* neighborIndices, const int* boxStarts, int V,
                                   int B, int pointDensity, int* counter,
                                   unsigned long long* sum, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(sum, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    long long total = (long long)pointDensity * pointDensity;
    if (total <= 0) return cudaSuccess;
    launch_k(k_overlap_mc, dim3(blocks_for(total, 128)), dim3(128), 0, st, pos, start, shapeId, neighborIndices,
                                                          boxStarts, V, B < 1 ? 1 : B,
                                                          pointDensity, counter, sum);
    return cudaGetLastError();
}

}  // namespace pcp
