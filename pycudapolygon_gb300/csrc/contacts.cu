// contacts.cu -- contact search and overlap energy/force on GB300 (sm_103a).
//
// Replaces the reference's edge-level cell list + per-edge narrow phase +
// compaction + two radix sorts + outersection search + exterior/interior
// kernels (camdennis/pyCudaPolygon src/kernels.cuh:661-1424, src/model.cu:
// 308-551, src/model.cpp:252-372) by:
//
//   prepass      one warp per polygon: exact FP64 edge vectors, FP32 copies of
//                the ring with its edge-midpoint cells, bounding circle
//   broad phase  polygon grid built by counting sort (histogram, prefix sum,
//                scatter) on cell key; candidate pairs a <= b whose bounding
//                circles overlap (a == b covers self-crossings)
//   narrow phase one warp per candidate pair, both rings staged in shared
//                memory by cp.async.bulk (TMA) with an mbarrier, double
//                buffered across the warp's pairs; a conservative FP32 box
//                test and the reference's cell-adjacency rule filter edge
//                pairs; survivors get the reference's exact FP64 crossing
//                test (no FMA contraction) in full-warp batches; the pair's
//                crossings are matched to their exits (outersections) in
//                shared memory and written out as packed records
//   force        one thread per record: exterior terms and the interior
//                chain of whole edges, FP64, forces by atomics
//
// The crossing set equals the reference's whenever its cell scan would see
// the pair: polygons whose bounding circles do not overlap cannot have
// crossing edges, and the reference's own 3x3 cell rule is applied to every
// edge pair.  Records are bit-identical; their order is restored to the
// reference's (si, i, j, sj) order only when a getter asks for them.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "pcp_common.cuh"
#include "pcp_internal.h"
#include "pcp_fire.cuh"

namespace pcp {

static inline int nblocks(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (int)b;
}

// ------------------------------------------------------------ prepass ----
// Smallest FP32 fan cross product that certifies a strictly positive one,
// per unit of the polygon's extent L (its box's larger side): each FP32
// coordinate relative to the box centre is within 1.8e-7 of the exact value
// for the FP64 positions, so a cross product of two (each below L) is within
// 4 L 1.8e-7 (+ L^2 2^-22 for rounding).
constexpr float kStarEpsPerL = 1e-6f;

// Reset of the contact counters (everything in Ctrl before `energy`).
__global__ void k_reset_contacts(Ctrl* __restrict__ ctrl, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int* w = reinterpret_cast<int*>(ctrl);
    int n = (int)(offsetof(Ctrl, energy) / sizeof(int));
    for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] = 0;
}

__global__ void __launch_bounds__(256)
k_prepass(double2* __restrict__ pos, const int* __restrict__ start,
          const int* __restrict__ cellLocation, int* __restrict__ cellOut, int P, int B,
          double2* __restrict__ edgeVec, float4* __restrict__ vtx, float4* __restrict__ polyInfo,
          float4* __restrict__ polyBox, int* __restrict__ polyFlags,
          Ctrl* __restrict__ ctrl, FireMove mv, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    __shared__ float s_r[8];
    const int p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float Rsafe = 0.f;
    const int st = p < P ? start[p] : 0;
    const int n = p < P ? start[p + 1] - st : 0;
    // polygons of up to 32 vertices: one vertex per lane, the next vertex by
    // shuffle instead of a second read of the positions just written
    const bool lanes = n >= 1 && n <= 32;
    double2 xl = make_double2(0.0, 0.0);
    if (mv.pos) {
        // start of a FIRE step: resets (Rmax was zeroed at the end of the
        // last step and is accumulated below), then this polygon's Verlet move
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            fire_step_resets(mv.c);
            zero_contact_counters_but_rmax(mv.c);
        }
        const double dt = mv.c->dt;
        const int bm = mv.c->bendMode;
        const double ba = mv.c->bendA, bs = mv.c->bendS;
        if (lanes) {
            if (lane < n) {
                xl = fire_move_vertex(mv, st + lane, dt, bm, ba, bs);
                pos[st + lane] = xl;
            }
        } else {
            for (int kl = lane; kl < n; kl += 32)
                pos[st + kl] = fire_move_vertex(mv, st + kl, dt, bm, ba, bs);
            __syncwarp();
        }
    } else if (lanes && lane < n) {
        xl = pos[st + lane];
    }
    if (p < P && lanes) {
        // the same values as the general form below, from registers
        const bool live = lane < n;
        const int kn = (lane + 1 >= n) ? 0 : lane + 1;
        const double2 xn = make_double2(__shfl_sync(PCP_FULL, xl.x, kn),
                                        __shfl_sync(PCP_FULL, xl.y, kn));
        const float fx = d2f_int(xl.x), fy = d2f_int(xl.y);
        const float fnx = __shfl_sync(PCP_FULL, fx, kn), fny = __shfl_sync(PCP_FULL, fy, kn);
        const float f0x = __shfl_sync(PCP_FULL, fx, 0), f0y = __shfl_sync(PCP_FULL, fy, 0);
        float mnx = 0.f, mxx = 0.f, mny = 0.f, mxy = 0.f, emax = 0.f;
        bool bad = false;
        if (live) {
            const int k = st + lane;
            edgeVec[k] = make_double2(wrap(xn.x - xl.x), wrap(xn.y - xl.y));
            int cell;
            if (cellOut) {
                cell = midpoint_cell_fast(xl, xn, make_float2(fx, fy), make_float2(fnx, fny), B);
                cellOut[k] = cell;
            } else {
                cell = cellLocation[k];
            }
            vtx[k] = make_float4(fx, fy, __int_as_float(cell % B), __int_as_float(cell / B));
            float lx = wrapf(fx - f0x), ly = wrapf(fy - f0y);
            float nxl = wrapf(fnx - fx), nyl = wrapf(fny - fy);
            if (!(isfinite(lx) && isfinite(ly) && isfinite(nxl) && isfinite(nyl))) bad = true;
            mnx = fminf(mnx, lx); mxx = fmaxf(mxx, lx);
            mny = fminf(mny, ly); mxy = fmaxf(mxy, ly);
            emax = fmaxf(emax, sqrtf(nxl * nxl + nyl * nyl));
        }
        mnx = warp_minf(mnx); mxx = warp_maxf(mxx);
        mny = warp_minf(mny); mxy = warp_maxf(mxy);
        emax = warp_maxf(emax);
        bad = __any_sync(PCP_FULL, bad);
        const float cxl = 0.5f * (mnx + mxx), cyl = 0.5f * (mny + mxy);
        const float L = fmaxf(fmaxf(mxx - mnx, mxy - mny), 0.f);
        float minCross = 3.0e38f, sweep = 0.f;
        bool crossNaN = false;
        if (live) {
            float ax = wrapf(fx - f0x) - cxl, ay = wrapf(fy - f0y) - cyl;
            float bx = wrapf(fnx - f0x) - cxl, by = wrapf(fny - f0y) - cyl;
            float c = ax * by - ay * bx;
            crossNaN |= isnan(c);
            minCross = fminf(minCross, c);
            sweep += atan2f(c, ax * bx + ay * by);
        }
        minCross = warp_minf(minCross);
        crossNaN = __any_sync(PCP_FULL, crossNaN);
        for (int o = 16; o > 0; o >>= 1) sweep += __shfl_xor_sync(PCP_FULL, sweep, o);
        const bool star = !crossNaN && L >= 1e-4f && minCross > kStarEpsPerL * L &&
                          fabsf(sweep - 6.2831853f) < 1.0f;
        if (lane == 0) {
            float cx = f0x + 0.5f * (mnx + mxx), cy = f0y + 0.5f * (mny + mxy);
            cx -= floorf(cx); cy -= floorf(cy);
            float w = mxx - mnx, h = mxy - mny;
            float R = 0.5f * sqrtf(w * w + h * h) * 1.0001f + 4e-6f;
            bool safe = !bad && isfinite(R) && R < 0.1f && n >= 3;
            polyInfo[p] = make_float4(cx, cy, R, emax);
            polyBox[p] = make_float4(mnx, mxx, mny, mxy);
            polyFlags[p] = safe ? ((star && n >= 4) ? 3 : 1) : 0;
            if (safe) Rsafe = R;
        }
    } else if (p < P && n <= 0) {   // empty polygon: no edges, never a candidate
        if (lane == 0) {
            polyInfo[p] = make_float4(0.f, 0.f, 0.f, 0.f);
            polyBox[p] = make_float4(0.f, 0.f, 0.f, 0.f);
            polyFlags[p] = 0;
        }
    } else if (p < P) {
        double2 q0 = pos[st];
        float f0x = d2f_int(q0.x), f0y = d2f_int(q0.y);
        float mnx = 0.f, mxx = 0.f, mny = 0.f, mxy = 0.f, emax = 0.f;
        bool bad = false;
        for (int kl = lane; kl < n; kl += 32) {
            int k = st + kl;
            int nx = (kl + 1 == n) ? st : k + 1;
            double2 pk = pos[k], pn = pos[nx];
            // r = wrap(p_next - p) exactly as updateNeighborsKernel (kernels.cuh:724-725)
            edgeVec[k] = make_double2(wrap(pn.x - pk.x), wrap(pn.y - pk.y));
            // FP32 copies by truncation on the integer pipe (within one float
            // ulp; the culls' margins allow for 1.2e-7)
            float fx = d2f_int(pk.x), fy = d2f_int(pk.y);
            float fnx = d2f_int(pn.x), fny = d2f_int(pn.y);
            // cell (x, y) of the edge midpoint as updateNeighborsKernel splits it
            // with the current box size (kernels.cuh:727-729); with cellOut the
            // cells are computed here from the same positions
            // (updateNeighborCellsKernel) and stored for the getters
            int cell;
            if (cellOut) {
                cell = midpoint_cell_fast(pk, pn, make_float2(fx, fy), make_float2(fnx, fny), B);
                cellOut[k] = cell;
            } else {
                cell = cellLocation[k];
            }
            vtx[k] = make_float4(fx, fy, __int_as_float(cell % B), __int_as_float(cell / B));
            float lx = wrapf(fx - f0x), ly = wrapf(fy - f0y);
            float nxl = wrapf(fnx - fx), nyl = wrapf(fny - fy);
            if (!(isfinite(lx) && isfinite(ly) && isfinite(nxl) && isfinite(nyl))) bad = true;
            mnx = fminf(mnx, lx); mxx = fmaxf(mxx, lx);
            mny = fminf(mny, ly); mxy = fmaxf(mxy, ly);
            emax = fmaxf(emax, sqrtf(nxl * nxl + nyl * nyl));
        }
        mnx = warp_minf(mnx); mxx = warp_maxf(mxx);
        mny = warp_minf(mny); mxy = warp_maxf(mxy);
        emax = warp_maxf(emax);
        bad = __any_sync(PCP_FULL, bad);
        // star test about the box centre c (vertex 0's frame): every fan
        // triangle (c, v_k, v_k+1) positive with margin and the fan winding
        // once (the angle steps, each in (0, pi), add up to 2 pi, not 4 pi)
        __syncwarp();
        const float cxl = 0.5f * (mnx + mxx), cyl = 0.5f * (mny + mxy);
        const float L = fmaxf(fmaxf(mxx - mnx, mxy - mny), 0.f);
        float minCross = 3.0e38f, sweep = 0.f;
        bool crossNaN = false;
        for (int kl = lane; kl < n; kl += 32) {
            float4 va = vtx[st + kl], vb = vtx[(kl + 1 == n) ? st : st + kl + 1];
            float ax = wrapf(va.x - f0x) - cxl, ay = wrapf(va.y - f0y) - cyl;
            float bx = wrapf(vb.x - f0x) - cxl, by = wrapf(vb.y - f0y) - cyl;
            float c = ax * by - ay * bx;
            crossNaN |= isnan(c);
            minCross = fminf(minCross, c);
            sweep += atan2f(c, ax * bx + ay * by);
        }
        minCross = warp_minf(minCross);
        crossNaN = __any_sync(PCP_FULL, crossNaN);
        for (int o = 16; o > 0; o >>= 1) sweep += __shfl_xor_sync(PCP_FULL, sweep, o);
        // (polygons under 1e-4 across are left to the search: there the
        // absolute FP32 error of the coordinates is not small against L)
        const bool star = !crossNaN && L >= 1e-4f && minCross > kStarEpsPerL * L &&
                          fabsf(sweep - 6.2831853f) < 1.0f;
        if (lane == 0) {
            float cx = f0x + 0.5f * (mnx + mxx), cy = f0y + 0.5f * (mny + mxy);
            cx -= floorf(cx); cy -= floorf(cy);
            float w = mxx - mnx, h = mxy - mny;
            float R = 0.5f * sqrtf(w * w + h * h) * 1.0001f + 4e-6f;
            bool safe = !bad && isfinite(R) && R < 0.1f && n >= 3;
            polyInfo[p] = make_float4(cx, cy, R, emax);
            polyBox[p] = make_float4(mnx, mxx, mny, mxy);
            // bit 0: well formed (extent < 0.2, finite); bit 1: also simple
            // with room to spare -- star-shaped about the box centre with
            // every fan triangle above kStarEpsPerL L in FP32 and winding
            // once, so non-adjacent edges lie in angular sectors about the
            // centre that are separated by sectors of positive width and the
            // FP64 crossing test cannot accept any of them; its self pair is
            // not searched
            polyFlags[p] = safe ? ((star && n >= 4) ? 3 : 1) : 0;
            if (safe) Rsafe = R;
        }
    }
    // one atomic per block for the largest safe radius
    if (lane == 0) s_r[warp] = Rsafe;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmaxf(r, s_r[w]);
        if (r > 0.f) atomic_max_nonneg_f(&ctrl->Rmax, r);
    }
}

// -------------------------------------------------------- broad phase ----
__device__ __forceinline__ int grid_dim_from(float Rmax) {
    float side = 2.0f * Rmax * 1.001f + 1e-4f;
    int G = (int)floorf(1.0f / side);
    if (!(G >= 1)) G = 1;
    if (G > kGridMax) G = kGridMax;
    return G;
}
__device__ __forceinline__ int grid_cell(float c, int G) {
    int i = (int)floorf(c * (float)G);
    if (i < 0) i = 0;
    if (i >= G) i = G - 1;
    return i;
}

__global__ void k_grid_count(const float4* __restrict__ polyInfo, const int* __restrict__ flags,
                             int P, int* __restrict__ gridCount, Ctrl* __restrict__ ctrl,
                             const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int G = grid_dim_from(ctrl->Rmax);
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) ctrl->G = G;
    if (p >= P || !flags[p]) return;
    float4 c = polyInfo[p];
    atomicAdd(&gridCount[grid_cell(c.y, G) * G + grid_cell(c.x, G)], 1);
}

// exclusive scan of the G*G counts in one block (G*G <= 65536)
__global__ void __launch_bounds__(1024)
k_grid_scan(int* __restrict__ gridCount, int* __restrict__ gridStart, int* __restrict__ gridFill,
            Ctrl* __restrict__ ctrl, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    __shared__ int warpSums[32];
    int G = ctrl->G;
    int N = G * G;
    int per = (N + blockDim.x - 1) / blockDim.x;
    int b0 = threadIdx.x * per;
    int local = 0;
    for (int i = 0; i < per; ++i) {
        int idx = b0 + i;
        if (idx < N) local += gridCount[idx];
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(PCP_FULL, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warpSums[w] = incl;
    __syncthreads();
    if (w == 0) {
        int v = lane < (int)(blockDim.x >> 5) ? warpSums[lane] : 0;
        int s = v;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(PCP_FULL, s, o);
            if (lane >= o) s += t;
        }
        warpSums[lane] = s - v;
    }
    __syncthreads();
    int run = warpSums[w] + incl - local;
    for (int i = 0; i < per; ++i) {
        int idx = b0 + i;
        if (idx < N) {
            gridStart[idx] = run;
            run += gridCount[idx];
            gridFill[idx] = 0;
            gridCount[idx] = 0;    // ready for the next search
        }
    }
    if (threadIdx.x == blockDim.x - 1) gridStart[N] = run;
}

__global__ void k_grid_scatter(const float4* __restrict__ polyInfo, const int* __restrict__ flags,
                               int P, const int* __restrict__ gridStart, int* __restrict__ gridFill,
                               int* __restrict__ sortedPoly, const Ctrl* __restrict__ ctrl,
                               const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P || !flags[p]) return;
    int G = ctrl->G;
    float4 c = polyInfo[p];
    int cell = grid_cell(c.y, G) * G + grid_cell(c.x, G);
    sortedPoly[gridStart[cell] + atomicAdd(&gridFill[cell], 1)] = p;
}

// The three steps above in one block, for systems of up to kFusedMaxPolys
// polygons: counts in shared memory when the grid has at most kFusedCells
// cells (else in gridCount, which is left zeroed), an exclusive scan into
// gridStart, and the scatter through atomic increments of the scanned
// starts (a counting sort; the order inside a cell is arbitrary, as with
// k_grid_scatter).
constexpr int kFusedCells = 8192;
constexpr int kFusedMaxPolys = 65536;
constexpr int kFusedRegItems = 8;
__global__ void __launch_bounds__(1024, 1)
k_grid_fused(const float4* __restrict__ polyInfo, const int* __restrict__ flags, int P,
             int* __restrict__ gridCount, int* __restrict__ gridStart,
             int* __restrict__ sortedPoly, Ctrl* __restrict__ ctrl, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    __shared__ int s_cnt[kFusedCells];
    __shared__ int warpSums[32];
    const int G = grid_dim_from(ctrl->Rmax);
    const int N = G * G;
    if (threadIdx.x == 0) ctrl->G = G;
    const bool inSmem = N <= kFusedCells;
    int* cnt = inSmem ? s_cnt : gridCount;
    if (inSmem)
        for (int i = threadIdx.x; i < N; i += blockDim.x) s_cnt[i] = 0;
    // up to kFusedRegItems polygons per thread: every load issued before the
    // first atomic, and the cells kept in registers for the scatter
    const bool inReg = P <= kFusedRegItems * (int)blockDim.x;
    int cell[kFusedRegItems];
    if (inReg) {
#pragma unroll
        for (int k = 0; k < kFusedRegItems; ++k) {
            const int p = threadIdx.x + k * blockDim.x;
            cell[k] = -1;
            if (p < P) {
                const int f = flags[p];
                const float2 c = *reinterpret_cast<const float2*>(&polyInfo[p]);
                if (f) cell[k] = grid_cell(c.y, G) * G + grid_cell(c.x, G);
            }
        }
    }
    __syncthreads();
    if (inReg) {
#pragma unroll
        for (int k = 0; k < kFusedRegItems; ++k)
            if (cell[k] >= 0) atomicAdd(&cnt[cell[k]], 1);
    } else {
        for (int p = threadIdx.x; p < P; p += blockDim.x) {
            if (!flags[p]) continue;
            float4 c = polyInfo[p];
            atomicAdd(&cnt[grid_cell(c.y, G) * G + grid_cell(c.x, G)], 1);
        }
    }
    __syncthreads();
    // exclusive scan: contiguous runs per thread, then across warps
    const int per = (N + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per;
    int local = 0;
    for (int i = 0; i < per; ++i) {
        int idx = b0 + i;
        if (idx < N) local += cnt[idx];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(PCP_FULL, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warpSums[w] = incl;
    __syncthreads();
    if (w == 0) {
        int v = lane < (int)(blockDim.x >> 5) ? warpSums[lane] : 0;
        int sc = v;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(PCP_FULL, sc, o);
            if (lane >= o) sc += t;
        }
        warpSums[lane] = sc - v;
    }
    __syncthreads();
    int run = warpSums[w] + incl - local;
    for (int i = 0; i < per; ++i) {
        int idx = b0 + i;
        if (idx < N) {
            int c = cnt[idx];
            gridStart[idx] = run;
            cnt[idx] = run;
            run += c;
        }
    }
    if (threadIdx.x == blockDim.x - 1) gridStart[N] = run;
    __syncthreads();
    if (inReg) {
#pragma unroll
        for (int k = 0; k < kFusedRegItems; ++k)
            if (cell[k] >= 0) sortedPoly[atomicAdd(&cnt[cell[k]], 1)] = threadIdx.x + k * blockDim.x;
    } else {
        for (int p = threadIdx.x; p < P; p += blockDim.x) {
            if (!flags[p]) continue;
            float4 c = polyInfo[p];
            sortedPoly[atomicAdd(&cnt[grid_cell(c.y, G) * G + grid_cell(c.x, G)], 1)] = p;
        }
    }
    if (!inSmem) {
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) gridCount[i] = 0;
    }
}

// One warp per polygon i: the lanes walk the polygons of the (up to) nine
// neighbouring grid cells and keep j > i whose bounding circle meets i's
// (the pair evaluations the benchmark counts) and whose bounding box, padded
// by the narrow phase's margin, meets i's (the pairs emitted: the narrow
// phase finds nothing in the others).  The polygons not well formed pair
// with everyone.  Pass 1 counts, the block reserves its slots with one
// atomic, pass 2 writes.
__device__ __forceinline__ bool box_pair(const float4& ci, const float4& bi, const float4& cj,
                                         const float4& bj) {
    float ddx = wrapf(cj.x - ci.x), ddy = wrapf(cj.y - ci.y);
    float m = 2.f * (4e-6f + 1e-3f * ci.w * cj.w) + 2e-6f;
    float hx = 0.5f * ((bi.y - bi.x) + (bj.y - bj.x)) + m;
    float hy = 0.5f * ((bi.w - bi.z) + (bj.w - bj.z)) + m;
    // NaN keeps the pair
    return !(fabsf(ddx) > hx || fabsf(ddy) > hy);
}

__global__ void __launch_bounds__(256)
k_candidates(const float4* __restrict__ polyInfo, const float4* __restrict__ polyBox,
             const int* __restrict__ flags, const int* __restrict__ start, int P,
             const int* __restrict__ gridStart, const int* __restrict__ sortedPoly,
             int2* __restrict__ pairs, int capPairs, Ctrl* __restrict__ ctrl, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    __shared__ int s_cnt[8];
    __shared__ unsigned long long s_evals[8];
    __shared__ int s_base;
    const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int n = i < P ? start[i + 1] - start[i] : 0;
    const bool active = i < P && n > 0;
    const bool safe = active && flags[i];
    float4 ci = make_float4(0.f, 0.f, 0.f, 0.f), bi = ci;
    // lanes 0..8 own the nine neighbouring grid cells; their ranges of
    // sortedPoly are laid end to end and dealt out one polygon per lane
    int ca = 0, len = 0;
    if (safe) {
        ci = polyInfo[i];
        bi = polyBox[i];
        const int G = ctrl->G;
        if (lane < 9) {
            int nx = grid_cell(ci.x, G) + lane / 3 - 1;
            int ny = grid_cell(ci.y, G) + lane % 3 - 1;
            if (nx < 0) nx += G; else if (nx >= G) nx -= G;
            if (ny < 0) ny += G; else if (ny >= G) ny -= G;
            int cell = ny * G + nx;
            ca = gridStart[cell];
            len = gridStart[cell + 1] - ca;
        }
    }
    // a repeated cell (G < 3) repeats its range exactly: keep the first
    for (int t = 0; t < 8; ++t) {
        int at = __shfl_sync(PCP_FULL, ca, t), lt2 = __shfl_sync(PCP_FULL, len, t);
        if (t < lane && lane < 9 && at == ca && lt2 == len) len = 0;
    }
    int incl = len;
#pragma unroll
    for (int d = 1; d < 16; d <<= 1) {
        int t = __shfl_up_sync(PCP_FULL, incl, d);
        if (lane >= d) incl += t;
    }
    const int total = __shfl_sync(PCP_FULL, incl, 8);
    // the tests of one candidate per lane, done once when the nine cells hold
    // at most 32 polygons (both passes use them)
    auto test_item = [&](int item, bool& circle, bool& box, int& j) {
        // owning cell: the first of lanes 0..8 whose running total exceeds item
        int own = 0;
#pragma unroll
        for (int t = 0; t < 9; ++t) own += (__shfl_sync(PCP_FULL, incl, t) <= item) ? 1 : 0;
        int oa = __shfl_sync(PCP_FULL, ca, own < 9 ? own : 8);
        int oi = __shfl_sync(PCP_FULL, incl - len, own < 9 ? own : 8);
        circle = false; box = false; j = 0;
        if (item < total) {
            j = sortedPoly[oa + item - oi];
            if (j > i) {
                float4 cj = polyInfo[j];
                float ddx = wrapf(cj.x - ci.x), ddy = wrapf(cj.y - ci.y);
                float rr = ci.z + cj.z + 1e-5f;
                circle = ddx * ddx + ddy * ddy <= rr * rr;
                box = circle && box_pair(ci, bi, cj, polyBox[j]);
            }
        }
    };
    const bool once = safe && total <= 32;
    bool circle1 = false, box1 = false;
    int j1 = 0;
    if (once) test_item(lane, circle1, box1, j1);
    // pass 0 counts, pass 1 writes from the reserved base
    int base = 0;
    for (int pass = 0; pass < 2; ++pass) {
        int cnt = 0;
        unsigned long long evals = 0;
        auto put = [&](bool ok, int a, int b) {
            unsigned mk = __ballot_sync(PCP_FULL, ok);
            if (pass == 1 && ok) {
                int slot = base + cnt + __popc(mk & lt);
                if (slot < capPairs) pairs[slot] = make_int2(a, b);
            }
            cnt += __popc(mk);
        };
        if (active) {
            // self crossings are searched unless the prepass certified the
            // polygon simple (kernels.cuh:766-775 records s1 == s2 crossings)
            if (n >= 4 && !(flags[i] & 2)) {
                put(lane == 0, i, i);
                if (pass == 0 && lane == 0) {
                    atomicAdd(&ctrl->numSelf, 1);
                    atomicAdd(&ctrl->selfEvals, 1ull);
                }
            }
            if (!safe) {
                // not well formed: paired with everyone (safe partners below i, all above)
                for (int j0 = 0; j0 < P; j0 += 32) {
                    int j = j0 + lane;
                    bool ok = j < P && j != i && (j > i || flags[j]) && start[j + 1] > start[j];
                    put(ok, j < i ? j : i, j < i ? i : j);
                    evals += ok ? 1 : 0;
                }
            } else if (once) {
                put(box1, i, j1);
                evals += circle1 ? 1 : 0;
            } else {
                for (int b0 = 0; b0 < total; b0 += 32) {
                    bool circle, box;
                    int j;
                    test_item(b0 + lane, circle, box, j);
                    put(box, i, j);
                    evals += circle ? 1 : 0;
                }
            }
        }
        if (pass == 0) {
            evals = (unsigned long long)warp_sumi((int)evals);
            if (lane == 0) { s_cnt[warp] = cnt; s_evals[warp] = evals; }
            __syncthreads();
            if (threadIdx.x == 0) {
                int tot = 0;
                unsigned long long ev = 0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                    int c = s_cnt[w];
                    s_cnt[w] = tot;
                    tot += c;
                    ev += s_evals[w];
                }
                int b0 = tot ? atomicAdd(&ctrl->numPairs, tot) : 0;
                if (b0 + tot > capPairs) atomicOr(&ctrl->flags, kFlagPairOverflow);
                if (ev) atomicAdd(&ctrl->pairEvals, ev);
                if (tot) atomicAdd(&ctrl->narrowEvals, (unsigned long long)tot);
                s_base = b0;
            }
            __syncthreads();
            base = s_base + s_cnt[warp];
        }
    }
}

// -------------------------------------------------------- narrow phase ----

// mbarrier / bulk-copy helpers (PTX ISA: mbarrier, cp.async.bulk)
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}
// Bounded wait: gives up after ~2^24 polls (far beyond any copy's latency)
// and reports it through the control block instead of hanging the GPU.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, uint32_t parity,
                                                  Ctrl* ctrl) {
    for (int it = 0; it < (1 << 24); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(&ctrl->flags, kFlagCapacity);
    atomicExch(&ctrl->errorCode, 100);
    return false;
}

struct PairCtx {
    int a, b;         // polygons (a <= b)
    int stA, stB, nA, nB;
    bool self;
};

__device__ __forceinline__ unsigned long long pack_key(int sj, int si, int i, int j) {
    return ((unsigned long long)(uint16_t)sj << 48) | ((unsigned long long)(uint16_t)si << 32) |
           ((unsigned long long)(uint16_t)i << 16) | (unsigned long long)(uint16_t)j;
}

// Process one staged pair with one warp.  ringA/ringB hold (x, y) of the
// two rings as float and the (x, y) index of each edge's midpoint cell.
// candA/candB are scratch for the edges that survive the overlap-box cull
// (capacity >= nA, nB).  Returns the number of records in recKey/recTU, or
// -1 when they do not fit in recCap.
//
// Culls, all conservative (they never drop a pair the FP64 test accepts):
//  1. overlap box: a crossing point lies in both polygons' bounding boxes,
//     so only edges whose box meets the intersection of the two polygon
//     boxes are kept (cross pairs only);
//  2. edge boxes: FP32 boxes padded by m = 4e-6 + 1e-3 La Lb must meet --
//     the FP32 coordinates are within 1.2e-7 of the FP64 ones and the FP64
//     predicate cannot accept a pair farther apart than 3.3e-4 |r| |s|
//     (its |denom| >= 1e-12 bounds the error of t and u);
//  3. the reference's 3x3 cell rule on the edge-midpoint cells.
struct EdgeCand { float4 box; int idx, cx, cy, pad; };

// Hint: bring the 128-byte line holding p into L1 (no register result).
__device__ __forceinline__ void prefetch_l1(const void* p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// Culls 1 and 2 of a staged pair: fills candA / candB with the edges whose
// boxes meet the overlap box (self pair: candA only) and returns their
// counts through nLA / nLB (0 when the polygon boxes are disjoint).
// The per-polygon records the culls read: longest edges, flags and boxes of
// the pair's two polygons.
struct PairRecs {
    float LA, LB;
    int flagA, flagB;
    float4 boxA, boxB;
};
__device__ __forceinline__ PairRecs load_pair_recs(const PairCtx& pc,
                                                   const float4* __restrict__ polyInfo,
                                                   const float4* __restrict__ polyBox,
                                                   const int* __restrict__ polyFlags) {
    PairRecs r;
    r.LA = polyInfo[pc.a].w; r.LB = polyInfo[pc.b].w;
    r.flagA = polyFlags[pc.a]; r.flagB = polyFlags[pc.b];
    r.boxA = polyBox[pc.a]; r.boxB = polyBox[pc.b];
    return r;
}

__device__ void narrow_cull(const PairCtx& pc, const float4* ringA, const float4* ringB,
                            EdgeCand* candA, EdgeCand* candB, const PairRecs& pr,
                            int& nLAout, int& nLBout) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int nA = pc.nA, nB = pc.nB;
    const float f0x = ringA[0].x, f0y = ringA[0].y;
    const float LA = pr.LA, LB = pr.LB;
    const float m = 4e-6f + 1e-3f * LA * LB;
    // polygon boxes in A's frame.  Two well-formed polygons (extent < 0.2,
    // and a candidate pair lies within 0.4 of A's vertex 0, so nothing wraps):
    // A's box was measured in this frame by the prepass (the same FP32
    // operations as the culls below) and B's box is moved from B's frame,
    // widened by 1e-6 for the rounding of the move.
    float ox0, ox1, oy0, oy1;
    // A polygon that is not well formed (the prepass's flag 0: extent of 0.2
    // or more, or non-finite) may span more than half the box, and then
    // coordinates taken relative to A's vertex 0 no longer give every edge
    // pair its own minimum image (kernels.cuh:778-790 wraps each difference
    // separately).  Such pairs keep every edge and skip the box tests; the
    // FP32 crossing filter and the exact test wrap per edge pair.
    const bool boxes = pr.flagA && pr.flagB;
    const float kInf = __int_as_float(0x7f800000);
    if (boxes) {
        const float4 ba = pr.boxA;
        ox0 = ba.x - m; ox1 = ba.y + m; oy0 = ba.z - m; oy1 = ba.w + m;
        if (!pc.self) {
            const float4 bb = pr.boxB;
            const float sx = wrapf(ringB[0].x - f0x), sy = wrapf(ringB[0].y - f0y);
            ox0 = fmaxf(ba.x, bb.x + sx - 1e-6f) - m; ox1 = fminf(ba.y, bb.y + sx + 1e-6f) + m;
            oy0 = fmaxf(ba.z, bb.z + sy - 1e-6f) - m; oy1 = fminf(ba.w, bb.w + sy + 1e-6f) + m;
            // disjoint boxes: no edge of A (padded by m) reaches past the gap
            if (ox0 > ox1 || oy0 > oy1) { nLAout = 0; nLBout = 0; return; }
        }
    } else {
        ox0 = -kInf; ox1 = kInf; oy0 = -kInf; oy1 = kInf;
    }
    // candidate edges of each ring (edge box padded by m meets the overlap box)
    auto collect = [&](const float4* ring, int n, EdgeCand* out, float pad) -> int {
        int cnt = 0;
        for (int e0 = 0; e0 < n; e0 += 32) {
            int e = e0 + lane;
            bool ok = false;
            EdgeCand c;
            if (e < n) {
                float4 v0 = ring[e], v1 = ring[(e + 1 == n) ? 0 : e + 1];
                float x0 = wrapf(v0.x - f0x), y0 = wrapf(v0.y - f0y);
                float x1 = wrapf(v1.x - f0x), y1 = wrapf(v1.y - f0y);
                c.box = boxes ? make_float4(fminf(x0, x1) - pad, fmaxf(x0, x1) + pad,
                                            fminf(y0, y1) - pad, fmaxf(y0, y1) + pad)
                              : make_float4(-kInf, kInf, -kInf, kInf);
                c.idx = e; c.cx = __float_as_int(v0.z); c.cy = __float_as_int(v0.w); c.pad = 0;
                // keep unless certainly outside the overlap box (NaN keeps it)
                ok = !(c.box.x > ox1 || c.box.y < ox0 || c.box.z > oy1 || c.box.w < oy0);
            }
            unsigned mk = __ballot_sync(PCP_FULL, ok);
            if (ok) out[cnt + __popc(mk & lt)] = c;
            cnt += __popc(mk);
        }
        return cnt;
    };
    int nLA = collect(ringA, nA, candA, m);
    int nLB = pc.self ? 0 : collect(ringB, nB, candB, 0.f);
    __syncwarp();
    const EdgeCand* cb = pc.self ? candA : candB;
    if (pc.self) nLB = nLA;
    nLAout = nLA;
    nLBout = nLB;
}

__device__ int narrow_pair(const PairCtx& pc, const float4* ringA, const float4* ringB,
                           EdgeCand* candA, EdgeCand* candB, int* queue,
                           unsigned long long* recKey, float2* recTU, int recCap, int B,
                           const double2* __restrict__ pos, const double2* __restrict__ edgeVec,
                           const float4* __restrict__ polyInfo,
                           const float4* __restrict__ polyBox,
                           const int* __restrict__ polyFlags) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int nA = pc.nA;
    int nLA = 0, nLB = 0;
    narrow_cull(pc, ringA, ringB, candA, candB, load_pair_recs(pc, polyInfo, polyBox, polyFlags),
                nLA, nLB);
    if (nLA == 0 || nLB == 0) return 0;
    const EdgeCand* cb = pc.self ? candA : candB;
    bool wrapB = B >= 3;
    int qn = 0;
    int rec = 0;
    bool overflow = false;
    auto run_batch = [&](int cnt) {
        bool hit = false;
        unsigned long long key = 0;
        float2 tuf = make_float2(0.f, 0.f);
        if (lane < cnt) {
            int e = queue[lane];
            int ea = e & 0xFFFF, eb = (e >> 16) & 0xFFFF;
            int id1 = pc.stA + ea, nid = pc.stB + eb;
            Crossing c = cross_exact(pos[id1], edgeVec[id1], pos[nid], edgeVec[nid]);
            if (c.hit) {
                hit = true;
                if (c.denom > 0) {   // kernels.cuh:796-799, 862-867
                    key = pack_key(pc.a, pc.b, eb, ea);
                    tuf = make_float2((float)c.tt, (float)c.uu);
                } else {             // kernels.cuh:800-804, 868-873
                    key = pack_key(pc.b, pc.a, ea, eb);
                    tuf = make_float2((float)c.uu, (float)c.tt);
                }
            }
        }
        unsigned mask = __ballot_sync(PCP_FULL, hit);
        int cnt2 = __popc(mask);
        if (rec + cnt2 > recCap) { overflow = true; return; }
        if (hit) {
            int slot = rec + __popc(mask & lt);
            recKey[slot] = key;
            recTU[slot] = tuf;
        }
        rec += cnt2;
    };
    // candidate edge pairs as (aw x bw) lane tiles: lane = a * bw + b, bw the
    // power of two >= nLB (at most 32), so few-edge lists fill the warp
    int lb = 0;
    while ((1 << lb) < nLB && lb < 5) ++lb;
    const int bw = 1 << lb, aw = 32 >> lb;
    const int la = lane >> lb, lbb = lane & (bw - 1);
    for (int b0 = 0; b0 < nLB && !overflow; b0 += bw) {
        for (int a0 = 0; a0 < nLA && !overflow; a0 += aw) {
            const int ia = a0 + la, ib = b0 + lbb;
            bool ok = ia < nLA && ib < nLB;
            EdgeCand ea, eb;
            if (ok) { ea = candA[ia]; eb = cb[ib]; }
            else {
                ea.box = eb.box = make_float4(0.f, 0.f, 0.f, 0.f);
                ea.idx = eb.idx = 0; ea.cx = eb.cx = 0; ea.cy = eb.cy = 0;
            }
            if (pc.self) {
                // id1 < nid, not adjacent (kernels.cuh:766-775)
                ok = ok && eb.idx > ea.idx + 1 && !(ea.idx == 0 && eb.idx == nA - 1);
            }
            ok = ok && !(eb.box.x > ea.box.y || eb.box.y < ea.box.x ||
                         eb.box.z > ea.box.w || eb.box.w < ea.box.z);
            if (wrapB) {
                int dx = abs(ea.cx - eb.cx), dy = abs(ea.cy - eb.cy);
                ok = ok && (dx <= 1 || dx == B - 1) && (dy <= 1 || dy == B - 1);
            }
            unsigned mk = __ballot_sync(PCP_FULL, ok);
            if (mk) {
                if (ok) queue[qn + __popc(mk & lt)] = ea.idx | (eb.idx << 16);
                qn += __popc(mk);
                __syncwarp();
                if (qn >= 32) {
                    run_batch(32);
                    __syncwarp();
                    int rest = qn - 32;
                    int v = lane < rest ? queue[32 + lane] : 0;
                    __syncwarp();
                    if (lane < rest) queue[lane] = v;
                    qn = rest;
                    __syncwarp();
                }
            }
        }
    }
    if (!overflow && qn > 0) run_batch(qn);
    __syncwarp();
    return overflow ? -1 : rec;
}

// Match each crossing to its exit in the same pair (updateOutersectionsKernel,
// kernels.cuh:981-1065): among records of the reverse group (sj' = si,
// si' = sj) skip those on the same edge that are not ahead (l == i and
// t >= u), take the smallest cyclic edge distance d = (l - i) mod n_si, then
// the smallest u, then the smallest key (first in the reference's sorted
// scan).  Writes the pair's records to global memory.
// The partner (exit) of crossing `key` among a pair's R records: in the
// reverse group (sj' = si, si' = sj), skipping records on the same edge that
// are not ahead (l == i and t >= u), the smallest cyclic edge distance
// d = (l - i) mod n_si, then the smallest u, then the smallest key
// (updateOutersectionsKernel, kernels.cuh:981-1065).  -1 when there is
// none; groupSeen tells whether the reverse group has any record at all.
__device__ __forceinline__ int find_partner(const PairCtx& pc, int R,
                                            const unsigned long long* recKey,
                                            const float2* recTU, unsigned long long key,
                                            float2 tu, bool& groupSeen) {
    const int sj = (int)(key >> 48), si = (int)((key >> 32) & 0xFFFF);
    const int i = (int)((key >> 16) & 0xFFFF);
    const int ni = (si == pc.a) ? pc.nA : pc.nB;
    const float tVal = tu.y;
    const unsigned long long grp = ((unsigned long long)si << 16) | (unsigned long long)sj;
    groupSeen = false;
    int best = -1, bestD = 0;
    float bestU = 0.f;
    unsigned long long bestK = 0;
    for (int c = 0; c < R; ++c) {
        const unsigned long long kc = recKey[c];
        if ((kc >> 32) != grp) continue;
        groupSeen = true;
        const int l = (int)(kc & 0xFFFF);
        const float uVal = recTU[c].x;
        if (l == i && tVal >= uVal) continue;
        const int d = (l - i + ni) % ni;
        const bool better = best < 0 || d < bestD || (d == bestD && (uVal < bestU ||
                            (uVal == bestU && kc < bestK)));
        if (better) { best = c; bestD = d; bestU = uVal; bestK = kc; }
    }
    return best;
}

// The largest key and a record that holds it, over the warp (lanes with no
// record pass key 0).
__device__ __forceinline__ void warp_max_key(unsigned long long& k, int& pos) {
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long tk = __shfl_xor_sync(PCP_FULL, k, o);
        const int tp = __shfl_xor_sync(PCP_FULL, pos, o);
        if (tk > k) { k = tk; pos = tp; }
    }
}

// Raise ctrl->maxKey to k (held by record pos).  A warp that raised it lists
// its record, so the record holding the final maximum is in the list (the
// last raise was made by its writer); k_fixup looks it up there instead of
// scanning every record.  One call per warp of the narrow phase.
__device__ __forceinline__ void publish_max_key(Ctrl* __restrict__ ctrl, ContactWS& ws,
                                                unsigned long long k, int pos) {
    const unsigned long long old = atomicMax(&ctrl->maxKey, k);
    if (old < k) {
        const int c = atomicAdd(&ctrl->numMaxCand, 1);
        if (c < kMaxCand) ws.maxCand[c] = pos;
        else atomicOr(&ctrl->flags, kFlagCapacity);
    }
}

__device__ unsigned long long match_and_write(const PairCtx& pc, int R,
                                              const unsigned long long* recKey,
                                              const float2* recTU, Ctrl* ctrl, ContactWS& ws,
                                              int& kmaxPos) {
    const int lane = threadIdx.x & 31;
    // the slot of the pair's records: the atomic's round trip overlaps the
    // matching below, whose results wait in registers (up to 32 records,
    // one per lane, in one round; more take further rounds)
    int base = 0;
    if (lane == 0) base = atomicAdd(&ctrl->numRecords, R);
    unsigned long long kmax = 0;
    int kpos = -1;
    for (int r0 = 0; r0 < R; r0 += 32) {
        const int r = r0 + lane;
        unsigned long long key = 0, outer = 0;
        float2 tu = make_float2(0.f, 0.f), ut = make_float2(0.f, 0.f);
        bool fix = false;
        if (r < R) {
            key = recKey[r];
            tu = recTU[r];
            bool groupSeen = false;
            const int best = find_partner(pc, R, recKey, recTU, key, tu, groupSeen);
            if (best >= 0) {
                outer = recKey[best];
                ut = recTU[best];
            } else {
                outer = key;
                ut = tu;
                fix = !groupSeen;
            }
        }
        if (r0 == 0) {
            base = __shfl_sync(PCP_FULL, base, 0);
            if (base + R > ws.capRecords) {
                if (lane == 0) atomicOr(&ctrl->flags, kFlagRecordOverflow);
                return 0ull;
            }
        }
        if (r < R) {
            int g = base + r;
            if (key > kmax) { kmax = key; kpos = g; }
            ws.recKey[g] = key;
            ws.recTU[g] = tu;
            ws.recOuter[g] = outer;
            ws.recUT[g] = ut;
            if (fix) {
                int f = atomicAdd(&ctrl->numFix, 1);
                if (f < ws.capFix) ws.fixList[f] = g;
                else atomicOr(&ctrl->flags, kFlagFixOverflow);
            }
        }
    }
    // the largest key (k_fixup's partner of last resort) and its record,
    // gathered by the caller and published once per warp
    warp_max_key(kmax, kpos);
    kmaxPos = kpos;
    return kmax;
}

__device__ __forceinline__ PairCtx make_ctx(int2 pr, const int* __restrict__ start) {
    PairCtx pc;
    pc.a = pr.x; pc.b = pr.y;
    pc.stA = start[pr.x]; pc.nA = start[pr.x + 1] - pc.stA;
    pc.stB = start[pr.y]; pc.nB = start[pr.y + 1] - pc.stB;
    pc.self = pr.x == pr.y;
    return pc;
}

constexpr int kNarrowWarps = 4;
// warp path: pairs whose crossings are still being tested (see k_narrow)
constexpr int kSlots = 4;
constexpr int kSlotRecords = 32;
struct PairSlot {
    int a, b, stA, stB, nA, nB, self, q;
    int R;             // records found so far
    int outstanding;   // queued edge pairs not yet tested
    int state;         // kSlot* bits
};
constexpr int kSlotBusy = 1, kSlotDone = 2, kSlotOverflow = 4;

struct alignas(16) WarpSmem {
    float4 ring[2][2 * kFastRing];
    EdgeCand candA[kFastRing];
    EdgeCand candB[kFastRing];
    unsigned long long recKey[kSlots][kSlotRecords];
    float2 recTU[kSlots][kSlotRecords];
    int queue[64];
    PairSlot slot[kSlots];
    int defer[16];     // pairs whose crossings overflowed their slot (see narrow_pair_global)
    unsigned long long bar[2];
};
constexpr int kDefer = 16;

// a pair whose crossings overflowed its slot, for k_narrow_over
__device__ __forceinline__ void push_over(int q, Ctrl* ctrl, ContactWS& ws) {
    int s = atomicAdd(&ctrl->numOver, 1);
    if (s < ws.capPairs) ws.overList[s] = q;
    else atomicOr(&ctrl->flags, kFlagSlowOverflow);
}

__device__ __forceinline__ void push_slow(int q, Ctrl* ctrl, ContactWS& ws) {
    int s = atomicAdd(&ctrl->numSlow, 1);
    if (s < ws.capSlow) ws.slowList[s] = q;
    else atomicOr(&ctrl->flags, kFlagSlowOverflow);
}

// Conservative FP32 form of the crossing test of edges (p, p2) and (q, q2):
// false only when the FP64 test of cross_exact certainly rejects the pair.
// The FP32 coordinates are within 6e-8 of the FP64 ones, so every component
// of r = p2 - p, s = q2 - q, g = q - p is within d = 1.5e-7 of the FP64
// vector.  Both take the same minimum image while every FP32 component stays
// below 0.4999: the unwrapped difference is then within 0.4999 + 1.3e-7 of
// the integer the FP32 wrap removed, so that integer is its unique nearest
// one, which the FP64 wrap removes too (edges of polygons a large FIRE move
// scrambled reach lengths near 0.5 and still get the filter).  And
// each of denom, g x s, g x r is within E = 4 M d + 2 d^2 + 4 2^-24 M^2 of
// its FP64 value (M bounds the components).  With |denom| > E + 1e-12 the
// FP64 denominator has the same sign and passes the 1e-12 test; t <= 0 is
// then certain when (g x s) sgn < -E, t >= 1 when (g x s - denom) sgn > 2.5 E
// (monotone rounding of the FP64 division), and likewise for u.
__device__ __forceinline__ bool maybe_cross(float4 p, float4 p2, float4 q, float4 q2) {
    const float rx = wrapf(p2.x - p.x), ry = wrapf(p2.y - p.y);
    const float sx = wrapf(q2.x - q.x), sy = wrapf(q2.y - q.y);
    const float gx = wrapf(q.x - p.x), gy = wrapf(q.y - p.y);
    const float M = fmaxf(fmaxf(fmaxf(fabsf(rx), fabsf(ry)), fmaxf(fabsf(sx), fabsf(sy))),
                          fmaxf(fabsf(gx), fabsf(gy)));
    if (!(M < 0.4999f)) return true;                    // (NaN too)
    const float d = 1.5e-7f, Mb = M + d;
    const float E = 4.f * Mb * d + 2.f * d * d + 2.4e-7f * Mb * Mb;
    const float den = rx * sy - ry * sx;
    if (!(fabsf(den) > E + 1e-12f)) return true;
    const float sg = den > 0.f ? 1.f : -1.f;
    const float nt = (gx * sy - gy * sx) * sg, nu = (gx * ry - gy * rx) * sg, dd = den * sg;
    if (nt < -E || nu < -E) return false;
    if (nt - dd > 2.5f * E || nu - dd > 2.5f * E) return false;
    return true;
}

// A pair of the warp path whose crossings overflow its record slot (more
// than kSlotRecords: dense overlaps, or polygons a huge FIRE move scrambled)
// is finished by its own warp with the records in global memory: the rings
// are read from global memory (the staged copies are in use), one pass over
// the candidate edge pairs counts the crossings, one atomic reserves their
// range of the record arrays, a second pass writes them, and the partners
// are matched within that range (find_partner, L2-resident).  The same
// culls, filters and exact test as the warp path, in the same order, so the
// two passes find the same crossings.  Needs the warp's queue and candidate
// buffers free (no edge pair pending).  Returns the largest key written.
struct GlobalPairBufs {
    EdgeCand* candA;   // [kFastRing]
    EdgeCand* candB;   // [kFastRing]
    int* queue;        // [64]
};
__device__ unsigned long long narrow_pair_global(const PairCtx& pc, const GlobalPairBufs& S,
                                                 int B, const double2* __restrict__ pos,
                                                 ContactWS& ws, Ctrl* __restrict__ ctrl,
                                                 int& kmaxPos) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const float4* ringA = ws.vtx + pc.stA;
    const float4* ringB = pc.self ? ringA : ws.vtx + pc.stB;
    int nLA = 0, nLB = 0;
    narrow_cull(pc, ringA, ringB, S.candA, S.candB,
                load_pair_recs(pc, ws.polyInfo, ws.polyBox, ws.polyFlags), nLA, nLB);
    if (nLA == 0 || nLB == 0) return 0ull;
    const EdgeCand* cb = pc.self ? S.candA : S.candB;
    const bool wrapB = B >= 3;
    int lb = 0;
    while ((1 << lb) < nLB && lb < 5) ++lb;
    const int bw = 1 << lb, aw = 32 >> lb;
    const int la = lane >> lb, lbb = lane & (bw - 1);
    int base = 0, R = 0;
    for (int pass = 0; pass < 2; ++pass) {
        int found = 0, qn = 0;
        // exact test of the first cnt queued edge pairs; pass 1 writes the hits
        auto test = [&](int cnt) {
            bool hit = false;
            unsigned long long key = 0;
            float2 tuf = make_float2(0.f, 0.f);
            if (lane < cnt) {
                const int e = S.queue[lane];
                const int ea = e & 0xFFFF, eb = e >> 16;
                const int id1 = pc.stA + ea, nid = pc.stB + eb;
                Crossing c = cross_exact(pos[id1], ws.edgeVec[id1], pos[nid], ws.edgeVec[nid]);
                if (c.hit) {
                    hit = true;
                    if (c.denom > 0) {   // kernels.cuh:796-799, 862-867
                        key = pack_key(pc.a, pc.b, eb, ea);
                        tuf = make_float2((float)c.tt, (float)c.uu);
                    } else {             // kernels.cuh:800-804, 868-873
                        key = pack_key(pc.b, pc.a, ea, eb);
                        tuf = make_float2((float)c.uu, (float)c.tt);
                    }
                }
            }
            const unsigned mk = __ballot_sync(PCP_FULL, hit);
            if (pass == 1 && hit) {
                const int g = base + found + __popc(mk & lt);
                ws.recKey[g] = key;
                ws.recTU[g] = tuf;
            }
            found += __popc(mk);
            // drop the tested entries from the front of the queue
            const int rest = qn - cnt;
            const int v = lane < rest ? S.queue[cnt + lane] : 0;
            __syncwarp();
            if (lane < rest) S.queue[lane] = v;
            qn = rest;
            __syncwarp();
        };
        for (int b0 = 0; b0 < nLB; b0 += bw) {
            for (int a0 = 0; a0 < nLA; a0 += aw) {
                const int ia = a0 + la, ib = b0 + lbb;
                bool ok = ia < nLA && ib < nLB;
                EdgeCand ea, eb;
                if (ok) { ea = S.candA[ia]; eb = cb[ib]; }
                else {
                    ea.box = eb.box = make_float4(0.f, 0.f, 0.f, 0.f);
                    ea.idx = eb.idx = 0; ea.cx = eb.cx = 0; ea.cy = eb.cy = 0;
                }
                if (pc.self) ok = ok && eb.idx > ea.idx + 1 && !(ea.idx == 0 && eb.idx == pc.nA - 1);
                ok = ok && !(eb.box.x > ea.box.y || eb.box.y < ea.box.x ||
                             eb.box.z > ea.box.w || eb.box.w < ea.box.z);
                if (wrapB) {
                    const int dx = abs(ea.cx - eb.cx), dy = abs(ea.cy - eb.cy);
                    ok = ok && (dx <= 1 || dx == B - 1) && (dy <= 1 || dy == B - 1);
                }
                if (ok) {
                    const int an = (ea.idx + 1 == pc.nA) ? 0 : ea.idx + 1;
                    const int bn = (eb.idx + 1 == pc.nB) ? 0 : eb.idx + 1;
                    ok = maybe_cross(ringA[ea.idx], ringA[an], ringB[eb.idx], ringB[bn]);
                }
                const unsigned mk = __ballot_sync(PCP_FULL, ok);
                if (mk) {
                    if (ok) S.queue[qn + __popc(mk & lt)] = ea.idx | (eb.idx << 16);
                    qn += __popc(mk);
                    __syncwarp();
                    if (qn >= 32) test(32);
                }
            }
        }
        if (qn > 0) test(qn);
        if (pass == 0) {
            R = found;
            if (R == 0) return 0ull;
            if (lane == 0) base = atomicAdd(&ctrl->numRecords, R);
            base = __shfl_sync(PCP_FULL, base, 0);
            if (base + R > ws.capRecords) {
                if (lane == 0) atomicOr(&ctrl->flags, kFlagRecordOverflow);
                return 0ull;
            }
        }
    }
    __syncwarp();   // the warp's record writes before its lanes read them
    const unsigned long long* keys = ws.recKey + base;
    const float2* tus = ws.recTU + base;
    unsigned long long kmax = 0ull;
    int kpos = -1;
    for (int r = lane; r < R; r += 32) {
        const unsigned long long key = keys[r];
        const float2 tu = tus[r];
        bool groupSeen = false;
        const int best = find_partner(pc, R, keys, tus, key, tu, groupSeen);
        const int g = base + r;
        ws.recOuter[g] = best >= 0 ? keys[best] : key;
        ws.recUT[g] = best >= 0 ? tus[best] : tu;
        if (best < 0 && !groupSeen) {
            const int f = atomicAdd(&ctrl->numFix, 1);
            if (f < ws.capFix) ws.fixList[f] = g;
            else atomicOr(&ctrl->flags, kFlagFixOverflow);
        }
        if (key > kmax) { kmax = key; kpos = g; }
    }
    warp_max_key(kmax, kpos);
    kmaxPos = kpos;
    return kmax;
}

// Warp per pair (pairs claimed dynamically), rings staged by bulk copies into
// a double buffer with bounded mbarrier waits.  The FP32 culls and the FP32
// crossing test run per pair; the edge pairs they cannot reject are queued,
// tagged with their pair's slot, and go through the exact FP64 test 32 at a
// time across up to kSlots pairs, so the FP64 pipe sees full warps.  A pair
// is matched and written once its last queued edge pair has been tested.
__global__ void __launch_bounds__(32 * kNarrowWarps)
k_narrow(const double2* __restrict__ pos, const int* __restrict__ start, int B,
         ContactWS ws, Ctrl* __restrict__ ctrl, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    WarpSmem& S = reinterpret_cast<WarpSmem*>(smem_raw)[threadIdx.x / 32];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int numPairs = min(ctrl->numPairs, ws.capPairs);
    if (lane == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        fence_barrier_init();
    }
    if (lane < kSlots) S.slot[lane].state = 0;
    __syncwarp();
    uint32_t phase[2] = {0u, 0u};
    int qn_ = 0;   // queued edge pairs
    unsigned long long warpMaxKey = 0ull;
    int warpMaxPos = -1;

    // exact FP64 test of the first cnt queued edge pairs
    auto run_batch = [&](int cnt) {
        bool hit = false;
        unsigned long long key = 0;
        float2 tuf = make_float2(0.f, 0.f);
        int t = -1;
        if (lane < cnt) {
            int e = S.queue[lane];
            t = e >> 16;
            const PairSlot& sl = S.slot[t];
            if (!(sl.state & kSlotOverflow)) {
                int ea = e & 0xFF, eb = (e >> 8) & 0xFF;
                int id1 = sl.stA + ea, nid = sl.stB + eb;
                Crossing c = cross_exact(pos[id1], ws.edgeVec[id1], pos[nid], ws.edgeVec[nid]);
                if (c.hit) {
                    hit = true;
                    if (c.denom > 0) {   // kernels.cuh:796-799, 862-867
                        key = pack_key(sl.a, sl.b, eb, ea);
                        tuf = make_float2((float)c.tt, (float)c.uu);
                    } else {             // kernels.cuh:800-804, 868-873
                        key = pack_key(sl.b, sl.a, ea, eb);
                        tuf = make_float2((float)c.uu, (float)c.tt);
                    }
                }
            }
        }
        for (int k = 0; k < kSlots; ++k) {
            unsigned me = __ballot_sync(PCP_FULL, t == k);
            if (!me) continue;
            unsigned mh = __ballot_sync(PCP_FULL, hit && t == k);
            int R0 = S.slot[k].R;
            if (hit && t == k) {
                int at = R0 + __popc(mh & lt);
                if (at < kSlotRecords) { S.recKey[k][at] = key; S.recTU[k][at] = tuf; }
            }
            __syncwarp();
            if (lane == 0) {
                S.slot[k].R = R0 + __popc(mh);
                if (R0 + __popc(mh) > kSlotRecords) S.slot[k].state |= kSlotOverflow;
                S.slot[k].outstanding -= __popc(me);
            }
            __syncwarp();
        }
        // drop the tested entries from the front of the queue
        int rest = qn_ - cnt;
        int v = lane < rest ? S.queue[cnt + lane] : 0;
        __syncwarp();
        if (lane < rest) S.queue[lane] = v;
        qn_ = rest;
        __syncwarp();
    };
    // match and write (or defer, when its records overflowed the slot) every
    // slot whose pair is enumerated and fully tested
    int nDefer = 0;
    auto finalize_ready = [&]() {
        for (int k = 0; k < kSlots; ++k) {
            const int st = S.slot[k].state;
            if ((st & kSlotBusy) && (st & kSlotDone) && S.slot[k].outstanding == 0) {
                const PairSlot sl = S.slot[k];
                if (sl.state & kSlotOverflow) {
                    if (nDefer < kDefer) {
                        if (lane == 0) S.defer[nDefer] = sl.q;
                        ++nDefer;
                    } else if (lane == 0) {
                        push_over(sl.q, ctrl, ws);
                    }
                } else if (sl.R > 0) {
                    PairCtx pc;
                    pc.a = sl.a; pc.b = sl.b; pc.stA = sl.stA; pc.stB = sl.stB;
                    pc.nA = sl.nA; pc.nB = sl.nB; pc.self = sl.self != 0;
                    int kp = -1;
                    const unsigned long long km =
                        match_and_write(pc, sl.R, S.recKey[k], S.recTU[k], ctrl, ws, kp);
                    if (km > warpMaxKey) { warpMaxKey = km; warpMaxPos = kp; }
                }
                __syncwarp();
                if (lane == 0) S.slot[k].state = 0;
                __syncwarp();
            }
        }
    };
    auto free_slot = [&]() -> int {
        for (int k = 0; k < kSlots; ++k)
            if (!(S.slot[k].state & kSlotBusy)) return k;
        return -1;
    };
    // finish every pending edge pair and slot, then the deferred pairs (they
    // take the queue and candidate buffers, which are then free)
    auto run_deferred = [&]() {
        if (qn_ > 0) run_batch(qn_);
        finalize_ready();
        for (int d = 0; d < nDefer; ++d) {
            const int qd = S.defer[d];
            int kp = -1;
            const unsigned long long km =
                narrow_pair_global(make_ctx(ws.pairs[qd], start),
                                   GlobalPairBufs{S.candA, S.candB, S.queue}, B, pos, ws, ctrl, kp);
            if (km > warpMaxKey) { warpMaxKey = km; warpMaxPos = kp; }
        }
        nDefer = 0;
        __syncwarp();
    };

    // pairs claimed one at a time from a shared cursor, the next one while
    // the current one is processed: warps whose blocks became resident
    // late (beside another kernel of the step) take fewer pairs
    auto claim = [&]() -> int {
        int v = 0;
        if (lane == 0) v = atomicAdd(&ctrl->pairCursor, 1);
        return __shfl_sync(PCP_FULL, v, 0);
    };
    int q = claim();
    // the culls' per-polygon records, loaded into registers one pair ahead:
    // lanes 0/1 polyInfo of a/b, 2/3 polyBox of a/b, 4/5 polyFlags of a/b
    auto issue = [&](int qq, int stage, float4& rec) -> bool {
        // returns true when a copy was issued for pair qq into `stage`
        if (qq >= numPairs) return false;
        PairCtx pc = make_ctx(ws.pairs[qq], start);
        if (pc.nA > kFastRing || pc.nB > kFastRing || pc.nA < 3 || pc.nB < 3) return false;
        if (lane < 6) {
            const int pp = (lane & 1) ? pc.b : pc.a;
            rec = lane < 2 ? ws.polyInfo[pp]
                : lane < 4 ? ws.polyBox[pp]
                           : make_float4(__int_as_float(ws.polyFlags[pp]), 0.f, 0.f, 0.f);
        }
        if (lane == 0) {
            // order this warp's earlier generic reads of the buffer before the
            // async-proxy writes that refill it
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            uint32_t bytesA = 16u * (uint32_t)pc.nA;
            uint32_t bytesB = pc.self ? 0u : 16u * (uint32_t)pc.nB;
            mbar_arrive_expect(&S.bar[stage], bytesA + bytesB);
            bulk_g2s(&S.ring[stage][0], ws.vtx + pc.stA, bytesA, &S.bar[stage]);
            if (!pc.self) bulk_g2s(&S.ring[stage][kFastRing], ws.vtx + pc.stB, bytesB, &S.bar[stage]);
        }
        // the FP64 rings of the exact test into L1 while the current pair is
        // processed (lines of 8 vertices)
        if (lane >= 8 && lane < 24) {
            const int k = lane & 7;                  // line k of a ring (8 vertices of 16 B)
            const bool ringB = lane >= 16;
            const int st0 = ringB ? pc.stB : pc.stA, n0 = ringB ? pc.nB : pc.nA;
            if (8 * k < n0 && !(ringB && pc.self)) {
                prefetch_l1(pos + st0 + 8 * k);
                prefetch_l1(ws.edgeVec + st0 + 8 * k);
            }
        }
        return true;
    };
    const bool wrapB = B >= 3;
    int stage = 0;
    float4 recCur = make_float4(0.f, 0.f, 0.f, 0.f);
    bool inflight = issue(q, stage, recCur);
    while (q < numPairs) {
        const int qn = claim();
        PairCtx pc = make_ctx(ws.pairs[q], start);
        if (!inflight) {
            // too large (or degenerate) for the warp path: hand to the block path
            if (lane == 0 && pc.nA >= 1 && pc.nB >= 1) push_slow(q, ctrl, ws);
            inflight = issue(qn, stage, recCur);
            q = qn;
            continue;
        }
        // prefetch the next pair into the other buffer while this one is processed
        int other = stage ^ 1;
        float4 recNext = recCur;
        bool nextInflight = issue(qn, other, recNext);
        if (!mbar_wait_bounded(&S.bar[stage], phase[stage], ctrl)) {
            // the copy never landed: wait (bounded) for the prefetch too, then stop
            if (nextInflight) mbar_wait_bounded(&S.bar[other], phase[other], ctrl);
            return;
        }
        phase[stage] ^= 1u;
        // a slot for this pair (test what is queued when all are taken)
        int t = free_slot();
        if (t < 0) {
            if (qn_ > 0) run_batch(qn_);
            finalize_ready();
            t = free_slot();
        }
        if (lane == 0) {
            PairSlot& sl = S.slot[t];
            sl.a = pc.a; sl.b = pc.b; sl.stA = pc.stA; sl.stB = pc.stB;
            sl.nA = pc.nA; sl.nB = pc.nB; sl.self = pc.self ? 1 : 0; sl.q = q;
            sl.R = 0; sl.outstanding = 0; sl.state = kSlotBusy;
        }
        __syncwarp();
        const float4* ringA = &S.ring[stage][0];
        const float4* ringB = pc.self ? ringA : &S.ring[stage][kFastRing];
        int nLA = 0, nLB = 0;
        PairRecs pr;
        pr.LA = __shfl_sync(PCP_FULL, recCur.w, 0);
        pr.LB = __shfl_sync(PCP_FULL, recCur.w, 1);
        pr.boxA = make_float4(__shfl_sync(PCP_FULL, recCur.x, 2), __shfl_sync(PCP_FULL, recCur.y, 2),
                              __shfl_sync(PCP_FULL, recCur.z, 2), __shfl_sync(PCP_FULL, recCur.w, 2));
        pr.boxB = make_float4(__shfl_sync(PCP_FULL, recCur.x, 3), __shfl_sync(PCP_FULL, recCur.y, 3),
                              __shfl_sync(PCP_FULL, recCur.z, 3), __shfl_sync(PCP_FULL, recCur.w, 3));
        pr.flagA = __float_as_int(__shfl_sync(PCP_FULL, recCur.x, 4));
        pr.flagB = __float_as_int(__shfl_sync(PCP_FULL, recCur.x, 5));
        narrow_cull(pc, ringA, ringB, S.candA, S.candB, pr, nLA, nLB);
        const EdgeCand* cb = pc.self ? S.candA : S.candB;
        const int nA = pc.nA, nB = pc.nB;
        // candidate edge pairs as (aw x bw) lane tiles: lane = a * bw + b
        int lb = 0;
        while ((1 << lb) < nLB && lb < 5) ++lb;
        const int bw = 1 << lb, aw = 32 >> lb;
        const int la = lane >> lb, lbb = lane & (bw - 1);
        for (int b0 = 0; b0 < nLB; b0 += bw) {
            for (int a0 = 0; a0 < nLA; a0 += aw) {
                const int ia = a0 + la, ib = b0 + lbb;
                bool ok = ia < nLA && ib < nLB;
                EdgeCand ea, eb;
                if (ok) { ea = S.candA[ia]; eb = cb[ib]; }
                else {
                    ea.box = eb.box = make_float4(0.f, 0.f, 0.f, 0.f);
                    ea.idx = eb.idx = 0; ea.cx = eb.cx = 0; ea.cy = eb.cy = 0;
                }
                if (pc.self) {
                    // id1 < nid, not adjacent (kernels.cuh:766-775)
                    ok = ok && eb.idx > ea.idx + 1 && !(ea.idx == 0 && eb.idx == nA - 1);
                }
                ok = ok && !(eb.box.x > ea.box.y || eb.box.y < ea.box.x ||
                             eb.box.z > ea.box.w || eb.box.w < ea.box.z);
                if (wrapB) {
                    int dx = abs(ea.cx - eb.cx), dy = abs(ea.cy - eb.cy);
                    ok = ok && (dx <= 1 || dx == B - 1) && (dy <= 1 || dy == B - 1);
                }
                if (ok) {
                    const int an = (ea.idx + 1 == nA) ? 0 : ea.idx + 1;
                    const int bn = (eb.idx + 1 == nB) ? 0 : eb.idx + 1;
                    ok = maybe_cross(ringA[ea.idx], ringA[an], ringB[eb.idx], ringB[bn]);
                }
                unsigned mk = __ballot_sync(PCP_FULL, ok);
                if (mk) {
                    if (ok) S.queue[qn_ + __popc(mk & lt)] = ea.idx | (eb.idx << 8) | (t << 16);
                    if (lane == 0) S.slot[t].outstanding += __popc(mk);
                    qn_ += __popc(mk);
                    __syncwarp();
                    if (qn_ >= 32) {
                        run_batch(32);
                        finalize_ready();   // other pairs may be complete now
                    }
                }
            }
        }
        if (lane == 0) S.slot[t].state |= kSlotDone;
        __syncwarp();
        finalize_ready();
        stage = other;
        inflight = nextInflight;
        recCur = recNext;
        q = qn;
    }
    run_deferred();
    if (lane == 0 && warpMaxKey) publish_max_key(ctrl, ws, warpMaxKey, warpMaxPos);
}

// Pairs whose crossings overflowed their warp's record slot when that warp's
// own deferred list was full (a FIRE step that scrambled the polygons makes
// nearly every pair such a pair): one warp per pair, records straight to
// the global arrays (narrow_pair_global), pairs claimed from a cursor.
constexpr int kOverWarps = 4;
struct alignas(16) OverSmem {
    EdgeCand candA[kFastRing];
    EdgeCand candB[kFastRing];
    int queue[64];
};
__global__ void __launch_bounds__(32 * kOverWarps)
k_narrow_over(const double2* __restrict__ pos, const int* __restrict__ start, int B,
              ContactWS ws, Ctrl* __restrict__ ctrl, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    __shared__ OverSmem sm[kOverWarps];
    OverSmem& S = sm[threadIdx.x / 32];
    const int lane = threadIdx.x & 31;
    const int numOver = min(ctrl->numOver, ws.capPairs);
    unsigned long long warpMaxKey = 0ull;
    int warpMaxPos = -1;
    for (;;) {
        int i = 0;
        if (lane == 0) i = atomicAdd(&ctrl->overCursor, 1);
        i = __shfl_sync(PCP_FULL, i, 0);
        if (i >= numOver) break;
        int kp = -1;
        const unsigned long long km =
            narrow_pair_global(make_ctx(ws.pairs[ws.overList[i]], start),
                               GlobalPairBufs{S.candA, S.candB, S.queue}, B, pos, ws, ctrl, kp);
        if (km > warpMaxKey) { warpMaxKey = km; warpMaxPos = kp; }
    }
    if (lane == 0 && warpMaxKey) publish_max_key(ctrl, ws, warpMaxKey, warpMaxPos);
}

// Block path: one warp per block, rings loaded with plain loads into a large
// dynamic shared-memory area; for polygons above kFastRing vertices and for
// pairs with more than kFastRecords crossings.
__global__ void __launch_bounds__(32)
k_narrow_slow(const double2* __restrict__ pos, const int* __restrict__ start, int B,
              ContactWS ws, Ctrl* __restrict__ ctrl, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    // k_narrow has finished claiming: its cursor back to 0 for a rerun of
    // the narrow phase alone
    if (blockIdx.x == 0 && threadIdx.x == 0) ctrl->pairCursor = 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float4* ring = reinterpret_cast<float4*>(smem_raw);                    // kSlowRing
    EdgeCand* cand = reinterpret_cast<EdgeCand*>(ring + kSlowRing);          // kSlowRing
    unsigned long long* recKey = reinterpret_cast<unsigned long long*>(cand + kSlowRing);
    float2* recTU = reinterpret_cast<float2*>(recKey + kSlowRecords);
    int* queue = reinterpret_cast<int*>(recTU + kSlowRecords);
    const int lane = threadIdx.x & 31;
    int numSlow = min(ctrl->numSlow, ws.capSlow);
    unsigned long long warpMaxKey = 0ull;
    int warpMaxPos = -1;
    for (;;) {
        int s = 0;
        if (lane == 0) s = atomicAdd(&ctrl->slowCursor, 1);
        s = __shfl_sync(PCP_FULL, s, 0);
        if (s >= numSlow) break;
        int q = ws.slowList[s];
        PairCtx pc = make_ctx(ws.pairs[q], start);
        int tot = pc.self ? pc.nA : pc.nA + pc.nB;
        if (pc.nA < 1 || pc.nB < 1) continue;
        if (tot > kSlowRing || pc.nA > 65535 || pc.nB > 65535) {
            if (lane == 0) atomicOr(&ctrl->flags, kFlagCapacity);
            continue;
        }
        for (int t = lane; t < pc.nA; t += 32) ring[t] = ws.vtx[pc.stA + t];
        if (!pc.self)
            for (int t = lane; t < pc.nB; t += 32) ring[pc.nA + t] = ws.vtx[pc.stB + t];
        __syncwarp();
        const float4* ringB = pc.self ? ring : ring + pc.nA;
        // the two candidate lists share one buffer: A from the front, B behind it
        int R = narrow_pair(pc, ring, ringB, cand, cand + pc.nA, queue, recKey, recTU,
                            kSlowRecords, B, pos, ws.edgeVec, ws.polyInfo, ws.polyBox,
                            ws.polyFlags);
        if (R < 0) {
            if (lane == 0) atomicOr(&ctrl->flags, kFlagCapacity);
        } else if (R > 0) {
            int kp = -1;
            const unsigned long long km = match_and_write(pc, R, recKey, recTU, ctrl, ws, kp);
            if (km > warpMaxKey) { warpMaxKey = km; warpMaxPos = kp; }
        }
        __syncwarp();
    }
    if (lane == 0 && warpMaxKey) publish_max_key(ctrl, ws, warpMaxKey, warpMaxPos);
}

// A crossing whose reverse group is empty: the reference's binary search
// (kernels.cuh:993-1000) stops at the last record when every key is below
// sij, and that record is then tried as the partner.  Reproduced here, once
// every record is written (the kernel after the narrow phase): each block
// finds the record holding the largest key among the few that raised it
// (publish_max_key), then the fix list is dealt out over the grid.
__global__ void __launch_bounds__(256)
k_fixup(ContactWS ws, Ctrl* __restrict__ ctrl, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    const int nf = min(ctrl->numFix, ws.capFix);
    if (nf == 0) return;
    const int I = min(ctrl->numRecords, ws.capRecords);
    const int nc = min(ctrl->numMaxCand, kMaxCand);
    const unsigned long long kmax = ctrl->maxKey;
    __shared__ int s_mi;
    if (threadIdx.x == 0) s_mi = -1;
    __syncthreads();
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int g = ws.maxCand[c];
        if (g >= 0 && g < I && ws.recKey[g] == kmax) s_mi = g;   // keys are unique
    }
    __syncthreads();
    const int mi = s_mi;
    if (mi < 0) return;
    const float2 tuMax = ws.recTU[mi];
    const int l = (int)(kmax & 0xFFFF);
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        const int g = ws.fixList[f];
        const unsigned long long key = ws.recKey[g];
        const int sj = (int)(key >> 48), si = (int)((key >> 32) & 0xFFFF);
        const int i = (int)((key >> 16) & 0xFFFF);
        const unsigned long long sij = ((unsigned long long)si << 48) | ((unsigned long long)sj << 32);
        if (!(sij > kmax)) continue;
        if (l == i && ws.recTU[g].y >= tuMax.x) continue;
        ws.recOuter[g] = kmax;
        ws.recUT[g] = tuMax;
    }
}

// ---------------------------------------------------------------- force ----
__device__ __forceinline__ void add_f(double2* F, int v, double fx, double fy) {
    double* f = reinterpret_cast<double*>(F) + 2 * (size_t)v;
    atomicAdd(f, fx);
    atomicAdd(f + 1, fy);
}

// updateForceEnergyExteriorKernel (kernels.cuh:1067-1273) and, per record,
// the interior chain of updateForceEnergyInteriorKernel (kernels.cuh:
// 1354-1424): whole edges of si strictly between the entry edge i and the
// exit edge l, each taken relative to the record's own entry point.
//
// GB300's FP64 pipe charges a warp instruction whatever its active lanes, so
// the work is cut into lane-sized pieces: a warp takes kForceRecs records;
// the exterior part of each record is split over a lane pair (one gDf per
// lane), then the interior-chain edges of all of the warp's records are
// dealt out one per lane.  Small blocks spread the few thousand warps over
// every SM.
constexpr int kForceRecs = 16;
constexpr int kForceWarps = 2;

// kEdge: the edge vectors wrap(x_next - x) of the current positions are
// given in `edge` (the FIRE step computes them beside the contact search), so
// the kernel loads them instead of forming them (bit-identical values).
template <bool kEdge>
__global__ void __launch_bounds__(32 * kForceWarps)
k_overlap_force(const double2* __restrict__ pos, const int* __restrict__ start,
                int V, ContactWS ws, Ctrl* __restrict__ ctrl,
                double2* __restrict__ force, const double2* __restrict__ edge, int decide,
                cudaGraphConditionalHandle rbCond, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    const int lane = threadIdx.x & 31;
    const int half = lane & 1;
    const int I = min(ctrl->numRecords, ws.capRecords);
    const int warpsTotal = gridDim.x * kForceWarps;
    double eLocal = 0.0;
    for (int base = (blockIdx.x * kForceWarps + (threadIdx.x >> 5)) * kForceRecs; base < I;
         base += warpsTotal * kForceRecs) {
        const int r = base + (lane >> 1);
        bool valid = r < I;
        // load 1: the record (keys and both crossing parameters)
        unsigned long long inter = 0, outer = 0;
        float tRec = 0.f, uRec = 0.f;
        if (valid) {
            inter = ws.recKey[r]; outer = ws.recOuter[r];
            tRec = ws.recTU[r].y; uRec = ws.recUT[r].y;
        }
        valid = valid && inter != outer;
        // load 2: both polygons' vertex ranges.  The topology is the CSR
        // one (next = the following vertex of the polygon, cyclic), so every
        // vertex index below is formed without reading `next`.
        int start1 = 0, n1 = 0, iLoc = 0, lLoc = 0, lDist = 0;
        int a = 0, za = 0, v0 = 0, v1 = 0, v2 = 0, v3 = 0;
        bool same = false;
        if (valid) {
            const int s1 = (int)((inter >> 32) & 0xFFFF), s2 = (int)(inter >> 48);
            iLoc = (int)((inter >> 16) & 0xFFFF);
            const int jLoc = (int)(inter & 0xFFFF);
            const int kLoc = (int)((outer >> 16) & 0xFFFF);
            lLoc = (int)(outer & 0xFFFF);
            start1 = start[s1];
            const int end1 = start[s1 + 1];
            const int start2 = start[s2], end2 = start[s2 + 1];
            n1 = end1 - start1;
            const int n2 = end2 - start2;
            const int i = start1 + iLoc, j = start2 + jLoc, k = start2 + kLoc, l = start1 + lLoc;
            if (i >= V || j >= V || k >= V || l >= V || iLoc >= n1 || lLoc >= n1 || jLoc >= n2 ||
                kLoc >= n2) {
                if (half == 0) atomicOr(&ctrl->flags, kFlagNonFinite);
                valid = false;
                n1 = 0;
            } else {
                auto nx1 = [&](int loc) { return start1 + (loc + 1 == n1 ? 0 : loc + 1); };
                auto nx2 = [&](int loc) { return start2 + (loc + 1 == n2 ? 0 : loc + 1); };
                // Both lanes of the pair run one h/g12 and one gDf on operands
                // chosen by parity (no divergent branches):
                //   i == l : h(fij, fkl); even: gDf(i, zi, j, zj) . g1,
                //            odd: gDf(k, zk, i, zi) . g2; energy once
                //   i != l : even: h(fij, zi), gDf(i, zi, j, zj) . g1, zi += g2;
                //            odd: h(l, fkl), gDf(k, zk, l, zl) . g2, l += g1
                same = (i == l);
                a = half ? k : i;                        // this lane's edge (a, za)
                za = half ? nx2(kLoc) : nx1(iLoc);
                v0 = a; v1 = za;
                if (half == 0) { v2 = j; v3 = nx2(jLoc); }
                else if (same) { v2 = i; v3 = nx1(iLoc); }
                else { v2 = l; v3 = nx1(lLoc); }
            }
        }
        // load 3: the vertices.  The crossing points: the even lane of the
        // pair takes f_ij on edge (i, zi), the odd one f_kl on edge (k, zk),
        // and they swap them.
        double2 pa = make_double2(0.0, 0.0), pza = pa, ra = pa, fa = pa, q2 = pa, d3 = pa;
        double2 sp = make_double2(0.0, 0.0);
        if (valid) {
            pa = pos[a];
            pza = pos[za];
            q2 = pos[v2];
            if (kEdge) { ra = edge[a]; d3 = edge[v2]; }
            else {
                const double2 q3 = pos[v3];
                ra = make_double2(wrap(pza.x - pa.x), wrap(pza.y - pa.y));
                d3 = make_double2(wrap(q3.x - q2.x), wrap(q3.y - q2.y));
            }
            const double ta = f2d_int(half ? uRec : tRec);
            fa = make_double2(wrap(pa.x + ta * ra.x), wrap(pa.y + ta * ra.y));
        }
        const double2 fo = make_double2(__shfl_xor_sync(PCP_FULL, fa.x, 1),
                                        __shfl_xor_sync(PCP_FULL, fa.y, 1));
        if (valid) {
            const double2 fij = half ? fo : fa, fkl = half ? fa : fo;
            sp = fij;
            double2 hA = (!same && half) ? q2 : fij;
            double2 hB = (same || half) ? fkl : pza;
            double dyg, sx;
            double eh = h_parts(hA, hB, sp, dyg, sx);
            if (!same || half == 0) eLocal += eh;
            // gDf is linear in g: with -g it gives the force terms directly
            // (g1 = (dyg, -sx) on the even lane, g2 = (dyg, sx) on the odd
            // one; x1 = g2 moves zi, x2 = g1 moves l)
            const double ndy = neg_int(dyg), nsx = neg_int(sx);
            const double2 ng = make_double2(ndy, half ? nsx : sx);
            const double2 nx1v = (!same && !half) ? make_double2(ndy, nsx) : make_double2(0.0, 0.0);
            const double2 nx2v = (!same && half) ? make_double2(ndy, sx) : make_double2(0.0, 0.0);
            double2 o[4];
            // (a, za) is this lane's own edge; (v2, v3) the other one
            gDf_dd(pa, ra, q2, d3, ng, o);
            add_f(force, v0, o[0].x, o[0].y);
            add_f(force, v1, o[1].x + nx1v.x, o[1].y + nx1v.y);
            add_f(force, v2, o[2].x + nx2v.x, o[2].y + nx2v.y);
            add_f(force, v3, o[3].x, o[3].y);
            if (n1 > 0) lDist = ((lLoc - iLoc) % n1 + n1) % n1;
        }
        // interior chains: the even lane of each pair owns its record's chain
        int cnt = (valid && half == 0 && lDist > 1) ? lDist - 1 : 0;
        int incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int t = __shfl_up_sync(PCP_FULL, incl, d);
            if (lane >= d) incl += t;
        }
        const int total = __shfl_sync(PCP_FULL, incl, 31);
        // rounds of 32 chain edges, one per lane; the vertices of the next
        // round are fetched before this round's arithmetic
        struct ChainItem {
            double2 pm, pn, sp;      // pn: the edge vector when kEdge
            int mv, nv;
            bool live;
        };
        auto fetch = [&](int b) -> ChainItem {
            ChainItem c;
            const int item = b + lane;
            // owner = first lane whose inclusive count exceeds item
            int own = 0;
#pragma unroll
            for (int w = 16; w > 0; w >>= 1) {
                int v = __shfl_sync(PCP_FULL, incl, own + w - 1);
                if (v <= item) own += w;
            }
            const int oIncl = __shfl_sync(PCP_FULL, incl, own);
            const int oCnt = __shfl_sync(PCP_FULL, cnt, own);
            const int oStart = __shfl_sync(PCP_FULL, start1, own);
            const int oN = __shfl_sync(PCP_FULL, n1, own);
            const int oI = __shfl_sync(PCP_FULL, iLoc, own);
            c.sp = make_double2(__shfl_sync(PCP_FULL, sp.x, own), __shfl_sync(PCP_FULL, sp.y, own));
            c.live = item < total;
            c.mv = 0; c.nv = 0;
            c.pm = c.pn = make_double2(0.0, 0.0);
            if (c.live) {
                int mLoc = oI + item - (oIncl - oCnt) + 1;
                if (mLoc >= oN) mLoc -= oN;
                c.mv = oStart + mLoc;
                c.nv = oStart + (mLoc + 1 == oN ? 0 : mLoc + 1);   // next[mv]
                c.pm = pos[c.mv];
                c.pn = kEdge ? edge[c.mv] : pos[c.nv];
            }
            return c;
        };
        if (total > 0) {
            ChainItem cur = fetch(0);
            for (int b = 0; b < total; b += 32) {
                ChainItem nxt = cur;
                if (b + 32 < total) nxt = fetch(b + 32);
                if (cur.live) {
                    double dyg, sx;
                    if (kEdge) {
                        dyg = cur.pn.y;
                        eLocal += h_parts_edge(cur.pm, cur.pn, cur.sp, sx);
                    } else {
                        eLocal += h_parts(cur.pm, cur.pn, cur.sp, dyg, sx);
                    }
                    const double ndy = neg_int(dyg);
                    add_f(force, cur.mv, ndy, sx);             // -g1
                    add_f(force, cur.nv, ndy, neg_int(sx));    // -g2
                }
                cur = nxt;
            }
        }
    }
    eLocal = warp_sum(eLocal);
    if (lane == 0 && eLocal != 0.0) atomicAdd(&ctrl->energy, eLocal / 2.0);
    if (decide) {
        // the FIRE step's force pass: the last block to finish decides the
        // energy rollback, so that the rollback body can start beside the
        // projection
        if (lane == 0) __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            const unsigned int t = atomicAdd(&ctrl->forceTicket, 1u);
            if (t == gridDim.x - 1) {
                __threadfence();
                (void)fire_decide(ctrl, true, rbCond, 1);
            }
        }
    }
}

// ------------------------------------------------------------ launchers ----
static const size_t kSlowSmem = (size_t)kSlowRing * (16 + 32) + (size_t)kSlowRecords * 16 + 64 * 4;

// Opt the narrow-phase kernels into their shared-memory sizes; called once
// per process before any launch or graph capture.
cudaError_t contacts_init() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_narrow, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(WarpSmem) * kNarrowWarps));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_narrow_slow, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kSlowSmem);
    if (e != cudaSuccess) return e;
    done = true;
    return cudaSuccess;
}

cudaError_t launch_contacts(const double2* pos, const int* start, const int* shapeId,
                            const int* cellLocation, int P, int V, int B, ContactWS& ws,
                            Ctrl* ctrl, const int* gate, cudaStream_t st, int stages,
                            int* cellOut) {
    // stages: bit 0 = reset + prepass + broad phase, bit 1 = narrow phase,
    // bit 2 = the counters were reset by the caller's kernel (no reset)
    (void)shapeId; (void)V;
    if (B < 1) B = 1;
    if (stages & 1) {
    if (!(stages & 4)) launch_k(k_reset_contacts, dim3(1), dim3(64), 0, st, ctrl, gate);
    if (P <= 0) return cudaGetLastError();
    if (!(stages & kContactsNoPrepass)) {
        FireMove none = {};
        launch_k(k_prepass, dim3(nblocks(P, 8)), dim3(256), 0, st, const_cast<double2*>(pos), start,
                 cellLocation, cellOut, P, B, ws.edgeVec, ws.vtx, ws.polyInfo, ws.polyBox,
                 ws.polyFlags, ctrl, none, gate);
    }
    if (P <= kFusedMaxPolys) {
        launch_k(k_grid_fused, dim3(1), dim3(1024), 0, st, ws.polyInfo, ws.polyFlags, P,
                 ws.gridCount, ws.gridStart, ws.sortedPoly, ctrl, gate);
    } else {
        launch_k(k_grid_count, dim3(nblocks(P, 256)), dim3(256), 0, st, ws.polyInfo, ws.polyFlags, P, ws.gridCount,
                                                      ctrl, gate);
        launch_k(k_grid_scan, dim3(1), dim3(1024), 0, st, ws.gridCount, ws.gridStart, ws.gridFill, ctrl, gate);
        launch_k(k_grid_scatter, dim3(nblocks(P, 256)), dim3(256), 0, st, ws.polyInfo, ws.polyFlags, P, ws.gridStart,
                                                        ws.gridFill, ws.sortedPoly, ctrl, gate);
    }
    launch_k(k_candidates, dim3(nblocks(P, 8)), dim3(256), 0, st, ws.polyInfo, ws.polyBox, ws.polyFlags, start, P,
                                                  ws.gridStart, ws.sortedPoly, ws.pairs,
                                                  ws.capPairs, ctrl, gate);
    }
    if ((stages & 2) && P > 0) {
        size_t smem = sizeof(WarpSmem) * kNarrowWarps;
        int grid = ws.narrowBlocks > 0 ? ws.narrowBlocks : sm_count() * 4;
        launch_k(k_narrow, dim3(grid), dim3(32 * kNarrowWarps), smem, st, pos, start, B, ws, ctrl, gate);
        // usually empty: launched after the narrow phase has finished, so that
        // its blocks do not sit on the SMs beside it (and beside SHAKE)
        launch_k_serial(k_narrow_over, dim3(sm_count() * 4), dim3(32 * kOverWarps), 0, st, pos,
                        start, B, ws, ctrl, gate);
        // pairs for the block path are rare: a few blocks take them in turn
        launch_k(k_narrow_slow, dim3(16), dim3(32), kSlowSmem, st, pos, start, B, ws, ctrl, gate);
        launch_k(k_fixup, dim3(sm_count()), dim3(256), 0, st, ws, ctrl, gate);
    }
    return cudaGetLastError();
}

cudaError_t launch_prepass_move(double2* verlet, const int* start, int* cellOut, int P, int B,
                                ContactWS& ws, Ctrl* ctrl, const int* gate, cudaStream_t st,
                                const FireMove& mv) {
    if (B < 1) B = 1;
    if (P <= 0) return cudaSuccess;
    launch_k(k_prepass, dim3(nblocks(P, 8)), dim3(256), 0, st, verlet, start,
             static_cast<const int*>(nullptr), cellOut, P, B, ws.edgeVec, ws.vtx, ws.polyInfo,
             ws.polyBox, ws.polyFlags, ctrl, mv, gate);
    return cudaGetLastError();
}


cudaError_t launch_overlap_force(const double2* pos, const int* start,
                                 int V, ContactWS& ws, Ctrl* ctrl, double2* force,
                                 const int* gate, cudaStream_t st, const double2* edge,
                                 int decide, cudaGraphConditionalHandle rbCond) {
    // one pass over up to 4 * SMs * kForceWarps * kForceRecs records (a
    // smaller grid loops over the records)
    int grid = ws.forceBlocks > 0 ? ws.forceBlocks : sm_count() * 4;
    if (edge)
        launch_k(k_overlap_force<true>, dim3(grid), dim3(32 * kForceWarps), 0, st, pos, start, V, ws,
                 ctrl, force, edge, decide, rbCond, gate);
    else
        launch_k(k_overlap_force<false>, dim3(grid), dim3(32 * kForceWarps), 0, st, pos, start, V, ws,
                 ctrl, force, edge, decide, rbCond, gate);
    return cudaGetLastError();
}

}  // namespace pcp
