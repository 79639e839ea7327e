// gradient.cu -- overlap energy with its exact gradient (sm_103a).
//
// The reference's overlap energy (kernels.cuh:1067-1424) is, for every
// crossing record k with an exit partner, half the sum of h over the chain
// of segments inside the other polygon,
//     f1 -> p(i+1) -> ... -> p(l) -> f2      (i != l)     or   f1 -> f2  (i == l)
// where f1 = f_ij is where record k enters, f2 = f_kl where its partner
// leaves, and every h takes f1 as its start point s:
//     h(a, b, s) = (wrap(a.x - s.x) + wrap(b.x - s.x)) * dy,  dy = wrap(b.y - a.y).
// The reference's force is -sum (g1 . da + g2 . db) with s held fixed and
// without the 1/2 (g12, kernels.cuh:148-159): it is not the gradient of that
// energy.  This kernel evaluates, per record, either
//   mode kRefForce: the reference's force and energy (f1, f2 from the
//     float-rounded crossing parameters of the records), a second, plain
//     implementation of what k_overlap_force computes; or
//   mode kExactGrad: the energy with f1, f2 at the exact crossing points and
//     its exact gradient: 1/2 sum (g1 . da + g2 . db + gs . df1) with
//     gs = dh/ds = (-2 dy, 0); da, db, df1 are the identity for a vertex and
//     the crossing-point Jacobian (getDf, kernels.cuh:161-222) for f1, f2.
// The float rounding of the crossing parameters (kernels.cuh:857-858) makes
// the reference's energy a staircase at the 1e-8 level, so only the exact
// mode has a gradient that finite differences can confirm.
//
// One thread per record; each walks its chain.  Atomics add the per-vertex
// terms (this is the autograd path, not the FIRE step's hot path).
#include "pcp_common.cuh"
#include "pcp_internal.h"

namespace pcp {

namespace {

__device__ __forceinline__ double2 wrap2d(double2 d) { return make_double2(wrap(d.x), wrap(d.y)); }

__device__ __forceinline__ void add2(double2* g, int v, double2 a) {
    atomicAdd(&g[v].x, a.x);
    atomicAdd(&g[v].y, a.y);
}

// exact crossing parameter of edge (vi, vi + di) with edge (vj, vj + dj):
// u = (dj x dij) / (dj x di), the u of getDf (kernels.cuh:175-176)
__device__ __forceinline__ double cross_param(double2 vi, double2 di, double2 vj, double2 dj) {
    const double dijx = wrap(vj.x - vi.x), dijy = wrap(vj.y - vi.y);
    const double w = dj.x * di.y - dj.y * di.x;
    const double k = dj.x * dijy - dj.y * dijx;
    return k / w;
}

}  // namespace

template <int kMode>
__global__ void __launch_bounds__(256)
k_overlap_energy_grad(const double2* __restrict__ pos, const int* __restrict__ start, int V,
                      ContactWS ws, const Ctrl* __restrict__ ctrl, double2* __restrict__ out,
                      double* __restrict__ energy, int* __restrict__ bad) {
    pdl_enter();
    const int I = min(ctrl->numRecords, ws.capRecords);
    double eLocal = 0.0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < I; r += gridDim.x * blockDim.x) {
        const unsigned long long inter = ws.recKey[r], outer = ws.recOuter[r];
        if (inter == outer) continue;               // no exit partner (kernels.cuh:1078)
        const int s1 = (int)((inter >> 32) & 0xFFFF), s2 = (int)(inter >> 48);
        const int iLoc = (int)((inter >> 16) & 0xFFFF), jLoc = (int)(inter & 0xFFFF);
        const int kLoc = (int)((outer >> 16) & 0xFFFF), lLoc = (int)(outer & 0xFFFF);
        const int b1 = start[s1], n1 = start[s1 + 1] - b1;
        const int b2 = start[s2], n2 = start[s2 + 1] - b2;
        if (iLoc >= n1 || lLoc >= n1 || jLoc >= n2 || kLoc >= n2 || b1 + n1 > V || b2 + n2 > V) {
            atomicOr(bad, 1);
            continue;
        }
        auto nx1 = [&](int loc) { return b1 + (loc + 1 == n1 ? 0 : loc + 1); };
        auto nx2 = [&](int loc) { return b2 + (loc + 1 == n2 ? 0 : loc + 1); };
        const int i = b1 + iLoc, zi = nx1(iLoc), j = b2 + jLoc, zj = nx2(jLoc);
        const int k = b2 + kLoc, zk = nx2(kLoc), l = b1 + lLoc, zl = nx1(lLoc);
        const bool same = (i == l);
        const double2 pi = pos[i], pzi = pos[zi], pj = pos[j], pzj = pos[zj];
        const double2 pk = pos[k], pzk = pos[zk];
        // the edge the partner leaves through: (l, zl), or (i, zi) when i == l
        const double2 pm = same ? pi : pos[l], pzm = same ? pzi : pos[zl];
        const int m = same ? i : l, zm = same ? zi : zl;
        const double2 di = wrap2d(make_double2(pzi.x - pi.x, pzi.y - pi.y));
        const double2 dk = wrap2d(make_double2(pzk.x - pk.x, pzk.y - pk.y));
        double t1, t2;
        if (kMode == kExactGrad) {
            const double2 dj = wrap2d(make_double2(pzj.x - pj.x, pzj.y - pj.y));
            const double2 dm = wrap2d(make_double2(pzm.x - pm.x, pzm.y - pm.y));
            t1 = cross_param(pi, di, pj, dj);
            t2 = cross_param(pk, dk, pm, dm);
        } else {
            t1 = (double)ws.recTU[r].y;             // tu.y on si's edge (kernels.cuh:1104)
            t2 = (double)ws.recUT[r].y;
        }
        const double2 f1 = wrap2d(make_double2(pi.x + t1 * di.x, pi.y + t1 * di.y));
        const double2 f2 = wrap2d(make_double2(pk.x + t2 * dk.x, pk.y + t2 * dk.y));
        // coefficients collected for f1 and f2 (contracted with their
        // Jacobians at the end) and the direct vertex terms
        double2 c1 = make_double2(0.0, 0.0), c2 = make_double2(0.0, 0.0);
        double eRec = 0.0;
        const double sc = (kMode == kExactGrad) ? 0.5 : -1.0;
        // one chain segment a -> b with start point f1; ta/tb: 0 vertex,
        // 1 the point f1, 2 the point f2
        auto segment = [&](double2 a, int ta, int va, double2 b, int tb, int vb) {
            eRec += h_term(a, b, f1);
            double2 g1, g2;
            g12(a, b, f1, g1, g2);                  // g1.x = g2.x = dy
            if (kMode == kExactGrad) c1.x += sc * (-2.0 * g1.x);   // dh/ds = (-2 dy, 0)
            g1.x *= sc; g1.y *= sc; g2.x *= sc; g2.y *= sc;
            if (ta == 0) add2(out, va, g1); else if (ta == 1) { c1.x += g1.x; c1.y += g1.y; }
            else { c2.x += g1.x; c2.y += g1.y; }
            if (tb == 0) add2(out, vb, g2); else if (tb == 1) { c1.x += g2.x; c1.y += g2.y; }
            else { c2.x += g2.x; c2.y += g2.y; }
        };
        if (same) {
            segment(f1, 1, -1, f2, 2, -1);
        } else {
            segment(f1, 1, -1, pzi, 0, zi);
            // the whole edges strictly inside: m' = i+1 .. l-1 (cyclic), as the
            // interior kernel's iDist in (0, lDist) (kernels.cuh:1380-1389)
            int loc = iLoc + 1 == n1 ? 0 : iLoc + 1;
            for (int guard = 0; loc != lLoc && guard < n1; ++guard) {
                const int a = b1 + loc, za = nx1(loc);
                segment(pos[a], 0, a, pos[za], 0, za);
                loc = loc + 1 == n1 ? 0 : loc + 1;
            }
            segment(pm, 0, m, f2, 2, -1);
        }
        double2 o[4];
        gDf(pi, pzi, pj, pzj, c1, o);
        add2(out, i, o[0]); add2(out, zi, o[1]); add2(out, j, o[2]); add2(out, zj, o[3]);
        gDf(pk, pzk, pm, pzm, c2, o);
        add2(out, k, o[0]); add2(out, zk, o[1]); add2(out, m, o[2]); add2(out, zm, o[3]);
        eLocal += 0.5 * eRec;
    }
    for (int off = 16; off > 0; off >>= 1) eLocal += __shfl_down_sync(PCP_FULL, eLocal, off);
    if ((threadIdx.x & 31) == 0 && eLocal != 0.0) atomicAdd(energy, eLocal);
}

cudaError_t launch_overlap_energy_grad(const double2* pos, const int* start, int V,
                                       const ContactWS& ws, const Ctrl* ctrl, int mode,
                                       double2* out, double* energy, int* bad, cudaStream_t st) {
    const int grid = 2 * 152;
    if (mode == kExactGrad)
        launch_k(k_overlap_energy_grad<kExactGrad>, dim3(grid), dim3(256), 0, st, pos, start, V,
                 ws, ctrl, out, energy, bad);
    else
        launch_k(k_overlap_energy_grad<kRefForce>, dim3(grid), dim3(256), 0, st, pos, start, V,
                 ws, ctrl, out, energy, bad);
    return cudaGetLastError();
}

}  // namespace pcp
