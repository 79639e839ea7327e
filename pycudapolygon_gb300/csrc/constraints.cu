// constraints.cu -- constraint-space force projection, SHAKE, XPBD and the
// device-resident FIRE pieces (sm_103a).
//
// GB300 has little FP64 throughput (about 0.6 T DFMA/s) and charges a
// partly masked warp like a full one, so these per-polygon solves run one
// polygon per thread (full warps of independent polygons) and exploit the
// sparsity of the constraint Jacobians: the Gram matrix of the edge-length
// gradients is cyclic tridiagonal, so the reference's batched SVD
// (cusolverDnDgesvdaStridedBatched, model.cu:182-190) and dense
// (n+1)x(n+1) SHAKE system (model.cu:616-636) become O(n) solves.  The
// per-vertex intermediates live in a global scratch array indexed by vertex,
// so any polygon size is accepted.
#include <cuda_runtime.h>
#include <math.h>

#include "pcp_common.cuh"
#include "pcp_internal.h"

namespace pcp {

static inline int nblk(long long n, int t) {
    long long b = (n + t - 1) / t;
    return b < 1 ? 1 : (int)b;
}

// Solve three right-hand sides of a cyclic tridiagonal system
//   lo[k] x[k-1] + di[k] x[k] + up[k] x[k+1] = d[k]   (indices mod n, n >= 3)
// by Sherman-Morrison on top of the Thomas algorithm.  All arrays are strided
// views into per-vertex scratch; d0..d2 are overwritten by the solutions.
// cp is scratch.  Returns false when a pivot vanishes.
struct Tri {
    const double* lo; const double* di; const double* up;
};

__device__ bool cyclic_solve3(int n, Tri T, double* d0, double* d1, double* d2, double* cp,
                              double* zs) {
    const double gamma = -T.di[0];
    const double beta = T.lo[0];          // coefficient of x[n-1] in row 0
    const double alpha = T.up[n - 1];     // coefficient of x[0] in row n-1
    if (gamma == 0.0) return false;
    // forward sweep for the modified tridiagonal, 4 right-hand sides
    // (d0, d1, d2 and the Sherman-Morrison vector u = (gamma, 0.., alpha))
    double b0 = T.di[0] - gamma;
    if (b0 == 0.0) return false;
    double inv = 1.0 / b0;
    cp[0] = T.up[0] * inv;
    d0[0] *= inv; d1[0] *= inv; d2[0] *= inv;
    zs[0] = gamma * inv;
    for (int k = 1; k < n; ++k) {
        double bk = T.di[k];
        if (k == n - 1) bk -= alpha * beta / gamma;
        double m = bk - T.lo[k] * cp[k - 1];
        if (m == 0.0) return false;
        double im = 1.0 / m;
        cp[k] = (k < n - 1) ? T.up[k] * im : 0.0;
        d0[k] = (d0[k] - T.lo[k] * d0[k - 1]) * im;
        d1[k] = (d1[k] - T.lo[k] * d1[k - 1]) * im;
        d2[k] = (d2[k] - T.lo[k] * d2[k - 1]) * im;
        double uk = (k == n - 1) ? alpha : 0.0;
        zs[k] = (uk - T.lo[k] * zs[k - 1]) * im;
    }
    for (int k = n - 2; k >= 0; --k) {
        d0[k] -= cp[k] * d0[k + 1];
        d1[k] -= cp[k] * d1[k + 1];
        d2[k] -= cp[k] * d2[k + 1];
        zs[k] -= cp[k] * zs[k + 1];
    }
    double den = 1.0 + zs[0] + beta * zs[n - 1] / gamma;
    if (den == 0.0) return false;
    double f0 = (d0[0] + beta * d0[n - 1] / gamma) / den;
    double f1 = (d1[0] + beta * d1[n - 1] / gamma) / den;
    double f2 = (d2[0] + beta * d2[n - 1] / gamma) / den;
    for (int k = 0; k < n; ++k) {
        d0[k] -= f0 * zs[k];
        d1[k] -= f1 * zs[k];
        d2[k] -= f2 * zs[k];
    }
    return true;
}

// ------------------------------------------------------------ projection ----
// projectForceCUDA (model.cu:165-206; kernels.cuh:389-523): per polygon,
//   F' = F - J lambda,  (J^T J) lambda = J^T F            (edge-length span)
//   q  = a - J mu,      (J^T J) mu = J^T a                (a: unit area grad)
//   F'' = F' - q (q.F') / |q|^2   when |q| > 1e-14        (kernels.cuh:464)
// J column k = -t_k at vertex k, +t_k at vertex k+1 (buildEdgeGradMatrix,
// kernels.cuh:389-406); J^T J is cyclic tridiagonal with 2 on the diagonal
// and -t_k.t_{k+1} beside it.  Edges shorter than 1e-14 are left out, as
// the reference leaves their column zero.
//
// When `fire` is given (device-resident FIRE step) the kernel also applies
// the FIRE velocity half-kick v += dt/2 F'' and accumulates F.v, |v|^2 and
// |F|^2 (Model::minimizeFIREStep lines 471-472) if the step is neither a
// SHAKE failure nor an energy-increase rollback, and always max |F''|.
struct ProjScratch { double* s; int V; };

__global__ void __launch_bounds__(128)
k_project(const double2* __restrict__ pos, const int* __restrict__ start, int P,
          const double* __restrict__ constraints, double2* __restrict__ force,
          double* __restrict__ scratch, int V, Ctrl* fire, double2* __restrict__ vel,
          const int* gate) {
    if (gate_closed(gate)) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool proceed = false;
    double dt = 0.0;
    if (fire) {
        double E = fire->energy, E0 = fire->ePre;
        bool rb = E > E0 + fmax(fabs(E0) * 1e-10, 1e-14);
        proceed = !fire->shakeFailed && !rb && fire->rollback == 0;
        dt = fire->dt;
        if (p == 0 && fire->rollback == 0) {
            fire->proceed = proceed ? 1 : 0;
            // the energy-increase rollback path runs when the step is not a
            // SHAKE failure and the energy went up (model.cpp:450-453)
            fire->rbGate = (!fire->shakeFailed && rb && fire->active) ? 1 : 0;
        }
    }
    double sP = 0.0, sV = 0.0, sF = 0.0, mF = 0.0;
    if (p < P) {
        int st = start[p], n = start[p + 1] - st;
        if (n >= 3) {
            // scratch layout per vertex (stride V): tx ty lo di up r0 r1 r2 cp zs
            double* tx = scratch + 0 * (size_t)V + st;
            double* ty = scratch + 1 * (size_t)V + st;
            double* lo = scratch + 2 * (size_t)V + st;
            double* di = scratch + 3 * (size_t)V + st;
            double* up = scratch + 4 * (size_t)V + st;
            double* r0 = scratch + 5 * (size_t)V + st;
            double* r1 = scratch + 6 * (size_t)V + st;
            double* r2 = scratch + 7 * (size_t)V + st;
            double* cp = scratch + 8 * (size_t)V + st;
            double* zs = scratch + 9 * (size_t)V + st;
            for (int k = 0; k < n; ++k) {
                int kn = (k + 1 == n) ? 0 : k + 1;
                double2 a = pos[st + k], b = pos[st + kn];
                double dx = wrap(b.x - a.x), dy = wrap(b.y - a.y);
                double len = sqrt(dx * dx + dy * dy);
                if (len < 1e-14) { tx[k] = 0.0; ty[k] = 0.0; di[k] = 1.0; }
                else { double il = 1.0 / len; tx[k] = dx * il; ty[k] = dy * il; di[k] = 2.0; }
            }
            for (int k = 0; k < n; ++k) {
                int kn = (k + 1 == n) ? 0 : k + 1;
                double o = -(tx[k] * tx[kn] + ty[k] * ty[kn]);
                up[k] = o;
                lo[kn] = o;
                double2 f0 = force[st + k], f1 = force[st + kn];
                r0[k] = tx[k] * (f1.x - f0.x) + ty[k] * (f1.y - f0.y);
                const double* c0 = constraints + 6 * (size_t)(st + k);
                const double* c1 = constraints + 6 * (size_t)(st + kn);
                r1[k] = tx[k] * (c1[0] - c0[0]) + ty[k] * (c1[1] - c0[1]);
                r2[k] = 0.0;
            }
            Tri T{lo, di, up};
            bool ok = cyclic_solve3(n, T, r0, r1, r2, cp, zs);
            if (ok) {
                double qF = 0.0, qq = 0.0;
                for (int k = 0; k < n; ++k) {
                    int kp = (k == 0) ? n - 1 : k - 1;
                    // (J x)_k = -x_k t_k + x_{k-1} t_{k-1}
                    double jlx = -r0[k] * tx[k] + r0[kp] * tx[kp];
                    double jly = -r0[k] * ty[k] + r0[kp] * ty[kp];
                    double jmx = -r1[k] * tx[k] + r1[kp] * tx[kp];
                    double jmy = -r1[k] * ty[k] + r1[kp] * ty[kp];
                    const double* c0 = constraints + 6 * (size_t)(st + k);
                    double qx = c0[0] - jmx, qy = c0[1] - jmy;
                    double2 f = force[st + k];
                    double fx = f.x - jlx, fy = f.y - jly;
                    cp[k] = qx; zs[k] = qy;        // reuse scratch for q
                    r2[k] = fx; lo[k] = fy;        // and for F'
                    qF += qx * fx + qy * fy;
                    qq += qx * qx + qy * qy;
                }
                double mag = sqrt(qq);
                double coef = (mag > 1e-14) ? qF / qq : 0.0;
                for (int k = 0; k < n; ++k) {
                    double fx = r2[k] - coef * cp[k];
                    double fy = lo[k] - coef * zs[k];
                    force[st + k] = make_double2(fx, fy);
                    mF = fmax(mF, fmax(fabs(fx), fabs(fy)));
                    if (proceed) {
                        double2 v = vel[st + k];
                        v.x += 0.5 * dt * fx;
                        v.y += 0.5 * dt * fy;
                        vel[st + k] = v;
                        sP += fx * v.x + fy * v.y;
                        sV += v.x * v.x + v.y * v.y;
                        sF += fx * fx + fy * fy;
                    }
                }
            } else if (fire) {
                atomicOr(&fire->flags, kFlagNonFinite);
            }
        } else {
            for (int k = 0; k < n; ++k) {
                double2 f = force[st + k];
                mF = fmax(mF, fmax(fabs(f.x), fabs(f.y)));
                if (proceed) {
                    double2 v = vel[st + k];
                    v.x += 0.5 * dt * f.x; v.y += 0.5 * dt * f.y;
                    vel[st + k] = v;
                    sP += f.x * v.x + f.y * v.y;
                    sV += v.x * v.x + v.y * v.y;
                    sF += f.x * f.x + f.y * f.y;
                }
            }
        }
    }
    if (fire) {
        mF = warp_maxd(mF);
        if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&fire->maxF, mF);
        if (proceed) {
            sP = warp_sum(sP); sV = warp_sum(sV); sF = warp_sum(sF);
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(&fire->P, sP);
                atomicAdd(&fire->vv, sV);
                atomicAdd(&fire->ff, sF);
            }
        }
    }
}

cudaError_t launch_project(const double2* pos, const int* start, int P,
                           const double* constraints, double2* force, double* scratch, int V,
                           Ctrl* fireCtrl, const int* gate, double2* vel, cudaStream_t st) {
    if (P <= 0) return cudaSuccess;
    k_project<<<nblk(P, 128), 128, 0, st>>>(pos, start, P, constraints, force, scratch, V,
                                            fireCtrl, vel, gate);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ SHAKE ----
// shakeProjectCUDA (model.cu:616-636; the kernel itself, src/shake.h, is not
// in the reference tree).  Restated as matrix SHAKE with Newton steps in the
// multipliers:  sigma_k = |e_k| - L, sigma_n = A - A0;  x += G_ref^T dl with
// (G(x) G_ref^T) dl = -sigma(x), G_ref the constraint gradients at entry.
// G(x) G_ref^T is a cyclic tridiagonal block (edges) bordered by one row and
// column (area); it is solved through two cyclic tridiagonal solves.  Each
// iteration first tests max|sigma| < tol; the count is the number of updates.
__device__ __forceinline__ double poly_area_rel(const double2* x, int n) {
    // sum (X_k + X_{k+1}) dy_k / 2 relative to vertex 0 (kernels.cuh:327-332)
    double a = 0.0;
    double2 p0 = x[0];
    for (int k = 0; k < n; ++k) {
        int kn = (k + 1 == n) ? 0 : k + 1;
        double x1 = wrap(x[k].x - p0.x), x2 = wrap(x[kn].x - p0.x);
        double dy = wrap(x[kn].y - x[k].y);
        a += dy * (x2 + x1) / 2.0;
    }
    return a;
}

__global__ void __launch_bounds__(128)
k_shake(double2* __restrict__ pos, const int* __restrict__ start, int P,
        const double* __restrict__ targetEdge, const double* __restrict__ targetArea,
        int maxIter, double tol, int* __restrict__ itersOut, double* __restrict__ scratch,
        int V, const int* gate) {
    if (gate_closed(gate)) return;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    int it = 0;
    if (p < P) {
        int st = start[p], n = start[p + 1] - st;
        if (n >= 3 && maxIter > 0) {
            double L = targetEdge[p], A0 = targetArea[p];
            double2* x = pos + st;
            double* erx = scratch + 0 * (size_t)V + st;   // reference unit edges
            double* ery = scratch + 1 * (size_t)V + st;
            double* arx = scratch + 2 * (size_t)V + st;   // reference area gradient
            double* ary = scratch + 3 * (size_t)V + st;
            double* ecx = scratch + 4 * (size_t)V + st;   // current unit edges
            double* ecy = scratch + 5 * (size_t)V + st;
            double* lo = scratch + 6 * (size_t)V + st;
            double* di = scratch + 7 * (size_t)V + st;
            double* up = scratch + 8 * (size_t)V + st;
            double* y = scratch + 9 * (size_t)V + st;     // -sigma_e -> T^-1 (-sigma_e)
            double* w = scratch + 10 * (size_t)V + st;    // border column -> T^-1 w
            double* dummy = scratch + 11 * (size_t)V + st;
            double* cp = scratch + 12 * (size_t)V + st;
            double* zs = scratch + 13 * (size_t)V + st;
            double* vrow = scratch + 14 * (size_t)V + st; // border row
            double* acx = scratch + 15 * (size_t)V + st;  // current area gradient
            double* acy = scratch + 16 * (size_t)V + st;
            for (int k = 0; k < n; ++k) {
                int kn = (k + 1 == n) ? 0 : k + 1, kp = (k == 0) ? n - 1 : k - 1;
                double ex = wrap(x[kn].x - x[k].x), ey = wrap(x[kn].y - x[k].y);
                double len = sqrt(ex * ex + ey * ey);
                if (len > 0.0) { erx[k] = ex / len; ery[k] = ey / len; }
                else { erx[k] = 0.0; ery[k] = 0.0; }
                arx[k] = 0.5 * wrap(x[kn].y - x[kp].y);
                ary[k] = 0.5 * wrap(x[kp].x - x[kn].x);
            }
            for (; it < maxIter; ++it) {
                double worst = 0.0;
                for (int k = 0; k < n; ++k) {
                    int kn = (k + 1 == n) ? 0 : k + 1;
                    double ex = wrap(x[kn].x - x[k].x), ey = wrap(x[kn].y - x[k].y);
                    double len = sqrt(ex * ex + ey * ey);
                    double s = len - L;
                    y[k] = -s;
                    if (!(fabs(s) <= worst)) worst = fabs(s);
                    if (len > 0.0) { ecx[k] = ex / len; ecy[k] = ey / len; }
                    else { ecx[k] = 0.0; ecy[k] = 0.0; }
                }
                double sA = poly_area_rel(x, n) - A0;
                if (!(fabs(sA) <= worst)) worst = fabs(sA);
                if (worst < tol) break;
                if (!isfinite(worst)) { it = maxIter; break; }
                double dcorner = 0.0;
                for (int k = 0; k < n; ++k) {
                    int kn = (k + 1 == n) ? 0 : k + 1, kp = (k == 0) ? n - 1 : k - 1;
                    acx[k] = 0.5 * wrap(x[kn].y - x[kp].y);
                    acy[k] = 0.5 * wrap(x[kp].x - x[kn].x);
                    dcorner += acx[k] * arx[k] + acy[k] * ary[k];
                }
                for (int j = 0; j < n; ++j) {
                    int jn = (j + 1 == n) ? 0 : j + 1, jp = (j == 0) ? n - 1 : j - 1;
                    double cx = ecx[j], cy = ecy[j];
                    di[j] = 2.0 * (cx * erx[j] + cy * ery[j]);
                    up[j] = -(cx * erx[jn] + cy * ery[jn]);
                    lo[j] = -(cx * erx[jp] + cy * ery[jp]);
                    w[j] = cx * (arx[jn] - arx[j]) + cy * (ary[jn] - ary[j]);
                    vrow[j] = (acx[jn] - acx[j]) * erx[j] + (acy[jn] - acy[j]) * ery[j];
                    dummy[j] = 0.0;
                }
                Tri T{lo, di, up};
                if (!cyclic_solve3(n, T, y, w, dummy, cp, zs)) { it = maxIter; break; }
                double vy = 0.0, vz = 0.0;
                for (int j = 0; j < n; ++j) { vy += vrow[j] * y[j]; vz += vrow[j] * w[j]; }
                double den = dcorner - vz;
                if (den == 0.0) { it = maxIter; break; }
                double mu = (-sA - vy) / den;
                for (int c = 0; c < n; ++c) {
                    int cn = (c + 1 == n) ? 0 : c + 1;
                    double l = y[c] - mu * w[c];
                    x[c].x -= l * erx[c]; x[c].y -= l * ery[c];
                    x[cn].x += l * erx[c]; x[cn].y += l * ery[c];
                }
                for (int k = 0; k < n; ++k) { x[k].x += mu * arx[k]; x[k].y += mu * ary[k]; }
            }
            for (int k = 0; k < n; ++k) {
                double2 v = x[k];
                x[k] = make_double2(v.x - floor(v.x), v.y - floor(v.y));
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) it = max(it, __shfl_xor_sync(PCP_FULL, it, o));
    if ((threadIdx.x & 31) == 0 && it > 0) atomicMax(itersOut, it);
}

cudaError_t launch_shake(double2* pos, const int* start, int P, const double* targetEdge,
                         const double* targetArea, int maxIter, double tol, int* maxItersOut,
                         double* scratch, int V, const int* gate, cudaStream_t st) {
    if (P <= 0) return cudaSuccess;
    k_shake<<<nblk(P, 128), 128, 0, st>>>(pos, start, P, targetEdge, targetArea, maxIter, tol,
                                          maxItersOut, scratch, V, gate);
    return cudaGetLastError();
}

// ------------------------------------------------------------------- XPBD ----
// One iteration of xpbdProjectCUDA (model.cu:228-250; kernels.cuh:532-604),
// one polygon per thread: edges of even local index, then odd ones (and the
// closing edge of an odd ring last, where the reference races), then one
// area correction along the area gradient taken before the correction.
// devOut[2p] / devOut[2p+1] receive the edge / area deviations after it
// (xpbdEdgeDeviationKernel / xpbdAreaDeviationKernel, kernels.cuh:606-623).
__global__ void k_xpbd(double2* __restrict__ pos, const int* __restrict__ start, int P,
                       const double* __restrict__ tl, const double* __restrict__ ta,
                       double* __restrict__ devOut) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    int st = start[p], n = start[p + 1] - st;
    double2* x = pos + st;
    double L = tl[p];
    for (int color = 0; color < 3; ++color) {
        for (int kl = 0; kl < n; ++kl) {
            int c = kl % 2;
            if ((n % 2) && kl == n - 1) c = 2;
            if (c != color) continue;
            int kn = (kl + 1 == n) ? 0 : kl + 1;
            double ex = wrap(x[kn].x - x[kl].x), ey = wrap(x[kn].y - x[kl].y);
            double len = sqrt(ex * ex + ey * ey);
            if (len < 1e-14) continue;
            double cc = 0.5 * (len - L) / len;
            x[kl].x += cc * ex; x[kl].y += cc * ey;
            x[kn].x -= cc * ex; x[kn].y -= cc * ey;
        }
    }
    double xs = x[0].x, ys = x[0].y;
    double area = 0.0, g2 = 0.0;
    for (int k = 0; k < n; ++k) {
        int kn = (k + 1 == n) ? 0 : k + 1, kp = (k == 0) ? n - 1 : k - 1;
        double xk = wrap(x[k].x - xs), yk = wrap(x[k].y - ys);
        double xn = wrap(x[kn].x - xs), yn = wrap(x[kn].y - ys);
        double xp = wrap(x[kp].x - xs), yp = wrap(x[kp].y - ys);
        area += 0.5 * (xk * yn - xn * yk);
        double a = 0.5 * (yn - yp), b = 0.5 * (xp - xn);
        g2 += a * a + b * b;
    }
    double al = (area - ta[p]) / fmax(g2, 1e-24);
    // gradients from the positions before the correction
    double2 first = x[0], prevOrig = x[n - 1];
    for (int k = 0; k < n; ++k) {
        int kn = (k + 1 == n) ? 0 : k + 1;
        double2 nb = (kn == 0) ? first : x[kn];
        double2 pb = prevOrig;
        double xn = wrap(nb.x - xs), yn = wrap(nb.y - ys);
        double xp = wrap(pb.x - xs), yp = wrap(pb.y - ys);
        prevOrig = x[k];
        x[k].x -= al * 0.5 * (yn - yp);
        x[k].y -= al * 0.5 * (xp - xn);
    }
    double me = 0.0;
    for (int k = 0; k < n; ++k) {
        int kn = (k + 1 == n) ? 0 : k + 1;
        double ex = wrap(x[kn].x - x[k].x), ey = wrap(x[kn].y - x[k].y);
        me = fmax(me, fabs(sqrt(ex * ex + ey * ey) - L));
    }
    devOut[2 * p] = me;
    devOut[2 * p + 1] = fabs(area - ta[p]);
}

cudaError_t launch_xpbd_iteration(double2* pos, const int* start, int P,
                                  const double* targetEdge, const double* targetArea,
                                  double* devOut, cudaStream_t st) {
    if (P <= 0) return cudaSuccess;
    k_xpbd<<<nblk(P, 128), 128, 0, st>>>(pos, start, P, targetEdge, targetArea, devOut);
    return cudaGetLastError();
}

// ------------------------------------------------------------------- FIRE ----
// The reference's FIRE kernels (src/FIRE.h) are absent; restated from their
// call contract (model.cu:576-608, model.cpp:405-486) and the velocity-Verlet
// FIRE of Bitzek et al., PRL 97, 170201 (2006):
//   updatePositionAndVelocity  v += dt/2 F; x = frac(x + dt v)
//   updateVelocity             v += dt/2 F    (fused into k_project)
//   bend (P = F.v first)       v = (1-a) v + a |v| F/|F|
//   rederive after SHAKE       v += wrap(x_shake - x_verlet) / dt
// All FIRE scalars stay in the device control block; the step is a fixed
// launch sequence, so it is captured once as a CUDA graph.

// step start: save positions, record E_pre, Verlet half-kick + drift
__global__ void k_fire_begin(double2* __restrict__ pos, double2* __restrict__ vel,
                             const double2* __restrict__ force, double2* __restrict__ save,
                             int V, Ctrl* __restrict__ c, const int* gate) {
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double dt = c->dt;
    if (i < V) {
        double2 x = pos[i], v = vel[i], f = force[i];
        save[i] = x;
        v.x += 0.5 * dt * f.x; v.y += 0.5 * dt * f.y;
        double px = x.x + dt * v.x, py = x.y + dt * v.y;
        vel[i] = v;
        pos[i] = make_double2(px - floor(px), py - floor(py));
    }
}

// per-step resets of the control block (runs before k_fire_begin)
__global__ void k_fire_reset(Ctrl* __restrict__ c, const int* gate) {
    if (gate_closed(gate)) return;
    c->ePre = c->energy;
    c->energy = 0.0;
    c->snapDt = c->dt; c->snapAlpha = c->alpha; c->snapNPos = c->nPos;
    c->maxF = 0.0;
    c->P = 0.0; c->vv = 0.0; c->ff = 0.0;
    c->shakeIters1 = 0; c->shakeIters2 = 0;
    c->needRetry = 0; c->retryGate = 0;
    c->shakeFailed = 0;
    c->rollback = 0; c->rbGate = 0; c->proceed = 0;
}

// which == 1: after the first SHAKE attempt; which == 2: after the retry
__global__ void k_fire_shake_check(Ctrl* __restrict__ c, int which, const int* gate) {
    if (gate_closed(gate)) return;
    if (which == 1) {
        c->shakeLast = c->shakeIters1;
        c->needRetry = (c->shakeIters1 >= c->shakeIter) ? 1 : 0;
        c->retryGate = c->needRetry && c->active;
    } else {
        if (c->needRetry) {
            c->shakeLast = c->shakeIters2;
            c->shakeFailed = (c->shakeIters2 >= 10 * c->shakeIter) ? 1 : 0;
        }
    }
}

// SHAKE failure: restore the step's start positions and zero v; success:
// rederive v from the SHAKE displacement (model.cpp:431-438)
__global__ void k_fire_after_shake(double2* __restrict__ pos, double2* __restrict__ vel,
                                   const double2* __restrict__ save,
                                   const double2* __restrict__ verlet, int V,
                                   const Ctrl* __restrict__ c, const int* gate) {
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    if (c->shakeFailed) {
        pos[i] = save[i];
        vel[i] = make_double2(0.0, 0.0);
    } else {
        double dt = c->dt;
        double2 x = pos[i], y = verlet[i], v = vel[i];
        v.x += wrap(x.x - y.x) / dt;
        v.y += wrap(x.y - y.y) / dt;
        vel[i] = v;
    }
}

// energy-increase rollback (model.cpp:453-465): restore positions, zero v,
// zero the force and energy before they are recomputed
__global__ void k_fire_rollback(double2* __restrict__ pos, double2* __restrict__ vel,
                                double2* __restrict__ force, const double2* __restrict__ save,
                                int V, Ctrl* __restrict__ c, const int* gate) {
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) { c->energy = 0.0; c->maxF = 0.0; }
    if (i >= V) return;
    pos[i] = save[i];
    vel[i] = make_double2(0.0, 0.0);
    force[i] = make_double2(0.0, 0.0);
}

// zero force + energy (+ maxF) under a gate (updateForceEnergy's memsets)
__global__ void k_zero_force(double2* __restrict__ force, int V, Ctrl* __restrict__ c,
                             const int* gate) {
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) { c->energy = 0.0; c->maxF = 0.0; }
    if (i < V) force[i] = make_double2(0.0, 0.0);
}

// velocity update for models without projection (soft-body / hybrid):
// v += dt/2 F, accumulate F.v, |v|^2, |F|^2, max |F|
__global__ void k_fire_velocity(double2* __restrict__ vel, const double2* __restrict__ force,
                                int V, Ctrl* __restrict__ c, const int* gate) {
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double E = c->energy, E0 = c->ePre;
    bool rb = E > E0 + fmax(fabs(E0) * 1e-10, 1e-14);
    bool proceed = !c->shakeFailed && !rb && c->rollback == 0;
    if (i == 0 && c->rollback == 0) {
        c->proceed = proceed ? 1 : 0;
        c->rbGate = (!c->shakeFailed && rb && c->active) ? 1 : 0;
    }
    double sP = 0.0, sV = 0.0, sF = 0.0, mF = 0.0;
    if (i < V) {
        double2 f = force[i];
        mF = fmax(fabs(f.x), fabs(f.y));
        if (proceed) {
            double dt = c->dt;
            double2 v = vel[i];
            v.x += 0.5 * dt * f.x; v.y += 0.5 * dt * f.y;
            vel[i] = v;
            sP = f.x * v.x + f.y * v.y;
            sV = v.x * v.x + v.y * v.y;
            sF = f.x * f.x + f.y * f.y;
        }
    }
    mF = warp_maxd(mF);
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&c->maxF, mF);
    if (proceed) {
        sP = warp_sum(sP); sV = warp_sum(sV); sF = warp_sum(sF);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&c->P, sP); atomicAdd(&c->vv, sV); atomicAdd(&c->ff, sF);
        }
    }
}

// max |F| only (rollback path of models without projection)
__global__ void k_fire_maxf(const double2* __restrict__ force, int V, Ctrl* __restrict__ c,
                            const int* gate) {
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double mF = 0.0;
    if (i < V) { double2 f = force[i]; mF = fmax(fabs(f.x), fabs(f.y)); }
    mF = warp_maxd(mF);
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg(&c->maxF, mF);
}

// bend v toward F when the step proceeds (model.cpp:471-484)
__global__ void k_fire_bend(double2* __restrict__ vel, const double2* __restrict__ force,
                            int V, const Ctrl* __restrict__ c, const int* gate) {
    if (gate_closed(gate)) return;
    if (!c->proceed) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V) return;
    double P = c->P;
    if (P > 0.0) {
        double fn = sqrt(c->ff), vn = sqrt(c->vv), a = c->alpha;
        if (fn > 0.0) {
            double s = a * vn / fn;
            double2 v = vel[i], f = force[i];
            vel[i] = make_double2((1.0 - a) * v.x + s * f.x, (1.0 - a) * v.y + s * f.y);
        }
    } else {
        vel[i] = make_double2(0.0, 0.0);
    }
}

// scalar bookkeeping of the step (model.cpp:444-485) and the stop test of
// Model::minimizeFIRE (model.cpp:500)
__global__ void k_fire_scalars(Ctrl* __restrict__ c, const int* gate) {
    if (gate_closed(gate)) return;
    if (c->flags & (kFlagPairOverflow | kFlagRecordOverflow | kFlagSlowOverflow |
                    kFlagFixOverflow | kFlagCapacity)) {
        // a contact buffer overflowed: stop here; the host grows the buffers
        // and redoes this step from its snapshot
        c->needsRecovery = 1;
        c->active = 0;
        return;
    }
    double dt = c->dt, alpha = c->alpha;
    int nPos = c->nPos;
    if (c->shakeFailed) {
        c->outE = c->energy;
        dt *= c->fDec; alpha = c->alphaStart; nPos = 0;
    } else if (c->rollback) {
        c->outE = c->ePre;
        dt *= c->fDec; alpha = c->alphaStart; nPos = 0;
    } else {
        c->outE = c->energy;
        if (c->P > 0.0) {
            if (++nPos >= c->nMin) {
                double nd = fmin(dt * c->fInc, c->dtMax);
                if (nd > dt) alpha *= c->fAlpha;
                dt = nd;
            }
        } else {
            dt *= c->fDec; alpha = c->alphaStart; nPos = 0;
        }
    }
    c->dt = dt; c->alpha = alpha; c->nPos = nPos;
    c->stepsDone += 1;
    if (c->maxF <= c->threshold) { c->converged = 1; c->active = 0; }
    if (c->stepLimit > 0 && c->stepsDone >= c->stepLimit) c->active = 0;
}

// mark the rollback as taken (the flag the rollback kernels gate on is set
// by k_project / k_fire_velocity; the scalars kernel needs `rollback`)
__global__ void k_fire_mark_rollback(Ctrl* __restrict__ c, const int* gate) {
    if (gate_closed(gate)) return;
    c->rollback = 1;
}

// --------------------------------------------------------------- launchers ----
cudaError_t launch_fire_reset(Ctrl* c, const int* gate, cudaStream_t st) {
    k_fire_reset<<<1, 1, 0, st>>>(c, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_begin(double2* pos, double2* vel, const double2* force, double2* save,
                              int V, Ctrl* c, const int* gate, cudaStream_t st) {
    k_fire_begin<<<nblk(V, 256), 256, 0, st>>>(pos, vel, force, save, V, c, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_shake_check(Ctrl* c, int which, const int* gate, cudaStream_t st) {
    k_fire_shake_check<<<1, 1, 0, st>>>(c, which, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_after_shake(double2* pos, double2* vel, const double2* save,
                                    const double2* verlet, int V, Ctrl* c, const int* gate,
                                    cudaStream_t st) {
    k_fire_after_shake<<<nblk(V, 256), 256, 0, st>>>(pos, vel, save, verlet, V, c, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_rollback(double2* pos, double2* vel, double2* force, const double2* save,
                                 int V, Ctrl* c, const int* gate, cudaStream_t st) {
    k_fire_mark_rollback<<<1, 1, 0, st>>>(c, gate);
    k_fire_rollback<<<nblk(V, 256), 256, 0, st>>>(pos, vel, force, save, V, c, gate);
    return cudaGetLastError();
}
cudaError_t launch_zero_force(double2* force, int V, Ctrl* c, const int* gate, cudaStream_t st) {
    k_zero_force<<<nblk(V, 256), 256, 0, st>>>(force, V, c, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_velocity(double2* vel, const double2* force, int V, Ctrl* c,
                                 const int* gate, cudaStream_t st) {
    k_fire_velocity<<<nblk(V, 256), 256, 0, st>>>(vel, force, V, c, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_maxf(const double2* force, int V, Ctrl* c, const int* gate,
                             cudaStream_t st) {
    k_fire_maxf<<<nblk(V, 256), 256, 0, st>>>(force, V, c, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_finish(double2* vel, const double2* force, int V, Ctrl* c,
                               const int* gate, cudaStream_t st) {
    k_fire_bend<<<nblk(V, 256), 256, 0, st>>>(vel, force, V, c, gate);
    k_fire_scalars<<<1, 1, 0, st>>>(c, gate);
    return cudaGetLastError();
}

}  // namespace pcp
