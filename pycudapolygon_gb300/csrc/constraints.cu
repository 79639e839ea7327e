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

#include <mutex>

#include "pcp_common.cuh"
#include "pcp_internal.h"
#include "pcp_fire.cuh"

namespace pcp {

static inline int nblk(long long n, int t) {
    long long b = (n + t - 1) / t;
    return b < 1 ? 1 : (int)b;
}

// Strided view of one per-vertex scratch array: element k of the polygon a
// thread works on lives at p[k * s].  In shared memory the arrays are laid out
// [array][k][lane] (s = 32, bank-conflict free); in the global fallback they
// are indexed by vertex (s = 1).
struct Arr {
    double* p;
    int s;
    __device__ __forceinline__ double& operator[](int k) const { return p[(size_t)k * s]; }
};

struct Scratch {
    double* base;
    size_t arrStride;   // distance between arrays
    int kStride;        // distance between consecutive vertices
    __device__ __forceinline__ Arr arr(int a) const { return Arr{base + (size_t)a * arrStride, kStride}; }
};

// Scratch of the polygon handled by this thread: shared memory when the
// launch provided it (smemN > 0 vertices per thread), else the global array.
__device__ __forceinline__ Scratch thread_scratch(double* smem, int smemN, double* global, int V,
                                                  int st) {
    if (smemN > 0) return Scratch{smem + (threadIdx.x & 31), (size_t)smemN * 32, 32};
    return Scratch{global + st, (size_t)V, 1};
}

// Solve `nr` (1..3) right-hand sides of a cyclic tridiagonal system
//   lo[k] x[k-1] + di[k] x[k] + up[k] x[k+1] = d[k]   (indices mod n, n >= 3)
// by Sherman-Morrison on top of the Thomas algorithm.  The right-hand sides
// are overwritten by the solutions; cp and zs are scratch.  Returns false
// when a pivot vanishes.
__device__ bool cyclic_solve(int n, Arr lo, Arr di, Arr up, int nr, Arr d0, Arr d1, Arr d2,
                             Arr cp, Arr zs) {
    const double gamma = -di[0];
    const double beta = lo[0];          // coefficient of x[n-1] in row 0
    const double alpha = up[n - 1];     // coefficient of x[0] in row n-1
    if (gamma == 0.0) return false;
    double b0 = di[0] - gamma;
    if (b0 == 0.0) return false;
    double inv = 1.0 / b0;
    cp[0] = up[0] * inv;
    d0[0] *= inv;
    if (nr > 1) d1[0] *= inv;
    if (nr > 2) d2[0] *= inv;
    zs[0] = gamma * inv;
    double cpPrev = cp[0], z0 = d0[0], z1 = nr > 1 ? d1[0] : 0.0, z2 = nr > 2 ? d2[0] : 0.0;
    double zsPrev = zs[0];
    for (int k = 1; k < n; ++k) {
        double bk = di[k];
        if (k == n - 1) bk -= alpha * beta / gamma;
        double l = lo[k];
        double m = bk - l * cpPrev;
        if (m == 0.0) return false;
        double im = 1.0 / m;
        cpPrev = (k < n - 1) ? up[k] * im : 0.0;
        cp[k] = cpPrev;
        z0 = (d0[k] - l * z0) * im; d0[k] = z0;
        if (nr > 1) { z1 = (d1[k] - l * z1) * im; d1[k] = z1; }
        if (nr > 2) { z2 = (d2[k] - l * z2) * im; d2[k] = z2; }
        double uk = (k == n - 1) ? alpha : 0.0;
        zsPrev = (uk - l * zsPrev) * im;
        zs[k] = zsPrev;
    }
    for (int k = n - 2; k >= 0; --k) {
        double c = cp[k];
        z0 = d0[k] - c * z0; d0[k] = z0;
        if (nr > 1) { z1 = d1[k] - c * z1; d1[k] = z1; }
        if (nr > 2) { z2 = d2[k] - c * z2; d2[k] = z2; }
        zsPrev = zs[k] - c * zsPrev; zs[k] = zsPrev;
    }
    double den = 1.0 + zs[0] + beta * zs[n - 1] / gamma;
    if (den == 0.0) return false;
    double f0 = (d0[0] + beta * d0[n - 1] / gamma) / den;
    double f1 = nr > 1 ? (d1[0] + beta * d1[n - 1] / gamma) / den : 0.0;
    double f2 = nr > 2 ? (d2[0] + beta * d2[n - 1] / gamma) / den : 0.0;
    for (int k = 0; k < n; ++k) {
        double z = zs[k];
        d0[k] -= f0 * z;
        if (nr > 1) d1[k] -= f1 * z;
        if (nr > 2) d2[k] -= f2 * z;
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
// the reference leaves their column zero.  One polygon per thread, 32
// threads per block so that small systems still spread over the SMs.
//
// When `fire` is given (device-resident FIRE step) the kernel also applies
// the FIRE velocity half-kick v += dt/2 F'' and accumulates F.v, |v|^2 and
// |F|^2 (Model::minimizeFIREStep lines 471-472) if the step is neither a
// SHAKE failure nor an energy-increase rollback, and always max |F''|.
constexpr int kProjArrays = 11;
constexpr int kConsThreads = 32;

__device__ void fire_scalars(Ctrl* __restrict__ c);

// End of the step's force pass (the projection, or the velocity half-kick
// of the soft models): the last block to finish does the scalar bookkeeping
// of the step, unless the energy-increase rollback runs next (the pass in
// its body ends the step then).  Every thread of the block calls this.
__device__ __forceinline__ void fire_pass_end(Ctrl* __restrict__ c, bool rollbackNext) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int t = atomicAdd(&c->bendTicket, 1u);
        if (t == gridDim.x - 1) {
            __threadfence();
            if (!rollbackNext) fire_scalars(c);
        }
    }
}

// fire_decide once per block (an FP64 compare costs a warp instruction, so
// once per block rather than once per warp), published by block 0; every
// thread of the block calls this.
struct FireView {
    bool proceed, rbNext;
    double dt;
};
__device__ __forceinline__ FireView fire_view(Ctrl* __restrict__ c,
                                              cudaGraphConditionalHandle rbCond, int useCond) {
    __shared__ int s_bits;
    __shared__ double s_dt;
    if (threadIdx.x == 0) {
        s_bits = fire_decide(c, blockIdx.x == 0, rbCond, useCond);
        s_dt = c->dt;
    }
    __syncthreads();
    return FireView{(s_bits & 1) != 0, (s_bits & 2) != 0, s_dt};
}

// The projection's view of the step.  In the step's own pass (mainPass) the
// force pass has decided and published the rollback already, and a rollback
// body may be running beside this kernel (it resets the energy), so the
// published outcome is read; otherwise (the rollback body's pass) the test
// itself, unpublished.  Every thread of the block calls this.
__device__ __forceinline__ FireView fire_view_proj(Ctrl* __restrict__ c, int mainPass) {
    __shared__ int s_bits;
    __shared__ double s_dt;
    if (threadIdx.x == 0) {
        s_bits = mainPass ? ((__ldcg(&c->proceed) ? 1 : 0) | (__ldcg(&c->rbGate) ? 2 : 0))
                          : fire_decide(c, false, 0, 0);
        s_dt = c->dt;
    }
    __syncthreads();
    return FireView{(s_bits & 1) != 0, (s_bits & 2) != 0, s_dt};
}

__global__ void __launch_bounds__(kConsThreads)
k_project(const double2* __restrict__ pos, const int* __restrict__ start, int P,
          const double* __restrict__ constraints, double2* __restrict__ force,
          double* __restrict__ scratch, int V, int smemN, int areaFromPositions, Ctrl* fire,
          double2* __restrict__ vel, int mainPass, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    extern __shared__ double cons_smem[];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool proceed = false, rbNext = false;
    double dt = 0.0;
    if (fire) {
        const FireView fv = fire_view_proj(fire, mainPass);
        if (mainPass && fv.rbNext) return;     // the rollback body redoes the pass
        proceed = fv.proceed; rbNext = fv.rbNext; dt = fv.dt;
    }
    double sP = 0.0, sV = 0.0, sF = 0.0, mF = 0.0;
    if (p < P) {
        int st = start[p], n = start[p + 1] - st;
        int useSmem = (n <= smemN) ? smemN : 0;
        if (n >= 3) {
            Scratch S = thread_scratch(cons_smem, useSmem, scratch, V, st);
            Arr tx = S.arr(0), ty = S.arr(1), lo = S.arr(2), di = S.arr(3), up = S.arr(4);
            Arr r0 = S.arr(5), r1 = S.arr(6), ac = S.arr(7), cp = S.arr(8), zs = S.arr(9);
            Arr ad = S.arr(10);   // unit area gradient (x in ac, y in ad)
            double an = 0.0;
            for (int k = 0; k < n; ++k) {
                int kn = (k + 1 == n) ? 0 : k + 1, kp = (k == 0) ? n - 1 : k - 1;
                double a0, a1;
                if (areaFromPositions) {
                    double2 xp = pos[st + kp], xn = pos[st + kn];
                    a0 = -wrap(xp.y - xn.y); a1 = wrap(xp.x - xn.x);
                    an += a0 * a0 + a1 * a1;
                } else {
                    const double* c = constraints + 6 * (size_t)(st + k);
                    a0 = c[0]; a1 = c[1];
                }
                ac[k] = a0; ad[k] = a1;
            }
            if (areaFromPositions && an > 0.0) {
                double ir = 1.0 / sqrt(an);
                for (int k = 0; k < n; ++k) { ac[k] *= ir; ad[k] *= ir; }
            }
            for (int k = 0; k < n; ++k) {
                int kn = (k + 1 == n) ? 0 : k + 1;
                double2 a = pos[st + k], b = pos[st + kn];
                double dx = wrap(b.x - a.x), dy = wrap(b.y - a.y);
                double len = sqrt(dx * dx + dy * dy);
                if (len < 1e-14) { tx[k] = 0.0; ty[k] = 0.0; di[k] = 1.0; }
                else { double il = 1.0 / len; tx[k] = dx * il; ty[k] = dy * il; di[k] = 2.0; }
            }
            double tx0 = tx[0], ty0 = ty[0];
            double txk = tx0, tyk = ty0;
            double2 f0 = force[st];
            double2 fk = f0;
            double ck0 = ac[0], ck1 = ad[0];
            double ak0 = ck0, ak1 = ck1;
            for (int k = 0; k < n; ++k) {
                int kn = (k + 1 == n) ? 0 : k + 1;
                double txn = (kn == 0) ? tx0 : tx[kn], tyn = (kn == 0) ? ty0 : ty[kn];
                double o = -(txk * txn + tyk * tyn);
                up[k] = o;
                lo[kn] = o;
                double2 f1 = (kn == 0) ? f0 : force[st + kn];
                double a0 = (kn == 0) ? ck0 : ac[kn], a1 = (kn == 0) ? ck1 : ad[kn];
                r0[k] = txk * (f1.x - fk.x) + tyk * (f1.y - fk.y);
                r1[k] = txk * (a0 - ak0) + tyk * (a1 - ak1);
                txk = txn; tyk = tyn; fk = f1; ak0 = a0; ak1 = a1;
            }
            bool ok = cyclic_solve(n, lo, di, up, 2, r0, r1, r1, cp, zs);
            if (ok) {
                double qF = 0.0, qq = 0.0;
                // reuse lo/up for F' and cp/zs for q
                double txp = tx[n - 1], typ = ty[n - 1], l0p = r0[n - 1], l1p = r1[n - 1];
                for (int k = 0; k < n; ++k) {
                    double txc = tx[k], tyc = ty[k], l0 = r0[k], l1 = r1[k];
                    // (J x)_k = -x_k t_k + x_{k-1} t_{k-1}
                    double jlx = -l0 * txc + l0p * txp, jly = -l0 * tyc + l0p * typ;
                    double jmx = -l1 * txc + l1p * txp, jmy = -l1 * tyc + l1p * typ;
                    double q0 = ac[k] - jmx, q1 = ad[k] - jmy;
                    double2 f = force[st + k];
                    double fx = f.x - jlx, fy = f.y - jly;
                    cp[k] = q0; zs[k] = q1;
                    lo[k] = fx; up[k] = fy;
                    qF += q0 * fx + q1 * fy;
                    qq += q0 * q0 + q1 * q1;
                    txp = txc; typ = tyc; l0p = l0; l1p = l1;
                }
                double mag = sqrt(qq);
                double coef = (mag > 1e-14) ? qF / qq : 0.0;
                for (int k = 0; k < n; ++k) {
                    double fx = lo[k] - coef * cp[k];
                    double fy = up[k] - coef * zs[k];
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
            { const Sum4 t4 = warp_sum4(sP, sV, sF, 0.0); sP = t4.x; sV = t4.y; sF = t4.z; }
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(&fire->P, sP);
                atomicAdd(&fire->vv, sV);
                atomicAdd(&fire->ff, sF);
            }
        }
        if ((threadIdx.x & 31) == 0) __threadfence();
        fire_pass_end(fire, rbNext);
    }
}

// vertices per thread that fit in shared memory for `arrays` scratch arrays
static int smem_vertices(int nmax, int arrays) {
    size_t per = (size_t)arrays * kConsThreads * sizeof(double);
    size_t cap = 200 * 1024;
    if (nmax <= 0 || (size_t)nmax * per > cap) return 0;
    return nmax;
}

// ------------------------------------------------------------------ SHAKE ----
// shakeProjectCUDA (model.cu:616-636; the kernel itself, src/shake.h, is not
// in the reference tree).  Restated as matrix SHAKE, Newton steps in the
// multipliers with the correction solved in FP32:
//   s_k = (|e_k|^2 - L^2) / 2  (edge k, e_k = wrap(x_{k+1} - x_k)),
//   s_A = A - A0               (shoelace of updatePolygonGeometryKernel),
//   converged when max(max_k |s_k| / L, |s_A|) < tol  (|s_k|/L ~ ||e_k| - L|);
//   otherwise x += G_ref^T l with (G(x) G_ref^T) l = -s, G_ref the
//   constraint gradients where SHAKE started (rows -+e_k, grad A).
// Residuals and the update are FP64 (the tolerance is met in FP64); the
// matrix (a cyclic tridiagonal block bordered by the area row and column)
// is formed and solved in FP32 by parallel cyclic reduction with a
// Sherman-Morrison correction for the cyclic corners.  Each FP32 solve is
// accurate to ~1e-5 relative, so the iteration still converges in about as
// many steps as an FP64 Newton iteration while the FP64 work per vertex
// and iteration drops to ~45 operations.  One warp per polygon.
__device__ __forceinline__ int pow2_at_least(int n) {
    int N = 4;
    while (N < n) N <<= 1;
    return N;
}

struct ShakeWS {
    double2 *xs, *r, *ar;
    float2 *rf, *arf, *ef;
    float *vr, *lam;
    float *pa, *pb, *pc, *p0, *p1, *p2;   // [2][N] each
};

__device__ __forceinline__ ShakeWS shake_ws(unsigned char* base, int NV, int N) {
    ShakeWS w;
    double2* d = reinterpret_cast<double2*>(base);
    w.xs = d; w.r = d + NV; w.ar = d + 2 * NV;
    float2* f2 = reinterpret_cast<float2*>(d + 3 * NV);
    w.rf = f2; w.arf = f2 + NV; w.ef = f2 + 2 * NV;
    float* f = reinterpret_cast<float*>(f2 + 3 * NV);
    w.vr = f; w.lam = f + NV;
    float* q = f + 2 * NV;
    w.pa = q; w.pb = q + 2 * N; w.pc = q + 4 * N; w.p0 = q + 6 * N; w.p1 = q + 8 * N; w.p2 = q + 10 * N;
    return w;
}
// bytes of one polygon's workspace (NV vertex slots, N PCR rows); a multiple
// of 16 whenever NV is even
__host__ __device__ constexpr size_t shake_ws_bytes(int NV, int N) {
    return (size_t)NV * (3 * 16 + 3 * 8 + 2 * 4) + (size_t)N * 12 * 4;
}

// Parallel cyclic reduction of N rows (arrays [2][N]: buffer 0 holds the
// system, buffer 1 is scratch) with three right-hand sides; leaves the
// solutions x = r / b in p0, p1, p2 (buffer 0).  One warp, rows strided.
// Its results only steer iterations whose residuals are FP64, so the fast
// FP32 division (2 ulp) is enough.
__device__ void pcr3f(float* pa, float* pb, float* pc, float* p0, float* p1, float* p2, int N) {
    const int lane = threadIdx.x & 31;
    int cur = 0;
    for (int d = 1; d < N; d <<= 1) {
        int nxt = cur ^ 1;
        const float *a = pa + cur * N, *b = pb + cur * N, *c = pc + cur * N;
        const float *r0 = p0 + cur * N, *r1 = p1 + cur * N, *r2 = p2 + cur * N;
        float *a2 = pa + nxt * N, *b2 = pb + nxt * N, *c2 = pc + nxt * N;
        float *s0 = p0 + nxt * N, *s1 = p1 + nxt * N, *s2 = p2 + nxt * N;
        for (int i = lane; i < N; i += 32) {
            int im = i - d, ip = i + d;
            float na = 0.f, nc = 0.f;
            float nb = b[i], n0 = r0[i], n1 = r1[i], n2 = r2[i];
            if (im >= 0) {
                float k1 = __fdividef(a[i], b[im]);
                na = -k1 * a[im];
                nb -= k1 * c[im];
                n0 -= k1 * r0[im]; n1 -= k1 * r1[im]; n2 -= k1 * r2[im];
            }
            if (ip < N) {
                float k2 = __fdividef(c[i], b[ip]);
                nc = -k2 * c[ip];
                nb -= k2 * a[ip];
                n0 -= k2 * r0[ip]; n1 -= k2 * r1[ip]; n2 -= k2 * r2[ip];
            }
            a2[i] = na; b2[i] = nb; c2[i] = nc; s0[i] = n0; s1[i] = n1; s2[i] = n2;
        }
        __syncwarp();
        cur = nxt;
    }
    const float *b = pb + cur * N, *r0 = p0 + cur * N, *r1 = p1 + cur * N, *r2 = p2 + cur * N;
    for (int i = lane; i < N; i += 32) {
        float ib = __fdividef(1.0f, b[i]);
        float x0 = r0[i] * ib, x1 = r1[i] * ib, x2 = r2[i] * ib;
        p0[i] = x0; p1[i] = x1; p2[i] = x2;
    }
    __syncwarp();
}

__device__ __forceinline__ void pcr3(ShakeWS& w, int N) { pcr3f(w.pa, w.pb, w.pc, w.p0, w.p1, w.p2, N); }

// Sherman-Morrison split of a cyclic tridiagonal system held in PCR buffer 0
// (rows 0..n-1; a = sub-, b = main, c = super-diagonal; the cyclic corners
// sit in a[0] and c[n-1]): the corners are removed and the correction vector
// is placed in p2.  False when gamma == 0.
__device__ __forceinline__ bool sm_split(float* pa, float* pb, float* pc, float* p2, int n,
                                         float& gamma, float& beta) {
    const int lane = threadIdx.x & 31;
    gamma = -pb[0];
    beta = pa[0];
    float alpha = pc[n - 1];
    bool ok = gamma != 0.f;
    __syncwarp();
    if (lane == 0 && ok) {
        pb[0] = pb[0] - gamma;
        pb[n - 1] = pb[n - 1] - alpha * beta / gamma;
        pa[0] = 0.f;
        pc[n - 1] = 0.f;
        p2[0] = gamma;
        p2[n - 1] = alpha;
    }
    __syncwarp();
    return ok;
}

// Position correction of one vertex, x_k += -l_k r_k + l_{k-1} r_{k-1} +
// mu ar_k, with the FP32 multipliers.  In FP64 while the correction is
// large.  Once the sum S of the terms' magnitudes is below 2^-26 (the later
// iterations, whose corrections are the FP32 solve's small leftovers) the
// FP32 form is used: its error, at most 6 * 2^-24 * S < 6e-15, is far below
// the 1e-12 position tolerance, and it turns 8 FP64 operations per vertex
// into the 2 adds.
__device__ __forceinline__ void shake_update(double2& x, float lk, float lp, float mu, double mu64,
                                             double2 rk, double2 rp, double2 ak, float2 rkf,
                                             float2 rpf, float2 akf) {
    const float S = fabsf(lk) * (fabsf(rkf.x) + fabsf(rkf.y)) +
                    fabsf(lp) * (fabsf(rpf.x) + fabsf(rpf.y)) +
                    fabsf(mu) * (fabsf(akf.x) + fabsf(akf.y));
    if (S < 0x1p-26f) {
        const float dx = -lk * rkf.x + lp * rpf.x + mu * akf.x;
        const float dy = -lk * rkf.y + lp * rpf.y + mu * akf.y;
        x.x += f2d_int(dx);
        x.y += f2d_int(dy);
    } else {
        const double l64 = f2d_int(lk), p64 = f2d_int(lp);
        x.x += -l64 * rk.x + p64 * rp.x + mu64 * ak.x;
        x.y += -l64 * rk.y + p64 * rp.y + mu64 * ak.y;
    }
}

// End of a SHAKE launch, reached by every thread of the block: the largest
// iteration count, and in the first attempt of a FIRE step (model.cpp:431-436)
// the last block to finish reads it and decides the retry.
__device__ __forceinline__ void shake_finish(int it, int* itersOut, Ctrl* fire,
                                             cudaGraphConditionalHandle retryCond) {
    // one atomic per block: same-address atomics from every warp queue up
    __shared__ int s_it;
    if (threadIdx.x == 0) s_it = 0;
    __syncthreads();
    if ((threadIdx.x & 31) == 0 && it > 0) atomicMax_block(&s_it, it);
    __syncthreads();
    if (threadIdx.x == 0 && s_it > 0) atomicMax(itersOut, s_it);
    if (fire) {
        if (threadIdx.x == 0) {
            __threadfence();
            unsigned int t = atomicAdd(&fire->shakeTicket, 1u);
            if (t == gridDim.x - 1) {
                __threadfence();
                int it1 = atomicOr(itersOut, 0);
                fire->shakeLast = it1;
                int nr = (it1 >= fire->shakeIter) ? 1 : 0;
                int go = (nr && fire->active) ? 1 : 0;
                fire->needRetry = nr;
                fire->retryGate = go;
                cudaGraphSetConditional(retryCond, (unsigned int)go);
            }
        }
    }
}

__global__ void __launch_bounds__(256, 4) k_shake(double2* __restrict__ pos, const int* __restrict__ start, int P,
                        const double* __restrict__ targetEdge,
                        const double* __restrict__ targetArea, int maxIter, double tol,
                        int* __restrict__ itersOut, double* __restrict__ scratch, int nmaxSmem,
                        Ctrl* fire, cudaGraphConditionalHandle retryCond,
                        double2* __restrict__ vel, const Ctrl* __restrict__ dtc,
                        const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    extern __shared__ __align__(16) unsigned char shake_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    int p = blockIdx.x * wpb + warp;
    int it = 0;
    if (p < P) {
        int st = start[p], n = start[p + 1] - st;
        if (n >= 3 && maxIter > 0) {
            ShakeWS w;
            int N;
            if (n <= nmaxSmem) {
                N = pow2_at_least(nmaxSmem);
                w = shake_ws(shake_smem + (size_t)warp * shake_ws_bytes(nmaxSmem, N), nmaxSmem, N);
            } else {
                // per-polygon slice of the global scratch (kScratchPerVertex
                // doubles per vertex >= shake_ws_bytes(n, 2n) / 8)
                N = pow2_at_least(n);
                w = shake_ws(reinterpret_cast<unsigned char*>(scratch + (size_t)kScratchPerVertex * st),
                             n, N);
            }
            const double L = targetEdge[p], A0 = targetArea[p];
            // worst < tol on bit patterns (tol <= 0 or NaN: never)
            const unsigned long long tolBits =
                tol > 0.0 ? (unsigned long long)__double_as_longlong(tol) : 0ull;
            const double invL = L > 0.0 ? 1.0 / L : 1.0;
            const double hInvL = 0.5 * invL, L2 = L * L;
            // local coordinates u_k = wrap(x_k - x_0) (no minimum images in
            // the iterations), the same arithmetic as k_shake_lanes
            const double2 o = pos[st];
            for (int k = lane; k < n; k += 32) {
                double2 xk = pos[st + k];
                w.xs[k] = make_double2(wrap(xk.x - o.x), wrap(xk.y - o.y));
            }
            __syncwarp();
            for (int k = lane; k < n; k += 32) {
                int kn = (k + 1 == n) ? 0 : k + 1, kp = (k == 0) ? n - 1 : k - 1;
                double2 xk = w.xs[k], xn = w.xs[kn], xp = w.xs[kp];
                double2 r = make_double2(xn.x - xk.x, xn.y - xk.y);
                double2 a = make_double2(0.5 * (xn.y - xp.y), 0.5 * (xp.x - xn.x));
                w.r[k] = r; w.ar[k] = a;
                w.rf[k] = make_float2(d2f_int(r.x), d2f_int(r.y));
                w.arf[k] = make_float2(d2f_int(a.x), d2f_int(a.y));
            }
            __syncwarp();
            for (; it < maxIter; ++it) {
                // residuals (FP64)
                // worst residual as the bit pattern of a non-negative double
                // (patterns order like the values; NaN sorts highest)
                unsigned long long worst = 0ull;
                double area = 0.0;
                bool nonfinite = false;
                for (int k = lane; k < n; k += 32) {
                    int kn = (k + 1 == n) ? 0 : k + 1;
                    double2 xk = w.xs[k], xn = w.xs[kn];
                    double ex = xn.x - xk.x, ey = xn.y - xk.y;
                    double q = ex * ex + ey * ey - L2;     // 2 s_k
                    unsigned long long qb = abs_bits(q * hInvL);
                    if (qb > worst) worst = qb;
                    area += ey * (xn.x + xk.x);   // halved after the sum (exact)
                    w.ef[k] = make_float2(d2f_int(ex), d2f_int(ey));
                    w.lam[k] = d2f_int(-q) * 0.5f;   // right-hand side -s_k until the rows are built
                }
                worst = warp_max_u64(worst);
                area = warp_sum(area) * 0.5;
                nonfinite = __any_sync(PCP_FULL, nonfinite);
                double sA = area - A0;
                {
                    unsigned long long qa = abs_bits(sA);
                    if (qa > worst) worst = qa;
                }
                if (nonfinite || !finite_bits(worst)) { it = maxIter; break; }
                if (worst < tolBits) break;
                __syncwarp();
                // rows of G(x) G_ref^T (FP32) into PCR buffer 0
                float dc = 0.f;
                for (int k = lane; k < n; k += 32) {
                    int kn = (k + 1 == n) ? 0 : k + 1, kp = (k == 0) ? n - 1 : k - 1;
                    float2 e = w.ef[k], rk = w.rf[k], rn = w.rf[kn], rp = w.rf[kp];
                    float2 an = w.arf[kn], ak = w.arf[k];
                    // current area gradient at k and k+1 from the FP32 edge
                    // vectors: (x_k+1 - x_k-1) / 2 rotated, as in the residual
                    float2 ep = w.ef[kp], en = w.ef[kn];
                    float2 ck = make_float2(0.5f * (e.y + ep.y), -0.5f * (e.x + ep.x));
                    float2 cn = make_float2(0.5f * (en.y + e.y), -0.5f * (en.x + e.x));
                    w.pb[k] = 2.0f * (e.x * rk.x + e.y * rk.y);
                    w.pc[k] = -(e.x * rn.x + e.y * rn.y);
                    w.pa[k] = -(e.x * rp.x + e.y * rp.y);
                    w.p0[k] = w.lam[k];
                    w.p1[k] = e.x * (an.x - ak.x) + e.y * (an.y - ak.y);
                    w.p2[k] = 0.f;
                    w.vr[k] = (cn.x - ck.x) * rk.x + (cn.y - ck.y) * rk.y;
                    dc += ck.x * ak.x + ck.y * ak.y;
                }
                for (int k = n + lane; k < N; k += 32) {
                    w.pa[k] = 0.f; w.pb[k] = 1.f; w.pc[k] = 0.f;
                    w.p0[k] = 0.f; w.p1[k] = 0.f; w.p2[k] = 0.f;
                }
                for (int o = 16; o > 0; o >>= 1) dc += __shfl_xor_sync(PCP_FULL, dc, o);
                __syncwarp();
                // Sherman-Morrison: move the cyclic corners out of the matrix
                float gamma = -w.pb[0];
                float beta = w.pa[0], alpha = w.pc[n - 1];
                bool bad = !(gamma != 0.f);
                __syncwarp();
                if (lane == 0 && !bad) {
                    w.pb[0] = w.pb[0] - gamma;
                    w.pb[n - 1] = w.pb[n - 1] - alpha * beta / gamma;
                    w.pa[0] = 0.f;
                    w.pc[n - 1] = 0.f;
                    w.p2[0] = gamma;
                    w.p2[n - 1] = alpha;
                }
                __syncwarp();
                if (bad) { it = maxIter; break; }
                pcr3(w, N);
                float y0 = w.p0[0], yl = w.p0[n - 1], z0 = w.p1[0], zl = w.p1[n - 1];
                float s0 = w.p2[0], sl = w.p2[n - 1];
                float den = 1.f + s0 + beta * sl / gamma;
                float fy = (y0 + beta * yl / gamma) / den;
                float fz = (z0 + beta * zl / gamma) / den;
                __syncwarp();
                float vy = 0.f, vz = 0.f;
                for (int k = lane; k < n; k += 32) {
                    float s = w.p2[k];
                    float yk = w.p0[k] - fy * s, zk = w.p1[k] - fz * s;
                    w.p0[k] = yk; w.p1[k] = zk;
                    vy += w.vr[k] * yk; vz += w.vr[k] * zk;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    vy += __shfl_xor_sync(PCP_FULL, vy, o);
                    vz += __shfl_xor_sync(PCP_FULL, vz, o);
                }
                float mu = (-d2f_int(sA) - vy) / (dc - vz);
                bool finite = isfinite(mu);
                __syncwarp();
                for (int k = lane; k < n; k += 32) {
                    float l = w.p0[k] - mu * w.p1[k];
                    w.lam[k] = l;
                    finite = finite && isfinite(l);
                }
                if (!__all_sync(PCP_FULL, finite)) { it = maxIter; break; }
                __syncwarp();
                // x_k += -l_k r_k + l_{k-1} r_{k-1} + mu ar_k
                double mu64 = f2d_int(mu);
                for (int k = lane; k < n; k += 32) {
                    int kp = (k == 0) ? n - 1 : k - 1;
                    double2 x = w.xs[k];
                    shake_update(x, w.lam[k], w.lam[kp], mu, mu64, w.r[k], w.r[kp], w.ar[k], w.rf[k],
                                 w.rf[kp], w.arf[k]);
                    w.xs[k] = x;
                }
                __syncwarp();
            }
            __syncwarp();   // every lane has read pos[st] (o) before it is rewritten
            if (vel) {
                // FIRE step: v += wrap(x_shake - x_before) / dt, the reference's
                // rederivation from the displacement (model.cpp:436-438); a retry
                // adds its own displacement on top
                const double idt = 1.0 / dtc->dt;
                for (int k = lane; k < n; k += 32) {
                    double2 x = make_double2(o.x + w.xs[k].x, o.y + w.xs[k].y), y = pos[st + k],
                            v = vel[st + k];
                    x = make_double2(frac_unit(x.x), frac_unit(x.y));
                    v.x += wrap(x.x - y.x) * idt;
                    v.y += wrap(x.y - y.y) * idt;
                    vel[st + k] = v;
                    pos[st + k] = x;
                }
            } else {
                for (int k = lane; k < n; k += 32) {
                    double2 v = make_double2(o.x + w.xs[k].x, o.y + w.xs[k].y);
                    pos[st + k] = make_double2(frac_unit(v.x), frac_unit(v.y));
                }
            }
        }
    }
    shake_finish(it, itersOut, fire, retryCond);
}

__device__ __forceinline__ double2 shfl2(double2 v, int src) {
    return make_double2(__shfl_sync(PCP_FULL, v.x, src), __shfl_sync(PCP_FULL, v.y, src));
}
__device__ __forceinline__ float2 shfl2(float2 v, int src) {
    return make_float2(__shfl_sync(PCP_FULL, v.x, src), __shfl_sync(PCP_FULL, v.y, src));
}

// pcr3f with row i held by lane i (rows 0..N-1, N <= 32; partner rows read
// by shuffles), expression for expression: leaves the solutions in q0..q2.
__device__ __forceinline__ void lanes_pcr3(float a, float b, float c, float& q0, float& q1,
                                           float& q2, int N, int lane) {
    for (int d = 1; d < N; d <<= 1) {
        const float am = __shfl_up_sync(PCP_FULL, a, d), bm = __shfl_up_sync(PCP_FULL, b, d);
        const float cm = __shfl_up_sync(PCP_FULL, c, d);
        const float m0 = __shfl_up_sync(PCP_FULL, q0, d), m1 = __shfl_up_sync(PCP_FULL, q1, d);
        const float m2 = __shfl_up_sync(PCP_FULL, q2, d);
        const float ap = __shfl_down_sync(PCP_FULL, a, d), bp = __shfl_down_sync(PCP_FULL, b, d);
        const float cp = __shfl_down_sync(PCP_FULL, c, d);
        const float p0 = __shfl_down_sync(PCP_FULL, q0, d), p1 = __shfl_down_sync(PCP_FULL, q1, d);
        const float p2 = __shfl_down_sync(PCP_FULL, q2, d);
        float na = 0.f, nc = 0.f;
        float nb = b, n0 = q0, n1 = q1, n2 = q2;
        if (lane - d >= 0) {
            float k1 = __fdividef(a, bm);
            na = -k1 * am;
            nb -= k1 * cm;
            n0 -= k1 * m0; n1 -= k1 * m1; n2 -= k1 * m2;
        }
        if (lane + d < N) {
            float k2 = __fdividef(c, bp);
            nc = -k2 * cp;
            nb -= k2 * ap;
            n0 -= k2 * p0; n1 -= k2 * p1; n2 -= k2 * p2;
        }
        a = na; b = nb; c = nc; q0 = n0; q1 = n1; q2 = n2;
    }
    float ib = __fdividef(1.0f, b);
    float x0 = q0 * ib, x1 = q1 * ib, x2 = q2 * ib;
    q0 = x0; q1 = x1; q2 = x2;
}

// Unit tangent t_k of edge (k, k+1) of the wrapped positions held one vertex
// per lane (kernels.cuh:399: zero for an edge shorter than 1e-14).
__device__ __forceinline__ void lanes_tangent(double2 x, int kn, double2& t, double2& d) {
    const double2 xn = shfl2(x, kn);
    t = make_double2(0.0, 0.0);
    double dx = wrap(xn.x - x.x), dy = wrap(xn.y - x.y);
    d = make_double2(dx, dy);
    double len2 = dx * dx + dy * dy;
    // len2 >= 0, so its bit pattern orders like its value (NaN counts as long)
    bool ok = (unsigned long long)__double_as_longlong(len2) >=
              (unsigned long long)__double_as_longlong(1e-28);
    if (ok) { double il = rsqrt(len2); t = make_double2(dx * il, dy * il); }
}

// Unit area gradient of the polygon at vertex k, (x_k+1 - x_k-1) / 2 rotated
// and normalised over the polygon (updatePolygonGeometryKernel,
// kernels.cuh:303,313), one vertex per lane, from the edge vectors
// d_k = wrap(x_k+1 - x_k) that lanes_tangent forms: x_k+1 - x_k-1 =
// d_k-1 + d_k (one add instead of a wrapped difference).  Lanes >= n (live
// false) add nothing to the normalisation.
__device__ __forceinline__ void lanes_area_gradient(double2 d, bool live, int kp, double2& q) {
    const double2 dp = shfl2(d, kp);
    q = make_double2(dp.y + d.y, -dp.x - d.x);
    double an = live ? q.x * q.x + q.y * q.y : 0.0;
    an = warp_sum(an);
    // an > 0 on the bit pattern (an >= 0, or NaN)
    const unsigned long long anB = (unsigned long long)__double_as_longlong(an);
    double ir = (anB > 0ull && anB <= 0x7FF0000000000000ull) ? rsqrt(an) : 1.0;
    q = make_double2(q.x * ir, q.y * ir);
}

// k_shake for polygons of at most 32 vertices: one vertex per lane, the
// positions, reference gradients and rows held in registers, neighbours'
// values and the parallel cyclic reduction's partner rows read by warp
// shuffles instead of a shared-memory workspace.  Operation for operation the
// arithmetic of k_shake (same expressions, same reduction trees), so the two
// give bit-identical positions and iteration counts.  Lanes n..31 hold
// identity rows and contribute zero to every sum.
__global__ void __launch_bounds__(128, 7) k_shake_lanes(double2* __restrict__ pos,
                        const int* __restrict__ start, int P,
                        const double* __restrict__ targetEdge,
                        const double* __restrict__ targetArea, int maxIter, double tol,
                        int* __restrict__ itersOut, Ctrl* fire,
                        cudaGraphConditionalHandle retryCond, double2* __restrict__ vel,
                        const Ctrl* __restrict__ dtc, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    // 1/dt once per block (a DDIV is a dozen FP64 warp instructions)
    __shared__ double s_idt;
    if (vel && threadIdx.x == 0) s_idt = 1.0 / dtc->dt;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int it = 0;
    if (p < P) {
        const int st = start[p], n = start[p + 1] - st;
        if (n >= 3 && n <= 32 && maxIter > 0) {
            const bool live = lane < n;
            const int kn = (lane + 1 >= n) ? 0 : lane + 1;
            const int kp = (lane == 0) ? n - 1 : lane - 1;
            const int N = pow2_at_least(n);
            const double L = targetEdge[p], A0 = targetArea[p];
            // tol > 0 and L > 0 on the bit patterns (positive, up to +inf)
            const long long tolB = __double_as_longlong(tol), LB = __double_as_longlong(L);
            const unsigned long long tolBits =
                (tolB > 0 && tolB <= 0x7FF0000000000000ll) ? (unsigned long long)tolB : 0ull;
            const double invL = (LB > 0 && LB <= 0x7FF0000000000000ll) ? 1.0 / L : 1.0;
            const double hInvL = 0.5 * invL, L2 = L * L;
            // local coordinates u_k = wrap(x_k - x_0): the iterations need no
            // minimum images (a polygon spans far less than half the box)
            double2 x;
            {
                const double2 x0 = live ? pos[st + lane] : make_double2(0.0, 0.0);
                const double2 o = shfl2(x0, 0);
                x = live ? make_double2(wrap(x0.x - o.x), wrap(x0.y - o.y)) : make_double2(0.0, 0.0);
            }
            double2 r, ar;
            {
                const double2 xn = shfl2(x, kn), xp = shfl2(x, kp);
                r = make_double2(xn.x - x.x, xn.y - x.y);
                ar = make_double2(0.5 * (xn.y - xp.y), 0.5 * (xp.x - xn.x));
            }
            const float2 rf = make_float2(d2f_int(r.x), d2f_int(r.y));
            const float2 arf = make_float2(d2f_int(ar.x), d2f_int(ar.y));
            const double2 rp = shfl2(r, kp);
            const float2 rnf = shfl2(rf, kn), rpf = shfl2(rf, kp), anf = shfl2(arf, kn);
            for (; it < maxIter; ++it) {
                // residuals (FP64): q = |e|^2 - L^2 = 2 s_k
                const double2 xn = shfl2(x, kn);
                const double ex = xn.x - x.x, ey = xn.y - x.y;
                const double q = ex * ex + ey * ey - L2;
                unsigned long long worst = live ? abs_bits(q * hInvL) : 0ull;
                double area = live ? ey * (xn.x + x.x) : 0.0;
                worst = warp_max_u64(worst);
                // (sum * 0.5 is exact: one rounding either way)
                const double sA = fma(warp_sum(area), 0.5, -A0);
                {
                    unsigned long long qa = abs_bits(sA);
                    if (qa > worst) worst = qa;
                }
                if (!finite_bits(worst)) { it = maxIter; break; }
                if (worst < tolBits) break;
                // rows of G(x) G_ref^T (FP32)
                const float2 e = make_float2(d2f_int(ex), d2f_int(ey));
                const float2 ep = shfl2(e, kp), en = shfl2(e, kn);
                float a = 0.f, b = 1.f, c = 0.f, q0 = 0.f, q1 = 0.f, q2 = 0.f, vr = 0.f, dc = 0.f;
                if (live) {
                    const float2 ck = make_float2(0.5f * (e.y + ep.y), -0.5f * (e.x + ep.x));
                    const float2 cn = make_float2(0.5f * (en.y + e.y), -0.5f * (en.x + e.x));
                    b = 2.0f * (e.x * rf.x + e.y * rf.y);
                    c = -(e.x * rnf.x + e.y * rnf.y);
                    a = -(e.x * rpf.x + e.y * rpf.y);
                    q0 = d2f_int(-q) * 0.5f;
                    q1 = e.x * (anf.x - arf.x) + e.y * (anf.y - arf.y);
                    vr = (cn.x - ck.x) * rf.x + (cn.y - ck.y) * rf.y;
                    dc += ck.x * arf.x + ck.y * arf.y;
                }
                for (int o = 16; o > 0; o >>= 1) dc += __shfl_xor_sync(PCP_FULL, dc, o);
                // Sherman-Morrison: move the cyclic corners out of the matrix
                const float gamma = -__shfl_sync(PCP_FULL, b, 0);
                const float beta = __shfl_sync(PCP_FULL, a, 0);
                const float alpha = __shfl_sync(PCP_FULL, c, n - 1);
                if (!(gamma != 0.f)) { it = maxIter; break; }
                if (lane == 0) { b = b - gamma; a = 0.f; q2 = gamma; }
                if (lane == n - 1) { b = b - alpha * beta / gamma; c = 0.f; q2 = alpha; }
                lanes_pcr3(a, b, c, q0, q1, q2, N, lane);
                const float y0 = __shfl_sync(PCP_FULL, q0, 0), yl = __shfl_sync(PCP_FULL, q0, n - 1);
                const float z0 = __shfl_sync(PCP_FULL, q1, 0), zl = __shfl_sync(PCP_FULL, q1, n - 1);
                const float s0 = __shfl_sync(PCP_FULL, q2, 0), sl = __shfl_sync(PCP_FULL, q2, n - 1);
                float den = 1.f + s0 + beta * sl / gamma;
                float fy = (y0 + beta * yl / gamma) / den;
                float fz = (z0 + beta * zl / gamma) / den;
                float vy = 0.f, vz = 0.f;
                const float yk = q0 - fy * q2, zk = q1 - fz * q2;
                if (live) { vy += vr * yk; vz += vr * zk; }
                for (int o = 16; o > 0; o >>= 1) {
                    vy += __shfl_xor_sync(PCP_FULL, vy, o);
                    vz += __shfl_xor_sync(PCP_FULL, vz, o);
                }
                float mu = (-d2f_int(sA) - vy) / (dc - vz);
                bool finite = isfinite(mu);
                const float l = yk - mu * zk;
                if (live) finite = finite && isfinite(l);
                if (!__all_sync(PCP_FULL, finite)) { it = maxIter; break; }
                const float lp = __shfl_sync(PCP_FULL, l, kp);
                double mu64 = f2d_int(mu);
                if (live) shake_update(x, l, lp, mu, mu64, r, rp, ar, rf, rpf, arf);
            }
            // the positions SHAKE started from, read again (fewer live registers
            // through the iterations); lane 0's is x_0
            const double2 x0 = live ? pos[st + lane] : make_double2(0.0, 0.0);
            const double2 o = shfl2(x0, 0);
            if (live) {
                const double2 y = make_double2(frac_unit(o.x + x.x), frac_unit(o.y + x.y));
                if (vel) {
                    // FIRE step: v += wrap(x_shake - x_before) / dt, the
                    // reference's rederivation from the displacement
                    // (model.cpp:436-438); a retry adds its own displacement
                    const double idt = s_idt;
                    double2 v = vel[st + lane];
                    v.x += wrap(y.x - x0.x) * idt;
                    v.y += wrap(y.y - x0.y) * idt;
                    vel[st + lane] = v;
                }
                pos[st + lane] = y;
            }
        }
    }
    shake_finish(it, itersOut, fire, retryCond);
}

// The unit edge tangents and unit area gradients (normalised over the
// polygon) of the positions, one polygon per warp, stored for
// k_project_lanes as pre[i] = t_i, pre[V + i] = q_i, and the edge vectors
// wrap(x_next - x_i) for the overlap force as pre[2V + i].  The FIRE step
// runs this beside the end of the contact search, so that the force and the
// projection on the step's critical path start from them.
__global__ void __launch_bounds__(128) k_project_pre(const double2* __restrict__ pos,
                                                     const int* __restrict__ start, int P,
                                                     double2* __restrict__ pre, int V,
                                                     const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    const int lane = threadIdx.x & 31;
    const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (p >= P) return;
    const int st = start[p], n = start[p + 1] - st;
    // (polygons of 1 or 2 vertices too: the force may take their edges)
    if (n < 1 || n > 32) return;
    const bool live = lane < n;
    const int kn = (lane + 1 >= n) ? 0 : lane + 1;
    const int kp = (lane == 0) ? n - 1 : lane - 1;
    const double2 x = live ? pos[st + lane] : make_double2(0.0, 0.0);
    double2 t, q, d;
    lanes_tangent(x, kn, t, d);
    lanes_area_gradient(d, live, kp, q);
    if (live) { pre[st + lane] = t; pre[V + st + lane] = q; pre[2 * (size_t)V + st + lane] = d; }
}

// launch_project's choice: thread per polygon for at least 128 polygons per
// SM, else warp per polygon, in registers for polygons of up to 32 vertices
bool project_uses_lanes(int P, int nmax) { return nmax <= 32 && P < 128 * sm_count(); }

cudaError_t launch_project_pre(const double2* pos, const int* start, int P, int nmax,
                               double2* pre, int V, const int* gate, cudaStream_t st) {
    if (P <= 0 || !project_uses_lanes(P, nmax)) return cudaSuccess;
    launch_k(k_project_pre, dim3(nblk(P, 4)), dim3(128), 0, st, pos, start, P, pre, V, gate);
    return cudaGetLastError();
}

cudaError_t launch_shake(double2* pos, const int* start, int P, int nmax, const double* targetEdge,
                         const double* targetArea, int maxIter, double tol, int* maxItersOut,
                         double* scratch, int V, const int* gate, cudaStream_t st, Ctrl* fire,
                         cudaGraphConditionalHandle retryCond, double2* vel, const Ctrl* dtc) {
    (void)V;
    if (P <= 0) return cudaSuccess;
    if (nmax <= 32) {
        const int wpb = 4;
        launch_k(k_shake_lanes, dim3(nblk(P, wpb)), dim3(32 * wpb), 0, st, pos, start, P, targetEdge,
                 targetArea, maxIter, tol, maxItersOut, fire, retryCond, vel, dtc, gate);
        return cudaGetLastError();
    }
    // per-warp workspace in shared memory when it fits (polygons up to ~1000
    // vertices), else a per-polygon slice of the global scratch
    int nv = (nmax + 1) & ~1;          // even, so each workspace stays 16-byte aligned
    int N = 4;
    while (N < nv) N <<= 1;
    size_t per = shake_ws_bytes(nv, N);
    int wpb = 8;
    while (wpb > 1 && per * wpb > 200 * 1024) wpb >>= 1;
    int nmaxSmem = nv;
    if (per * wpb > 200 * 1024) { nmaxSmem = 0; per = 0; wpb = 8; }
    size_t smem = per * wpb;
    launch_k(k_shake, dim3(nblk(P, wpb)), dim3(32 * wpb), smem, st, pos, start, P, targetEdge, targetArea, maxIter,
                                                   tol, maxItersOut, scratch, nmaxSmem, fire,
                                                   retryCond, vel, dtc, gate);
    return cudaGetLastError();
}

// Warp-per-polygon form of the projection for systems with few polygons
// (4096 polygons give only 128 warps of thread-per-polygon work): per-vertex
// work runs across the lanes; (J^T J) x = J^T v is solved by mixed-precision
// iterative refinement -- the residual J^T (v - J x) and every update are
// FP64, each correction is solved in FP32 by parallel cyclic reduction
// (Sherman-Morrison split of the cyclic corners, rows padded to a power of
// two).  Each FP32 solve gains ~kappa * 6e-8 (kappa(J^T J) ~ (n/pi)^2), so
// three rounds reach FP64 accuracy for polygons of up to a few hundred
// vertices.  Same mathematics as k_project.
//
// areaFromPositions: take the unit area gradient from the positions (the
// normalised areaComp of updatePolygonGeometryKernel, kernels.cuh:303,313)
// instead of the constraints array; the device-resident FIRE step uses this
// because its positions are those the reference's last geometry call saw.
constexpr int kProjRounds = 3;

struct ProjWS {
    double2 *t, *f, *q;            // unit edges, F' and q (FP64)
    float2* tf;                    // unit edges (FP32)
    float *mb, *mc;                // J^T J diagonal and super-diagonal (FP32)
    float *pa, *pb, *pc, *p0, *p1, *p2;   // PCR rows [2][N]
};
__device__ __forceinline__ ProjWS proj_ws(unsigned char* base, int NV, int N) {
    ProjWS w;
    double2* d = reinterpret_cast<double2*>(base);
    w.t = d; w.f = d + NV; w.q = d + 2 * NV;
    w.tf = reinterpret_cast<float2*>(d + 3 * NV);
    float* f = reinterpret_cast<float*>(w.tf + NV);
    w.mb = f; w.mc = f + NV;
    float* q = f + 2 * NV;
    w.pa = q; w.pb = q + 2 * N; w.pc = q + 4 * N; w.p0 = q + 6 * N; w.p1 = q + 8 * N; w.p2 = q + 10 * N;
    return w;
}
// bytes of one polygon's workspace; a multiple of 16 when NV is even
__host__ __device__ constexpr size_t proj_ws_bytes(int NV, int N) {
    return (size_t)NV * (48 + 8 + 8) + (size_t)N * 12 * 4;
}

__global__ void __launch_bounds__(256, 4) k_project_warp(const double2* __restrict__ pos, const int* __restrict__ start,
                               int P, const double* __restrict__ constraints,
                               double2* __restrict__ force, double* __restrict__ scratch,
                               int nmaxSmem, int areaFromPositions, Ctrl* fire,
                               double2* __restrict__ vel, int mainPass, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    extern __shared__ __align__(16) unsigned char proj_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    int p = blockIdx.x * wpb + warp;
    bool proceed = false, rbNext = false;
    double dt = 0.0;
    if (fire) {
        const FireView fv = fire_view_proj(fire, mainPass);
        if (mainPass && fv.rbNext) return;     // the rollback body redoes the pass
        proceed = fv.proceed; rbNext = fv.rbNext; dt = fv.dt;
    }
    double sP = 0.0, sV = 0.0, sF = 0.0;
    unsigned long long mF = 0ull;      // max |F component| as a bit pattern
    bool bad = false;
    if (p < P) {
        int st = start[p], n = start[p + 1] - st;
        if (n >= 3) {
            ProjWS w;
            int N;
            if (n <= nmaxSmem) {
                N = pow2_at_least(nmaxSmem);
                w = proj_ws(proj_smem + (size_t)warp * proj_ws_bytes(nmaxSmem, N), nmaxSmem, N);
            } else {
                N = pow2_at_least(n);
                w = proj_ws(reinterpret_cast<unsigned char*>(scratch + (size_t)kScratchPerVertex * st),
                            n, N);
            }
            double an = 0.0;
            for (int k = lane; k < n; k += 32) {
                int kn = (k + 1 == n) ? 0 : k + 1, kp = (k == 0) ? n - 1 : k - 1;
                double2 xk = pos[st + k], xn = pos[st + kn];
                double dx = wrap(xn.x - xk.x), dy = wrap(xn.y - xk.y);
                double len2 = dx * dx + dy * dy;
                double2 t = make_double2(0.0, 0.0);
                // |e| >= 1e-14 (kernels.cuh:399); len2 >= 0, so its bit
                // pattern orders like its value (NaN counts as long)
                bool ok = (unsigned long long)__double_as_longlong(len2) >=
                          (unsigned long long)__double_as_longlong(1e-28);
                if (ok) { double il = rsqrt(len2); t = make_double2(dx * il, dy * il); }
                w.t[k] = t;
                w.tf[k] = make_float2(d2f_int(t.x), d2f_int(t.y));
                w.mb[k] = ok ? 2.0f : 1.0f;
                w.f[k] = force[st + k];
                double2 a;
                if (areaFromPositions) {
                    double2 xp = pos[st + kp];
                    a = make_double2(-wrap(xp.y - xn.y), wrap(xp.x - xn.x));
                    an += a.x * a.x + a.y * a.y;
                } else {
                    const double* c = constraints + 6 * (size_t)(st + k);
                    a = make_double2(c[0], c[1]);
                }
                w.q[k] = a;
            }
            if (areaFromPositions) {
                an = warp_sum(an);
                double ir = an > 0.0 ? rsqrt(an) : 1.0;
                for (int k = lane; k < n; k += 32) {
                    double2 a = w.q[k];
                    w.q[k] = make_double2(a.x * ir, a.y * ir);
                }
            }
            __syncwarp();
            for (int k = lane; k < n; k += 32) {
                int kn = (k + 1 == n) ? 0 : k + 1;
                double2 t = w.t[k], tn = w.t[kn];
                w.mc[k] = d2f_int(-(t.x * tn.x + t.y * tn.y));
            }
            __syncwarp();
            for (int round = 0; round < kProjRounds && !bad; ++round) {
                // residual right-hand sides J^T F', J^T q (FP64) and the FP32 rows
                for (int k = lane; k < n; k += 32) {
                    int kn = (k + 1 == n) ? 0 : k + 1, kp = (k == 0) ? n - 1 : k - 1;
                    double2 t = w.t[k], f0 = w.f[k], f1 = w.f[kn], a0 = w.q[k], a1 = w.q[kn];
                    w.p0[k] = d2f_int(t.x * (f1.x - f0.x) + t.y * (f1.y - f0.y));
                    w.p1[k] = d2f_int(t.x * (a1.x - a0.x) + t.y * (a1.y - a0.y));
                    w.p2[k] = 0.f;
                    w.pb[k] = w.mb[k];
                    w.pc[k] = w.mc[k];
                    w.pa[k] = w.mc[kp];
                }
                for (int k = n + lane; k < N; k += 32) {
                    w.pa[k] = 0.f; w.pb[k] = 1.f; w.pc[k] = 0.f;
                    w.p0[k] = 0.f; w.p1[k] = 0.f; w.p2[k] = 0.f;
                }
                __syncwarp();
                float gamma, beta;
                if (!sm_split(w.pa, w.pb, w.pc, w.p2, n, gamma, beta)) { bad = true; break; }
                pcr3f(w.pa, w.pb, w.pc, w.p0, w.p1, w.p2, N);
                float den = 1.f + w.p2[0] + beta * w.p2[n - 1] / gamma;
                float fl = (w.p0[0] + beta * w.p0[n - 1] / gamma) / den;
                float fm = (w.p1[0] + beta * w.p1[n - 1] / gamma) / den;
                __syncwarp();
                for (int k = lane; k < n; k += 32) {
                    float s = w.p2[k];
                    w.p0[k] -= fl * s;
                    w.p1[k] -= fm * s;
                }
                __syncwarp();
                // F' -= J lambda, q -= J mu with (J x)_k = -x_k t_k + x_{k-1} t_{k-1}.
                // An error in the direction of an update that leaves span(J)
                // is invisible to the next residual J^T F', so the first
                // (full-size) update uses the FP64 tangents; the later ones
                // are corrections of relative size ~1e-5 and take FP32
                // products (error ~1e-7 of the correction), added in FP64.
                if (round == 0) {
                    for (int k = lane; k < n; k += 32) {
                        int kp = (k == 0) ? n - 1 : k - 1;
                        double2 t = w.t[k], tp = w.t[kp];
                        double l0 = f2d_int(w.p0[k]), l0p = f2d_int(w.p0[kp]);
                        double l1 = f2d_int(w.p1[k]), l1p = f2d_int(w.p1[kp]);
                        double2 f = w.f[k], a = w.q[k];
                        f.x -= -l0 * t.x + l0p * tp.x; f.y -= -l0 * t.y + l0p * tp.y;
                        a.x -= -l1 * t.x + l1p * tp.x; a.y -= -l1 * t.y + l1p * tp.y;
                        w.f[k] = f; w.q[k] = a;
                    }
                } else {
                    for (int k = lane; k < n; k += 32) {
                        int kp = (k == 0) ? n - 1 : k - 1;
                        float2 t = w.tf[k], tp = w.tf[kp];
                        float l0 = w.p0[k], l0p = w.p0[kp];
                        float l1 = w.p1[k], l1p = w.p1[kp];
                        double2 f = w.f[k], a = w.q[k];
                        f.x += f2d_int(l0 * t.x - l0p * tp.x); f.y += f2d_int(l0 * t.y - l0p * tp.y);
                        a.x += f2d_int(l1 * t.x - l1p * tp.x); a.y += f2d_int(l1 * t.y - l1p * tp.y);
                        w.f[k] = f; w.q[k] = a;
                    }
                }
                __syncwarp();
            }
            if (!bad) {
                double qF = 0.0, qq = 0.0;
                for (int k = lane; k < n; k += 32) {
                    double2 f = w.f[k], q = w.q[k];
                    qF += q.x * f.x + q.y * f.y;
                    qq += q.x * q.x + q.y * q.y;
                }
                {
                    const double2 t2 = warp_sum2(qF, qq);
                    qF = t2.x; qq = t2.y;
                }
                // sqrt(qq) > 1e-14 (kernels.cuh:464)
                double coef = (qq > 1e-28) ? qF / qq : 0.0;
                for (int k = lane; k < n; k += 32) {
                    double2 f = w.f[k], q = w.q[k];
                    double fx = f.x - coef * q.x, fy = f.y - coef * q.y;
                    force[st + k] = make_double2(fx, fy);
                    mF = max_abs_bits(mF, fx, fy);
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
            }
        } else {
            for (int k = lane; k < n; k += 32) {
                double2 f = force[st + k];
                mF = max_abs_bits(mF, f.x, f.y);
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
        if (bad && lane == 0) atomicOr(&fire->flags, kFlagNonFinite);
        mF = warp_max_u64(mF);
        if (lane == 0 && mF) atomicMax(reinterpret_cast<unsigned long long*>(&fire->maxF), mF);
        if (proceed) {
            { const Sum4 t4 = warp_sum4(sP, sV, sF, 0.0); sP = t4.x; sV = t4.y; sF = t4.z; }
            if (lane == 0) {
                atomicAdd(&fire->P, sP);
                atomicAdd(&fire->vv, sV);
                atomicAdd(&fire->ff, sF);
            }
        }
        if (lane == 0) __threadfence();
        fire_pass_end(fire, rbNext);
    }
}

// k_project_warp for polygons of at most 32 vertices: one vertex per lane,
// tangents, F', q and the rows in registers, neighbours' values and the
// reduction's partner rows read by shuffles (no shared-memory workspace, no
// warp barriers).  The same mathematics and rounds as k_project_warp.
__global__ void __launch_bounds__(128, 7) k_project_lanes(const double2* __restrict__ pos,
                               const int* __restrict__ start, int P,
                               const double* __restrict__ constraints,
                               double2* __restrict__ force, int areaFromPositions, Ctrl* fire,
                               double2* __restrict__ vel, int mainPass,
                               const double2* __restrict__ pre, int V,
                               const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    const int lane = threadIdx.x & 31;
    const int p = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    bool proceed = false, rbNext = false;
    double dt = 0.0;
    if (fire) {
        const FireView fv = fire_view_proj(fire, mainPass);
        if (mainPass && fv.rbNext) return;     // the rollback body redoes the pass
        proceed = fv.proceed; rbNext = fv.rbNext; dt = fv.dt;
    }
    double sP = 0.0, sV = 0.0, sF = 0.0;
    unsigned long long mF = 0ull;      // max |F component| as a bit pattern
    bool bad = false;
    if (p < P) {
        const int st = start[p], n = start[p + 1] - st;
        const bool live = lane < n;
        double2 f = live ? force[st + lane] : make_double2(0.0, 0.0);
        if (n >= 3 && n <= 32) {
            const int kn = (lane + 1 >= n) ? 0 : lane + 1;
            const int kp = (lane == 0) ? n - 1 : lane - 1;
            const int N = pow2_at_least(n);
            double2 t, q;
            if (pre) {
                t = live ? pre[st + lane] : make_double2(0.0, 0.0);
                q = live ? pre[V + st + lane] : make_double2(0.0, 0.0);
            } else {
                const double2 x = live ? pos[st + lane] : make_double2(0.0, 0.0);
                double2 d;
                lanes_tangent(x, kn, t, d);
                if (areaFromPositions) {
                    lanes_area_gradient(d, live, kp, q);
                } else {
                    q = make_double2(0.0, 0.0);
                    if (live) {
                        const double* c = constraints + 6 * (size_t)(st + lane);
                        q = make_double2(c[0], c[1]);
                    }
                }
            }
            // J^T J diagonal: 2 for an edge of length >= 1e-14, else 1 (t = 0)
            const float mb = ((__double_as_longlong(t.x) | __double_as_longlong(t.y)) != 0) ? 2.0f : 1.0f;
            const float2 tf = make_float2(d2f_int(t.x), d2f_int(t.y));
            const double2 tn = shfl2(t, kn), tp = shfl2(t, kp);
            const float2 tpf = shfl2(tf, kp);
            const float mc = d2f_int(-(t.x * tn.x + t.y * tn.y));
            const float mcp = __shfl_sync(PCP_FULL, mc, kp);
            for (int round = 0; round < kProjRounds; ++round) {
                // residual right-hand sides J^T F', J^T q (FP64) and the FP32 rows
                const double2 fn = shfl2(f, kn), qn = shfl2(q, kn);
                float a = 0.f, b = 1.f, c = 0.f, q0 = 0.f, q1 = 0.f, q2 = 0.f;
                if (live) {
                    q0 = d2f_int(t.x * (fn.x - f.x) + t.y * (fn.y - f.y));
                    q1 = d2f_int(t.x * (qn.x - q.x) + t.y * (qn.y - q.y));
                    b = mb; c = mc; a = mcp;
                }
                // Sherman-Morrison: move the cyclic corners out of the matrix
                const float gamma = -__shfl_sync(PCP_FULL, b, 0);
                const float beta = __shfl_sync(PCP_FULL, a, 0);
                const float alpha = __shfl_sync(PCP_FULL, c, n - 1);
                if (!(gamma != 0.f)) { bad = true; break; }
                if (lane == 0) { b = b - gamma; a = 0.f; q2 = gamma; }
                if (lane == n - 1) { b = b - alpha * beta / gamma; c = 0.f; q2 = alpha; }
                lanes_pcr3(a, b, c, q0, q1, q2, N, lane);
                const float s0 = __shfl_sync(PCP_FULL, q2, 0), sl = __shfl_sync(PCP_FULL, q2, n - 1);
                const float y0 = __shfl_sync(PCP_FULL, q0, 0), yl = __shfl_sync(PCP_FULL, q0, n - 1);
                const float z0 = __shfl_sync(PCP_FULL, q1, 0), zl = __shfl_sync(PCP_FULL, q1, n - 1);
                float den = 1.f + s0 + beta * sl / gamma;
                float fl = (y0 + beta * yl / gamma) / den;
                float fm = (z0 + beta * zl / gamma) / den;
                const float l0 = q0 - fl * q2, l1 = q1 - fm * q2;
                const float l0p = __shfl_sync(PCP_FULL, l0, kp), l1p = __shfl_sync(PCP_FULL, l1, kp);
                // F' -= J lambda, q -= J mu with (J x)_k = -x_k t_k + x_{k-1} t_{k-1}:
                // the first (full-size) update with the FP64 tangents, the later
                // corrections (relative size ~1e-5) with FP32 products added in
                // FP64 -- an error outside span(J) would be invisible to the
                // next residual J^T F'
                if (live) {
                    if (round == 0) {
                        double L0 = f2d_int(l0), L0p = f2d_int(l0p);
                        double L1 = f2d_int(l1), L1p = f2d_int(l1p);
                        f.x = fma(-L0p, tp.x, fma(L0, t.x, f.x));
                        f.y = fma(-L0p, tp.y, fma(L0, t.y, f.y));
                        q.x = fma(-L1p, tp.x, fma(L1, t.x, q.x));
                        q.y = fma(-L1p, tp.y, fma(L1, t.y, q.y));
                    } else {
                        f.x += f2d_int(l0 * tf.x - l0p * tpf.x); f.y += f2d_int(l0 * tf.y - l0p * tpf.y);
                        q.x += f2d_int(l1 * tf.x - l1p * tpf.x); q.y += f2d_int(l1 * tf.y - l1p * tpf.y);
                    }
                }
            }
            if (!bad) {
                double qF = live ? q.x * f.x + q.y * f.y : 0.0;
                double qq = live ? q.x * q.x + q.y * q.y : 0.0;
                {
                    const double2 t2 = warp_sum2(qF, qq);
                    qF = t2.x; qq = t2.y;
                }
                // sqrt(qq) > 1e-14 (kernels.cuh:464), tested on the bit
                // pattern (qq >= 0 or NaN; 0x3A1FB0F6BE506019 is 1e-28); the
                // quotient by the Newton reciprocal.  qq <= 1 for the unit
                // area gradients; a qq of 2^126 or more (corrupt input) takes
                // coef = 0, within |qF| 2^-126 of qF / qq.
                const unsigned long long qqB = (unsigned long long)__double_as_longlong(qq);
                double coef = 0.0;
                if (qqB > 0x3A1FB0F6BE506019ull && qqB < 0x47D0000000000000ull)
                    coef = qF * rcp_newton(qq);
                f = make_double2(f.x - coef * q.x, f.y - coef * q.y);
                if (live) force[st + lane] = f;
            }
        }
        if (live && !bad) {
            mF = max_abs_bits(mF, f.x, f.y);
            if (proceed) {
                double2 v = vel[st + lane];
                v.x += 0.5 * dt * f.x;
                v.y += 0.5 * dt * f.y;
                vel[st + lane] = v;
                sP += f.x * v.x + f.y * v.y;
                sV += v.x * v.x + v.y * v.y;
                sF += f.x * f.x + f.y * f.y;
            }
        }
    }
    if (fire) {
        // block partials first, then one atomic per block and quantity
        __shared__ double s_sum[3][4];
        __shared__ unsigned long long s_max[4];
        const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (bad && lane == 0) atomicOr(&fire->flags, kFlagNonFinite);
        mF = warp_max_u64(mF);
        if (proceed) { { const Sum4 t4 = warp_sum4(sP, sV, sF, 0.0); sP = t4.x; sV = t4.y; sF = t4.z; } }
        if (lane == 0) { s_max[warp] = mF; s_sum[0][warp] = sP; s_sum[1][warp] = sV; s_sum[2][warp] = sF; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int w = 1; w < nw; ++w) {
                if (s_max[w] > mF) mF = s_max[w];
                sP += s_sum[0][w]; sV += s_sum[1][w]; sF += s_sum[2][w];
            }
            if (mF) atomicMax(reinterpret_cast<unsigned long long*>(&fire->maxF), mF);
            if (proceed) {
                atomicAdd(&fire->P, sP);
                atomicAdd(&fire->vv, sV);
                atomicAdd(&fire->ff, sF);
            }
        }
        fire_pass_end(fire, rbNext);
    }
}

__global__ void k_rcp_newton(const double* __restrict__ x, double* __restrict__ y, int n) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = rcp_newton(x[i]);
}

cudaError_t launch_rcp_newton(const double* x, double* y, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    launch_k(k_rcp_newton, dim3(nblk(n, 256)), dim3(256), 0, st, x, y, n);
    return cudaGetLastError();
}

cudaError_t constraints_init() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_project, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_shake, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_project_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    done = true;
    return cudaSuccess;
}

// One polygon per thread (J^T J by Thomas) when there are enough polygons to
// fill the GPU, else one polygon per warp (J^T J by parallel cyclic
// reduction): 4096 polygons give only 128 warps of thread-per-polygon work.
cudaError_t launch_project(const double2* pos, const int* start, int P, int nmax,
                           const double* constraints, double2* force, double* scratch, int V,
                           int areaFromPositions, Ctrl* fireCtrl, const int* gate, double2* vel,
                           cudaStream_t st, int mainPass,
                           const double2* pre) {
    if (P <= 0) return cudaSuccess;
    if (P >= 128 * sm_count()) {
        int sn = smem_vertices(nmax, kProjArrays);
        size_t smem = (size_t)sn * kProjArrays * kConsThreads * sizeof(double);
        launch_k(k_project, dim3(nblk(P, kConsThreads)), dim3(kConsThreads), smem, st, 
            pos, start, P, constraints, force, scratch, V, sn, areaFromPositions, fireCtrl, vel,
            mainPass, gate);
        return cudaGetLastError();
    }
    if (project_uses_lanes(P, nmax)) {
        const int wpb = 4;
        launch_k(k_project_lanes, dim3(nblk(P, wpb)), dim3(32 * wpb), 0, st, pos, start, P,
                 constraints, force, areaFromPositions, fireCtrl, vel, mainPass, pre, V,
                 gate);
        return cudaGetLastError();
    }
    int nv = (nmax + 1) & ~1;          // even, so each workspace stays 16-byte aligned
    int N = 4;
    while (N < nv) N <<= 1;
    size_t per = proj_ws_bytes(nv, N);
    int wpb = 8;
    while (wpb > 1 && per * wpb > 200 * 1024) wpb >>= 1;
    int nmaxSmem = nv;
    if (per * wpb > 200 * 1024) { nmaxSmem = 0; per = 0; wpb = 8; }
    launch_k(k_project_warp, dim3(nblk(P, wpb)), dim3(32 * wpb), per * wpb, st, pos, start, P, constraints, force,
                                                              scratch, nmaxSmem, areaFromPositions,
                                                              fireCtrl, vel, mainPass, gate);
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
    pdl_enter();
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
    launch_k(k_xpbd, dim3(nblk(P, 128)), dim3(128), 0, st, pos, start, P, targetEdge, targetArea, devOut);
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

// Step start (model.cpp:405-430): the per-step resets of the control block,
// snapshots of x, v and F (for the rollbacks and for buffer-overflow
// recovery), the Verlet half-kick and drift, the pre-SHAKE copy of the new
// positions (`verlet`, may be null) and F = 0 for the coming force pass.
__global__ void k_fire_begin(double2* __restrict__ pos, double2* __restrict__ vel,
                             double2* __restrict__ force, double2* __restrict__ save,
                             double2* __restrict__ velSnap, double2* __restrict__ forceSnap,
                             double2* __restrict__ verlet, int V, int resetContacts,
                             Ctrl* __restrict__ c, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double dt = c->dt;
    if (i == 0) {
        fire_step_resets(c);
        if (resetContacts) zero_contact_counters(c);
    }
    const int bm = c->bendMode;
    const double ba = c->bendA, bs = c->bendS;
    if (i < V) {
        double2 x = pos[i], v = vel[i], f = force[i];
        v = apply_bend(v, f, bm, ba, bs);     // the previous step's bend
        save[i] = x;
        velSnap[i] = v;
        forceSnap[i] = f;
        v.x += 0.5 * dt * f.x; v.y += 0.5 * dt * f.y;
        double px = x.x + dt * v.x, py = x.y + dt * v.y;
        vel[i] = v;
        double2 xn = make_double2(frac_unit(px), frac_unit(py));
        pos[i] = xn;
        if (verlet) verlet[i] = xn;
        force[i] = make_double2(0.0, 0.0);
    }
}

// Last kernel of the SHAKE-retry body (model.cpp:431-438): the retry's
// outcome; when it failed too, restore the step's start positions and zero
// v (the SHAKE kernels have already rederived v from their displacements).
__global__ void k_fire_retry_outcome(double2* __restrict__ pos, double2* __restrict__ vel,
                                     const double2* __restrict__ save, int V,
                                     Ctrl* __restrict__ c) {
    pdl_enter();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool failed = c->shakeIters2 >= 10 * c->shakeIter;
    if (i == 0) {
        c->shakeLast = c->shakeIters2;
        c->shakeFailed = failed ? 1 : 0;
        c->condLaunches += 2;          // the retry SHAKE and this kernel
    }
    if (i >= V || !failed) return;
    pos[i] = save[i];
    vel[i] = make_double2(0.0, 0.0);
}

// Energy-increase rollback (model.cpp:453-465), first kernel of the
// rollback body: restore positions, zero v and F, zero the energy, max |F|
// and (when the body searches contacts) the contact counters.
__global__ void k_fire_rollback(double2* __restrict__ pos, double2* __restrict__ vel,
                                double2* __restrict__ force, const double2* __restrict__ save,
                                int V, int resetContacts, Ctrl* __restrict__ c) {
    pdl_enter();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        c->rollback = 1;
        c->energy = 0.0;
        c->maxF = 0.0;
        c->bendTicket = 0;   // the body's force pass ends the step
        if (resetContacts) zero_contact_counters(c);
        c->condLaunches += (unsigned long long)c->rbBodyKernels;
    }
    if (i >= V) return;
    pos[i] = save[i];
    vel[i] = make_double2(0.0, 0.0);
    force[i] = make_double2(0.0, 0.0);
}

// zero force + energy (+ maxF) under a gate (updateForceEnergy's memsets)
__global__ void k_zero_force(double2* __restrict__ force, int V, Ctrl* __restrict__ c,
                             const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) { c->energy = 0.0; c->maxF = 0.0; }
    if (i < V) force[i] = make_double2(0.0, 0.0);
}

// velocity update for models without projection (soft-body / hybrid):
// v += dt/2 F, accumulate F.v, |v|^2, |F|^2, max |F|; decides the rollback
// and sets `rbCond` of the step graph when `useCond`
__global__ void k_fire_velocity(double2* __restrict__ vel, const double2* __restrict__ force,
                                int V, Ctrl* __restrict__ c, cudaGraphConditionalHandle rbCond,
                                int useCond, const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const FireView fv = fire_view(c, rbCond, useCond);
    const bool proceed = fv.proceed, rbNext = fv.rbNext;
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
        { const Sum4 t4 = warp_sum4(sP, sV, sF, 0.0); sP = t4.x; sV = t4.y; sF = t4.z; }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&c->P, sP); atomicAdd(&c->vv, sV); atomicAdd(&c->ff, sF);
        }
    }
    if ((threadIdx.x & 31) == 0) __threadfence();
    fire_pass_end(c, rbNext);
}

// max |F| only (rollback path of models without projection)
__global__ void k_fire_maxf(const double2* __restrict__ force, int V, Ctrl* __restrict__ c,
                            const int* gate) {
    pdl_enter();
    if (gate_closed(gate)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double mF = 0.0;
    if (i < V) { double2 f = force[i]; mF = fmax(fabs(f.x), fabs(f.y)); }
    mF = warp_maxd(mF);
    if ((threadIdx.x & 31) == 0) { atomic_max_nonneg(&c->maxF, mF); __threadfence(); }
    fire_pass_end(c, false);    // the rollback body's pass (model.cpp:462-466)
}

// scalar bookkeeping of the step (model.cpp:444-485) and the stop test of
// Model::minimizeFIRE (model.cpp:500); one thread
__device__ void fire_scalars(Ctrl* __restrict__ c) {
    if (c->flags & (kFlagPairOverflow | kFlagRecordOverflow | kFlagSlowOverflow |
                    kFlagFixOverflow | kFlagCapacity)) {
        // a contact buffer overflowed: stop here; the host grows the buffers
        // and redoes this step from its snapshot
        c->needsRecovery = 1;
        c->active = 0;
        c->bendMode = 0;   // the redo starts from the step's snapshot (bent already)
        return;
    }
    double dt = c->dt, alpha = c->alpha;
    int nPos = c->nPos;
    c->bendMode = 0;       // failure and rollback zeroed v already
    if (c->shakeFailed) {
        c->outE = c->energy;
        dt *= c->fDec; alpha = c->alphaStart; nPos = 0;
    } else if (c->rollback) {
        c->outE = c->ePre;
        dt *= c->fDec; alpha = c->alphaStart; nPos = 0;
    } else {
        c->outE = c->energy;
        if (c->P > 0.0) {
            // v <- (1 - alpha) v + alpha |v| / |F| F with this step's alpha
            // (model.cpp:471-478), applied by the next step's start
            const double fn = sqrt(c->ff), vn = sqrt(c->vv);
            if (fn > 0.0) {
                c->bendA = 1.0 - alpha;
                c->bendS = alpha * vn / fn;
                c->bendMode = 1;
            }
            if (++nPos >= c->nMin) {
                double nd = fmin(dt * c->fInc, c->dtMax);
                if (nd > dt) alpha *= c->fAlpha;
                dt = nd;
            }
        } else {
            c->bendMode = 2;   // v <- 0 (model.cpp:479-483)
            dt *= c->fDec; alpha = c->alphaStart; nPos = 0;
        }
    }
    c->dt = dt; c->alpha = alpha; c->nPos = nPos;
    c->stepsDone += 1;
    c->Rmax = 0.f;     // for the next step's fused start (see zero_contact_counters_but_rmax)
    const int it = c->shakeLast;
    c->shakeMinRun = min(c->shakeMinRun, it);
    c->shakeMaxRun = max(c->shakeMaxRun, it);
    c->shakeSumRun += it;
    if (c->stagnantLimit >= 0) {
        // pyCudaPolygon.py:723-727: |E - E_prev| < 1e-15 counted, stop past 5
        if (fabs(c->outE - c->prevE) < c->stagnantTol) c->stagnant += 1;
        if (c->stagnant > c->stagnantLimit) { c->stagnated = 1; c->active = 0; }
        c->prevE = c->outE;
    }
    if (c->maxF <= c->threshold) { c->converged = 1; c->active = 0; }
    if (c->stepLimit > 0 && c->stepsDone >= c->stepLimit) c->active = 0;
}


// A pending bend (Ctrl::bendMode) applied before the velocities are read
// outside a FIRE step; the host clears the mode after this kernel.
__global__ void k_fire_settle(double2* __restrict__ vel, const double2* __restrict__ force,
                              int V, const Ctrl* __restrict__ c) {
    pdl_enter();
    const int bm = c->bendMode;
    if (bm == 0) return;
    const double ba = c->bendA, bs = c->bendS;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < V) vel[i] = apply_bend(vel[i], force[i], bm, ba, bs);
}

__global__ void k_set_fire_params(Ctrl* __restrict__ c, FireScalars f) {
    pdl_enter();
    c->dt = f.dt; c->alpha = f.alpha; c->nPos = f.nPos;
    c->dtMax = f.dtMax; c->alphaStart = f.alphaStart; c->fAlpha = f.fAlpha; c->fInc = f.fInc;
    c->fDec = f.fDec; c->nMin = f.nMin; c->shakeIter = f.shakeIter; c->threshold = f.threshold;
    c->active = 1;
    if (f.resetRun) {
        c->converged = 0; c->stepsDone = 0;
        c->prevE = 1e9; c->stagnant = 0; c->stagnated = 0;    // pyCudaPolygon.py:707-710
        c->shakeMinRun = 1000000000; c->shakeMaxRun = 0; c->shakeSumRun = 0;
    }
    c->stagnantTol = f.stagnantTol;
    c->stagnantLimit = f.stagnantLimit;
    c->stepLimit = f.stepLimit;
    c->rbBodyKernels = f.rbBodyKernels;
    c->Rmax = 0.f;
}

// --------------------------------------------------------------- launchers ----
cudaError_t launch_set_fire_params(Ctrl* c, const FireScalars& f, cudaStream_t st) {
    launch_k(k_set_fire_params, dim3(1), dim3(1), 0, st, c, f);
    return cudaGetLastError();
}
cudaError_t launch_fire_begin(double2* pos, double2* vel, double2* force, double2* save,
                              double2* velSnap, double2* forceSnap, double2* verlet, int V,
                              int resetContacts, Ctrl* c, const int* gate, cudaStream_t st) {
    launch_k(k_fire_begin, dim3(nblk(V, 256)), dim3(256), 0, st, pos, vel, force, save, velSnap, forceSnap, verlet,
                                               V, resetContacts, c, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_retry_outcome(double2* pos, double2* vel, const double2* save, int V,
                                      Ctrl* c, cudaStream_t st) {
    launch_k(k_fire_retry_outcome, dim3(nblk(V, 256)), dim3(256), 0, st, pos, vel, save, V, c);
    return cudaGetLastError();
}
cudaError_t launch_fire_rollback(double2* pos, double2* vel, double2* force, const double2* save,
                                 int V, int resetContacts, Ctrl* c, cudaStream_t st) {
    launch_k(k_fire_rollback, dim3(nblk(V, 256)), dim3(256), 0, st, pos, vel, force, save, V, resetContacts, c);
    return cudaGetLastError();
}
cudaError_t launch_zero_force(double2* force, int V, Ctrl* c, const int* gate, cudaStream_t st) {
    launch_k(k_zero_force, dim3(nblk(V, 256)), dim3(256), 0, st, force, V, c, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_velocity(double2* vel, const double2* force, int V, Ctrl* c,
                                 cudaGraphConditionalHandle rbCond, int useCond,
                                 const int* gate, cudaStream_t st) {
    launch_k(k_fire_velocity, dim3(nblk(V, 256)), dim3(256), 0, st, vel, force, V, c, rbCond, useCond, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_maxf(const double2* force, int V, Ctrl* c, const int* gate,
                             cudaStream_t st) {
    launch_k(k_fire_maxf, dim3(nblk(V, 256)), dim3(256), 0, st, force, V, c, gate);
    return cudaGetLastError();
}
cudaError_t launch_fire_settle(double2* vel, const double2* force, int V, Ctrl* c,
                               cudaStream_t st) {
    launch_k(k_fire_settle, dim3(nblk(V, 256)), dim3(256), 0, st, vel, force, V, c);
    return cudaGetLastError();
}

// ---------------------------------------------- SHAKE without allocation ----
// Workspace of pcp_shake_project_noalloc: a fixed array in this module's own
// device memory, for callers that may not allocate device memory.  Polygon p
// works in doubles [kScratchPerVertex * start[p], kScratchPerVertex *
// start[p+1]) and writes every element of its slice before reading it, so
// nothing in the array has to start at zero.  There is one array per device
// and every call on that device shares it: calls whose kernels overlap on the
// GPU race on it.
static __device__ __align__(256) double
    g_shake_noalloc_scratch[(size_t)kScratchPerVertex * PCP_SHAKE_NOALLOC_MAX_VERTICES];

// Outcome of the last input check of pcp_shake_project_noalloc on this
// device (0 valid, 1 start[0] != 0 or start decreasing, 2 more vertices than
// the array holds); read back with cudaMemcpyFromSymbolAsync.
static __device__ int g_shake_noalloc_status;

// One block checks that the CSR offsets describe polygons inside the array:
// start[0] == 0, start non-decreasing, start[P] <= capacity.  k_shake writes
// doubles [kScratchPerVertex * start[p], kScratchPerVertex * start[p+1]) for
// polygon p, so this bounds every write into the array.
__global__ void k_shake_noalloc_check(const int* __restrict__ start, int P, int capacity) {
    int bad = 0;
    for (int p = threadIdx.x; p < P; p += blockDim.x)
        if (start[p + 1] < start[p]) bad = 1;
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        int status = 0;
        if (bad || start[0] != 0) status = 1;
        else if (start[P] > capacity) status = 2;
        g_shake_noalloc_status = status;
    }
}

cudaError_t shake_noalloc_check(const int* start, int P, int* status, cudaStream_t st) {
    launch_k(k_shake_noalloc_check, dim3(1), dim3(256), 0, st, start, P,
             (int)PCP_SHAKE_NOALLOC_MAX_VERTICES);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyFromSymbolAsync(status, g_shake_noalloc_status, sizeof(int), 0,
                                  cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

// Device address of the array on the current device.  It is looked up once
// per device, by the first call made with that device current; the lookup
// can load this module onto the device, so that first call belongs before
// any stream capture.
cudaError_t shake_noalloc_scratch(double** out) {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static double* addr[kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_shake_noalloc_scratch);
        if (e != cudaSuccess) return e;
        addr[dev] = static_cast<double*>(p);
    }
    *out = addr[dev];
    return cudaSuccess;
}

// k_shake with every polygon's workspace in `scratch` (none in shared
// memory, so the launch needs no attribute set-up)
cudaError_t launch_shake_noalloc(double2* pos, const int* start, int P, const double* targetEdge,
                                 const double* targetArea, int maxIter, double tol,
                                 int* maxItersOut, double* scratch, cudaStream_t st) {
    if (P <= 0) return cudaSuccess;
    constexpr int wpb = 8;
    launch_k(k_shake, dim3(nblk(P, wpb)), dim3(32 * wpb), 0, st, pos, start, P, targetEdge, targetArea, maxIter, tol,
                                               maxItersOut, scratch, 0, nullptr, 0, nullptr, nullptr,
                                               nullptr);
    return cudaGetLastError();
}

}  // namespace pcp
