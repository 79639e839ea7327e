// pcp_common.cuh -- shared device code for the GB300 (sm_103a) polygon kernels.
//
// FP64 arithmetic here restates the reference's device functions
// (camdennis/pyCudaPolygon src/kernels.cuh); the crossing predicate is
// evaluated without fused multiply-adds so that its decisions and its
// float-rounded (t, u) agree bit for bit with the FP64 restatement.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pcp_gb300.h"

#define PCP_WARP 32
#define PCP_FULL 0xffffffffu

namespace pcp {

// ---------------------------------------------- programmatic dependent launch
// Every kernel of the path starts with pdl_enter(): it waits until the
// kernel before it on the stream has finished and its writes are visible
// (griddepcontrol.wait, a no-op when the launch did not ask for overlap), then
// lets the next kernel's blocks be scheduled (griddepcontrol.launch_dependents)
// so that launch hides behind this kernel's run.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch with programmatic stream serialization (the kernel must begin with
// pdl_enter()).  Errors are reported through cudaGetLastError like <<< >>>.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                            cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// The same launch without programmatic dependent launch: the kernel's blocks
// are scheduled only once the previous kernel on the stream has finished, so
// none wait on an SM beside it (for wide grids that are usually empty).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k_serial(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                   cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.numAttrs = 0;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// ---------------------------------------------------------------- wraps ----

// wrap (kernels.cuh:115-119): minimum image into [-0.5, 0.5),
//   y = x + 1.5;  y = y - floor(y);  return y - 0.5;
// For y in [0, 3) (x in [-1.5, 1.5): every difference of two positions of
// the unit box) floor(y) is read from y's high word with integer compares,
// and (y - floor(y)) - 0.5 = y - (floor(y) + 0.5) holds exactly (both
// differences are exact), so the result is bit-identical with two FP64
// adds instead of three adds and a floor.  Other y take the literal form.
__device__ __forceinline__ double wrap(double x) {
    double y = x + 1.5;
    int hi = __double2hiint(y);
    if (hi >= 0 && hi < 0x40080000) {            // 0 <= y < 3 (and not NaN)
        // floor(y) + 0.5 as a double: 0.5, 1.5 or 2.5 (low word 0)
        int c = hi < 0x3FF00000 ? 0x3FE00000 : (hi < 0x40000000 ? 0x3FF80000 : 0x40040000);
        return y - __hiloint2double(c, 0);
    }
    y = y - floor(y);
    return y - 0.5;
}

// y - floor(y), with the FP64 floor replaced by bit tests where
// -1 <= y < 2 (a coordinate of [0, 1] moved by far less than 1): the same
// single rounding as y - floor(y) in each case (y, y - 1, y + 1; -0 gives +0).
__device__ __forceinline__ double frac_unit(double y) {
    const unsigned hi = (unsigned)__double2hiint(y);
    const unsigned lo = (unsigned)__double2loint(y);
    if (hi < 0x3FF00000u) return y;                          // 0 <= y < 1
    if (hi < 0x40000000u) return y - 1.0;                    // 1 <= y < 2
    if (hi == 0x80000000u && lo == 0u) return 0.0;           // -0
    if (hi >= 0x80000000u && (hi < 0xBFF00000u || (hi == 0xBFF00000u && lo == 0u)))
        return y + 1.0;                                      // -1 <= y < 0
    return y - floor(y);
}

__device__ __forceinline__ double2 wrap2(double2 v) {
    return make_double2(wrap(v.x), wrap(v.y));
}

// FP32 minimum image for the conservative prefilters (range [-0.5, 0.5]).
__device__ __forceinline__ float wrapf(float x) { return x - rintf(x); }

// The reference's `while` wrap loops into [0,1) (kernels.cuh:670-699).  For
// positions inside [0,1] they take at most one pass; the cap only stops
// corrupt input from spinning (the reference would not return there).
__device__ __forceinline__ double loop_wrap_unit(double x) {
    int it = 0;
    while (x < 0.0 && it < 64) { x += 1.0; ++it; }
    while (x >= 1.0 && it < 128) { x -= 1.0; ++it; }
    if (it >= 64 && isfinite(x) && (x < 0.0 || x >= 1.0)) x = x - floor(x);
    return x;
}

// (int)floor(v * B) clamped into [0, B) like kernels.cuh:700-704; NaN -> 0.
__device__ __forceinline__ int cell_coord(double v, int B) {
    double f = floor(v * (double)B);
    if (!(f >= 0.0)) return 0;
    if (f >= (double)B) return B - 1;
    return (int)f;
}

// Cell of the midpoint of the edge from a to b (updateNeighborCellsKernel,
// kernels.cuh:661-707).
__device__ __forceinline__ int midpoint_cell_of(double2 a, double2 b, int B) {
    double x = b.x - a.x + 0.5;
    double y = b.y - a.y + 0.5;
    x = loop_wrap_unit(x);
    y = loop_wrap_unit(y);
    x -= 0.5; y -= 0.5;
    x /= 2.0; y /= 2.0;
    x += a.x; y += a.y;
    x = loop_wrap_unit(x);
    y = loop_wrap_unit(y);
    return cell_coord(y, B) * B + cell_coord(x, B);
}

// The same cell, decided in FP32 when that is safe.  With the coordinates
// within one float ulp (6e-8) of the FP64 ones, the FP32 midpoint is within
// 2.6e-7 of the FP64 one (four further roundings) and its product with B adds
// at most 3e-8 B, so it lies within 2.9e-7 B cell widths of the FP64 value;
// when it is more than 1e-4 + 4e-7 B cell widths from every cell boundary
// (and the edge is short, so both minimum images agree) the FP64
// computation lands in the same cell.
// Otherwise, and for non-finite input, the FP64 form decides.  fa, fb are
// a and b rounded to float.
__device__ __forceinline__ int midpoint_cell_fast(double2 a, double2 b, float2 fa, float2 fb,
                                                  int B) {
    float ddx = wrapf(fb.x - fa.x), ddy = wrapf(fb.y - fa.y);
    float mx = fa.x + 0.5f * ddx, my = fa.y + 0.5f * ddy;
    mx -= floorf(mx);
    my -= floorf(my);
    float ux = mx * (float)B, uy = my * (float)B;
    const float margin = 1e-4f + 4e-7f * (float)B;
    bool sure = fabsf(ddx) < 0.45f && fabsf(ddy) < 0.45f &&
                fabsf(ux - rintf(ux)) > margin && fabsf(uy - rintf(uy)) > margin;
    if (sure) {
        int cx = min((int)ux, B - 1), cy = min((int)uy, B - 1);
        return cy * B + cx;
    }
    return midpoint_cell_of(a, b, B);
}

// Cell of the midpoint of the edge that starts at vertex idx.
__device__ __forceinline__ int midpoint_cell(const double2* __restrict__ pos,
                                             const int* __restrict__ start,
                                             const int* __restrict__ shapeId,
                                             int size, int idx, int B) {
    int v2 = idx + 1;
    if (idx == size - 1 || shapeId[idx] != shapeId[idx + 1]) v2 = start[shapeId[idx]];
    return midpoint_cell_of(pos[idx], pos[v2], B);
}

// Cells visited by updateNeighborsKernel's 3x3 stencil (kernels.cuh:737-762):
// every cell for B < 3, otherwise cyclic distance <= 1 on both axes.  The
// relation is symmetric, so it can be tested from either edge.
__device__ __forceinline__ bool cells_adjacent(int c1, int c2, int B) {
    if (B < 3) return true;
    int x1 = c1 % B, y1 = c1 / B, x2 = c2 % B, y2 = c2 / B;
    int dx = x1 - x2; if (dx < 0) dx = -dx;
    int dy = y1 - y2; if (dy < 0) dy = -dy;
    return (dx <= 1 || dx == B - 1) && (dy <= 1 || dy == B - 1);
}

// ------------------------------------------------------ exact predicate ----

// Crossing test of updateNeighborsKernel (kernels.cuh:778-807) with the edge
// vectors precomputed as r = wrap(p2 - p), s = wrap(q2 - q).  No contraction:
// every product and difference is rounded separately.
struct Crossing { double tt, uu, denom; bool hit; };

__device__ __forceinline__ Crossing cross_exact(double2 p, double2 r, double2 q, double2 s) {
    Crossing c;
    double gx = wrap(__dsub_rn(q.x, p.x));
    double gy = wrap(__dsub_rn(q.y, p.y));
    c.denom = __dsub_rn(__dmul_rn(r.x, s.y), __dmul_rn(r.y, s.x));
    c.hit = false;
    c.tt = 0.0; c.uu = 0.0;
    if (fabs(c.denom) < 1e-12) return c;
    double nt = __dsub_rn(__dmul_rn(gx, s.y), __dmul_rn(gy, s.x));
    double nu = __dsub_rn(__dmul_rn(gx, r.y), __dmul_rn(gy, r.x));
    c.tt = __ddiv_rn(nt, c.denom);
    c.uu = __ddiv_rn(nu, c.denom);
    c.hit = (c.tt > 0.0 && c.tt < 1.0 && c.uu > 0.0 && c.uu < 1.0);
    return c;
}

// ---------------------------------------------------- energy functions ----

// h (kernels.cuh:139-146)
__device__ __forceinline__ double h_term(double2 p1, double2 p2, double2 sp) {
    double r1x = wrap(p1.x - sp.x), r1y = wrap(p1.y - sp.y);
    double r2x = wrap(p2.x - sp.x), r2y = wrap(p2.y - sp.y);
    double dy = wrap(r2y - r1y);
    return (r1x + r2x) * dy;
}

// g12 (kernels.cuh:148-159): g1 = (dy, -(r1x+r2x)), g2 = (dy, r1x+r2x)
__device__ __forceinline__ void g12(double2 p1, double2 p2, double2 sp, double2& g1, double2& g2) {
    double r1x = wrap(p1.x - sp.x);
    double r2x = wrap(p2.x - sp.x);
    double dy = wrap(p2.y - p1.y);
    g1 = make_double2(dy, -(r1x + r2x));
    g2 = make_double2(dy, r1x + r2x);
}

// h and g12 together (they share r1x, r2x), the gradients in the parts
// they are made of: g1 = (dyg, -sx), g2 = (dyg, sx).  h's own dy,
// wrap(r2y - r1y) with r = wrap(p - sp), equals dyg = wrap(p2.y - p1.y) up
// to the roundings of the two relative coordinates (p1, p2 and sp lie within
// a polygon's size of each other), so h takes dyg as well: three wraps fewer,
// and the energy moves by a few ulps of its terms.
__device__ __forceinline__ double h_parts(double2 p1, double2 p2, double2 sp, double& dyg,
                                          double& sx) {
    const double r1x = wrap(p1.x - sp.x), r2x = wrap(p2.x - sp.x);
    dyg = wrap(p2.y - p1.y);
    sx = r1x + r2x;
    return sx * dyg;
}

// The same for an edge p1 -> p1 + d whose vector d = wrap(p2 - p1) the
// caller holds: r2x = r1x + d.x, so sx = 2 r1x + d.x and dyg = d.y.
__device__ __forceinline__ double h_parts_edge(double2 p1, double2 d, double2 sp, double& sx) {
    const double r1x = wrap(p1.x - sp.x);
    sx = fma(2.0, r1x, d.x);
    return sx * d.y;
}

// -x by a flip of the sign bit on the integer pipe
__device__ __forceinline__ double neg_int(double x) {
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}

// getDf (kernels.cuh:161-222): Jacobian of f = vi + u (vzi - vi), the point
// where edge (vi, vzi) meets edge (vj, vzj), with respect to (vi, vzi, vj,
// vzj).  Only its contractions with a row vector g are needed; this returns
// the four 2-vectors gT df restricted to each vertex:  out[p] = (g . df[:,2p],
// g . df[:,2p+1]).  Zero for near-parallel or degenerate edges.
// di = wrap(vzi - vi), when the caller has it already.
// dj = wrap(vzj - vj) as well, when the caller has it (vzj itself is then
// not needed).
__device__ __forceinline__ void gDf_dd(double2 vi, double2 di, double2 vj, double2 dj,
                                       double2 g, double2 out[4]) {
    double djx = dj.x, djy = dj.y;
    double dix = di.x, diy = di.y;
    double dijx = wrap(vj.x - vi.x), dijy = wrap(vj.y - vi.y);
    double w = djx * diy - djy * dix;
    double diN = dix * dix + diy * diy;
    double djN = djx * djx + djy * djy;
    // The degeneracy tests on the integer pipe: w^2, the limit and the
    // squared lengths are non-negative doubles (or NaN, for which every test
    // is false), and for those the unsigned order of the bit patterns is the
    // order of the values.  0x3A1FB0F6BE506019 is the pattern of 1e-28.
    const unsigned long long wwB = (unsigned long long)__double_as_longlong(w * w);
    const unsigned long long limB = (unsigned long long)__double_as_longlong(1e-12 * diN * djN);
    const unsigned long long tinyB = 0x3A1FB0F6BE506019ull;
    if ((wwB < limB && limB <= 0x7FF0000000000000ull) ||
        (unsigned long long)__double_as_longlong(diN) < tinyB ||
        (unsigned long long)__double_as_longlong(djN) < tinyB) {
        out[0] = out[1] = out[2] = out[3] = make_double2(0.0, 0.0);
        return;
    }
    double k = djx * dijy - djy * dijx;
    double iw = 1.0 / w;
    double u = k * iw;
    // g . du/d(vertex, component) = s (dk - u dw) with s = (g . di) / w, and
    // f = vi + u di passes g (1 - u) to vi and g u to vzi:
    //   vi : (1 - u) (s djy + gx, gy - s djx)
    //   vzi: u (s djy + gx, gy - s djx)
    //   vj : s ((-dijy - djy) + u diy, (djx + dijx) - u dix)
    //   vzj: s (dijy - u diy, u dix - dijx)
    const double s = (g.x * dix + g.y * diy) * iw;
    const double ax = fma(s, djy, g.x), ay = fma(-s, djx, g.y);
    const double omu = 1.0 - u;
    out[0] = make_double2(omu * ax, omu * ay);
    out[1] = make_double2(u * ax, u * ay);
    out[2] = make_double2(s * fma(u, diy, -dijy - djy), s * fma(-u, dix, djx + dijx));
    out[3] = make_double2(s * fma(-u, diy, dijy), s * fma(u, dix, -dijx));
}
__device__ __forceinline__ void gDf_di(double2 vi, double2 di, double2 vj, double2 vzj,
                                       double2 g, double2 out[4]) {
    gDf_dd(vi, di, vj, make_double2(wrap(vzj.x - vj.x), wrap(vzj.y - vj.y)), g, out);
}
__device__ __forceinline__ void gDf(double2 vi, double2 vzi, double2 vj, double2 vzj,
                                    double2 g, double2 out[4]) {
    gDf_di(vi, make_double2(wrap(vzi.x - vi.x), wrap(vzi.y - vi.y)), vj, vzj, g, out);
}

// ------------------------------------------- conversions on the INT pipe ----
// On GB300 the FP64<->FP32 conversions, FP64 compares and FP64 min/max run
// at the FP64 rate (about 1/64 of FP32), so the mixed-precision solvers
// convert with integer operations instead.
//
// FP32 -> FP64, exact for normal floats; zero and denormals give +-0.
__device__ __forceinline__ double f2d_int(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned sign = u & 0x80000000u;
    if (e == 0u) return __hiloint2double((int)sign, 0);
    if (e == 0xFFu) return (double)f;                         // inf / NaN (not expected)
    const unsigned m = u & 0x7FFFFFu;
    const unsigned hi = sign | ((e + (1023u - 127u)) << 20) | (m >> 3);
    return __hiloint2double((int)hi, (int)(m << 29));
}
// FP64 -> FP32 by truncation of the significand (within one float ulp of
// the value: inputs of the FP32 solves only); magnitudes below 2^-126 give
// +-0, above the float range +-inf, NaN stays NaN.
__device__ __forceinline__ float d2f_int(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7FFu) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) {
        const unsigned mag = hi & 0x7FFFFFFFu;
        const bool nan = mag > 0x7FF00000u || (mag == 0x7FF00000u && lo != 0u);
        return __uint_as_float(nan ? 0x7FC00000u : (sign | 0x7F800000u));
    }
    const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    return __uint_as_float(sign | ((unsigned)e << 23) | m);
}
// 1/x for a double with 2^-126 <= |x| < 2^126 (x and 1/x in the normal
// float range): the FP32 reciprocal of the truncated value (relative error
// below 2^-22) refined by
// two Newton-Raphson steps y <- y + y (1 - x y), each of which squares the
// relative error, so the result is within a few ulps of 1/x.  Four FP64 FMAs
// instead of a division's longer sequence.
__device__ __forceinline__ double rcp_newton(double x) {
    double y = f2d_int(__frcp_rn(d2f_int(x)));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

// |x| as the bit pattern of a non-negative double: for finite values the
// unsigned order of these patterns is the order of the magnitudes (NaN
// patterns sort above +inf).
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long t = __shfl_xor_sync(PCP_FULL, v, o);
        v = t > v ? t : v;
    }
    return v;
}
// true when the pattern is that of a finite double
__device__ __forceinline__ bool finite_bits(unsigned long long b) {
    return (b & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}
// running max of |x|, |y| as a bit pattern, NaN left out (as fmax does)
__device__ __forceinline__ unsigned long long max_abs_bits(unsigned long long m, double x,
                                                              double y) {
    const unsigned long long inf = 0x7FF0000000000000ull;
    unsigned long long a = abs_bits(x), b = abs_bits(y);
    if (a <= inf && a > m) m = a;
    if (b <= inf && b > m) m = b;
    return m;
}

// ------------------------------------------------------- warp helpers ----

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(PCP_FULL, v, o);
    return v;
}
// Two warp sums for the FP64 adds of one: at the first level the lower half
// of the warp keeps adding a and the upper half b (each lane sends its
// partner the value it drops), then each half reduces alone; the totals are
// broadcast from lanes 0 and 16.  5 FP64 adds instead of 10 (every lane gets
// the same bits; the association differs from warp_sum's).
__device__ __forceinline__ double2 warp_sum2(double a, double b) {
    const bool hi = (threadIdx.x & 16) != 0;
    double keep = hi ? b : a;
    keep += __shfl_xor_sync(PCP_FULL, hi ? a : b, 16);
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) keep += __shfl_xor_sync(PCP_FULL, keep, o);
    return make_double2(__shfl_sync(PCP_FULL, keep, 0), __shfl_sync(PCP_FULL, keep, 16));
}

// Four warp sums for 6 FP64 adds instead of 20: the warp splits into halves
// (a, b | c, d) and then quarters (a | b | c | d) before reducing; the totals
// are broadcast from lanes 0, 8, 16 and 24.
struct Sum4 { double x, y, z, w; };
__device__ __forceinline__ Sum4 warp_sum4(double a, double b, double c, double d) {
    const int lane = threadIdx.x & 31;
    const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
    double k0 = h16 ? c : a, k1 = h16 ? d : b;
    k0 += __shfl_xor_sync(PCP_FULL, h16 ? a : c, 16);
    k1 += __shfl_xor_sync(PCP_FULL, h16 ? b : d, 16);
    double keep = h8 ? k1 : k0;
    keep += __shfl_xor_sync(PCP_FULL, h8 ? k0 : k1, 8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) keep += __shfl_xor_sync(PCP_FULL, keep, o);
    return Sum4{__shfl_sync(PCP_FULL, keep, 0), __shfl_sync(PCP_FULL, keep, 8),
                __shfl_sync(PCP_FULL, keep, 16), __shfl_sync(PCP_FULL, keep, 24)};
}

__device__ __forceinline__ float warp_maxf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(PCP_FULL, v, o));
    return v;
}
__device__ __forceinline__ float warp_minf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(PCP_FULL, v, o));
    return v;
}
__device__ __forceinline__ double warp_maxd(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(PCP_FULL, v, o));
    return v;
}
__device__ __forceinline__ int warp_sumi(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(PCP_FULL, v, o);
    return v;
}

// max of non-negative doubles through their bit patterns (NaN ignored).
__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
    if (!(v >= 0.0)) return;
    atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_max_nonneg_f(float* addr, float v) {
    if (!(v >= 0.0f)) return;
    atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
}

// Gate: kernels of the device-resident FIRE step run only when the flag they
// are given is set (null = always run).
__device__ __forceinline__ bool gate_closed(const int* gate) {
    return gate != nullptr && *(volatile const int*)gate == 0;
}

}  // namespace pcp
