// pcp_fire.cuh -- device helpers of the FIRE step shared by the contact and
// constraint translation units (sm_103a).
#pragma once

#include <stddef.h>

#include "pcp_common.cuh"
#include "pcp_internal.h"

namespace pcp {

// zero the contact-search counters (everything in Ctrl before `energy`)
__device__ __forceinline__ void zero_contact_counters(Ctrl* c) {
    int* w = reinterpret_cast<int*>(c);
    constexpr int n = (int)(offsetof(Ctrl, energy) / sizeof(int));
#pragma unroll
    for (int i = 0; i < n; ++i) w[i] = 0;
}

// the same but for Rmax, which the prepass accumulates while this runs in
// the fused step-start kernel (it is zeroed at the end of the step before)
__device__ __forceinline__ void zero_contact_counters_but_rmax(Ctrl* c) {
    const float r = c->Rmax;
    zero_contact_counters(c);
    c->Rmax = r;
}

// per-step resets of the control block at the start of a FIRE step
__device__ __forceinline__ void fire_step_resets(Ctrl* c) {
    c->ePre = c->energy;
    c->energy = 0.0;
    c->snapDt = c->dt; c->snapAlpha = c->alpha; c->snapNPos = c->nPos;
    c->maxF = 0.0;
    c->P = 0.0; c->vv = 0.0; c->ff = 0.0;
    c->shakeIters1 = 0; c->shakeIters2 = 0;
    c->needRetry = 0; c->retryGate = 0;
    c->shakeFailed = 0;
    c->rollback = 0; c->rbGate = 0; c->proceed = 0;
    c->shakeTicket = 0; c->bendTicket = 0; c->forceTicket = 0;
}

// The rollback test at the end of the step's force evaluation
// (model.cpp:450-453): the velocities advance unless SHAKE failed or the
// energy went up, and the energy-increase rollback runs next when the energy
// went up and SHAKE did not fail.  One thread; `publish` stores the outcome
// (proceed, rbGate) and sets `rbCond` when `useCond`.  The energy is read
// past L1 (other blocks of the calling kernel may have just added to it).
// Returns proceed | rbNext << 1.
__device__ __forceinline__ int fire_decide(Ctrl* __restrict__ c, bool publish,
                                           cudaGraphConditionalHandle rbCond, int useCond) {
    const double E = __ldcg(&c->energy), E0 = __ldcg(&c->ePre);
    const int failed = __ldcg(&c->shakeFailed), rollback = __ldcg(&c->rollback);
    const int active = __ldcg(&c->active);
    const bool rb = E > E0 + fmax(fabs(E0) * 1e-10, 1e-14);
    const bool proceed = !failed && !rb && rollback == 0;
    const bool rbNext = rollback == 0 && !failed && rb && active;
    if (publish && rollback == 0) {
        c->proceed = proceed ? 1 : 0;
        c->rbGate = rbNext ? 1 : 0;
        if (useCond) cudaGraphSetConditional(rbCond, rbNext ? 1u : 0u);
    }
    return (proceed ? 1 : 0) | (rbNext ? 2 : 0);
}

// The previous step's velocity bend (model.cpp:471-484, Ctrl::bendMode),
// deferred to the start of this step: the same operations as at the end of
// the previous one.
__device__ __forceinline__ double2 apply_bend(double2 v, double2 f, int mode, double a, double s) {
    if (mode == 1) return make_double2(a * v.x + s * f.x, a * v.y + s * f.y);
    if (mode == 2) return make_double2(0.0, 0.0);
    return v;
}

// Verlet half-kick and drift of vertex i (model.cpp:405-430) after the
// previous step's bend, with the snapshots the rollbacks and the overflow
// recovery restore from; F = 0 for the coming force pass.  Returns the new
// position.
__device__ __forceinline__ double2 fire_move_vertex(const FireMove& mv, int i, double dt,
                                                    int bendMode, double bendA, double bendS) {
    double2 x = mv.pos[i], v = mv.vel[i], f = mv.force[i];
    v = apply_bend(v, f, bendMode, bendA, bendS);
    mv.save[i] = x;
    mv.velSnap[i] = v;
    mv.forceSnap[i] = f;
    v.x += 0.5 * dt * f.x; v.y += 0.5 * dt * f.y;
    double px = x.x + dt * v.x, py = x.y + dt * v.y;
    mv.vel[i] = v;
    double2 xn = make_double2(frac_unit(px), frac_unit(py));
    mv.pos[i] = xn;
    mv.force[i] = make_double2(0.0, 0.0);
    return xn;
}

}  // namespace pcp
