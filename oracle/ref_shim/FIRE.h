/*
 * Build shim for the reference's missing src/FIRE.h (TEST INFRASTRUCTURE;
 * used only by oracle/ref_build.py).
 *
 * src/model.cu:15 includes FIRE.h, which the reference does not ship.  The
 * wrappers at src/model.cu:576-608 need five symbols from it.  They are
 * declared here with the signatures those call sites imply, as stubs that do
 * nothing: the golden-vector driver (oracle/ref_golden.cpp) never reaches the
 * FIRE step, so the reference build is used only for the evaluation path
 * (contacts, outersections, overlap energy and force, geometry, projection,
 * soft-body terms, the grid overlap estimate).  dotProductFIRE aborts if it is
 * ever called, so a stub can never pass for a result.
 */
#pragma once
#include <cstdio>
#include <cstdlib>

__global__ void updatePositionAndVelocityFIREKernel(int, double*, double*, const double*, double) {}
__global__ void updateVelocityFIREKernel(int, double*, const double*, double) {}
__global__ void bendVelocityTowardsForceFIREKernel(int, double*, const double*, double, double, double) {}
__global__ void rederiveVelocityFromDisplacementKernel(int, double*, const double*, const double*, double) {}

static double dotProductFIRE(const double*, const double*, int, double*, double*) {
    std::fprintf(stderr, "ref build shim: FIRE.h is absent from the reference; FIRE is not available\n");
    std::abort();
}
