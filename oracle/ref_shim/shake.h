/*
 * Build shim for the reference's missing src/shake.h (TEST INFRASTRUCTURE;
 * used only by oracle/ref_build.py).
 *
 * src/model.cu:16 includes shake.h, which the reference does not ship;
 * shakeProjectCUDA (src/model.cu:619-636) launches shakeProjectKernel from
 * it.  This stub has the launch's signature and does nothing.  The
 * golden-vector driver (oracle/ref_golden.cpp) never calls shakeProject, so
 * no result depends on it.
 */
#pragma once

__global__ void shakeProjectKernel(int, const int*, const int*, const int*, double*,
                                   const double*, const double*, int, double, int*) {}
