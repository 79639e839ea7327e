/*
 * pcp_oracle.h -- CPU oracle for the pyCudaPolygon hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, FP64, -ffp-contract=off
 * restatement of the reference's algorithm (camdennis/pyCudaPolygon,
 * src/kernels.cuh, src/model.cu, src/model.cpp).  It exists to check the
 * CUDA implementation and to be timed as the CPU baseline.  Nothing in the
 * product path may call it: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py load it.
 *
 * Parity status:
 *   - contact list (cells, crossings, packing, sort order, outersections),
 *     geometry, overlap energy/force, projection: pinned against the
 *     reference's known answers (tests/testSaver neighbour answer) and its
 *     Python twins (getDf, getConstrainedForcePython, getCentersOfMass,
 *     shoelace), via the fixtures in tests/golden/.
 *   - FIRE and SHAKE: parity unpinned.  The reference's FIRE.h and shake.h
 *     are absent from its tree; both are restated from their call contract
 *     (model.cpp:405-486, model.cu:576-636) and the published algorithms.
 *
 * The model object mirrors the reference's `class Model` (src/model.hpp)
 * method for method; every function cites the reference code it restates.
 */
#ifndef PCP_ORACLE_H
#define PCP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* simControlStruct::modelEnum (src/enumTypes.h:6) */
enum { ORC_NORMAL = 0, ORC_EDGE_ONLY = 1, ORC_AREA_ONLY = 2, ORC_SOFT_BODY = 3,
       ORC_ABNORMAL = 4, ORC_HYBRID = 5 };

typedef struct orc_model orc_model;

/* ---- stateless device-function restatements (kernels.cuh:115-222) ---- */
double orc_wrap(double x);
double orc_h(const double pt1[2], const double pt2[2], const double sp[2]);
void   orc_g12(const double pt1[2], const double pt2[2], const double sp[2],
               double g1[2], double g2[2]);
void   orc_getDf(const double vi[2], const double vzi[2], const double vj[2],
                 const double vzj[2], double df[16]);
/* One crossing test exactly as updateNeighborsKernel (kernels.cuh:778-807).
 * Returns 1 when edge (p, p2) crosses edge (q, q2); fills tt, uu, denom. */
int    orc_cross(const double p[2], const double p2[2], const double q[2],
                 const double q2[2], double* tt, double* uu, double* denom);

/* Cell of the midpoint of the edge starting at vertex idx
 * (updateNeighborCellsKernel, kernels.cuh:661-707). */
int    orc_midpoint_cell(const double* pos, const int* startIndices, const int* shapeId,
                         int size, int idx, int B);

/* ---- model (src/model.hpp:18-185) ---- */
orc_model* orc_create(int size);
void orc_destroy(orc_model* m);
void orc_set_threads(int nthreads);

void orc_set_num_vertices(orc_model* m, int n);
int  orc_set_positions(orc_model* m, const double* pos, int len);
void orc_set_forces(orc_model* m, const double* f, int len);
void orc_set_velocities(orc_model* m, const double* v, int len);
void orc_set_energy(orc_model* m, double e);
void orc_set_start_indices(orc_model* m, const int* si, int len);
void orc_set_target_areas(orc_model* m, const double* a, int len);
void orc_set_target_edge_lengths(orc_model* m, const double* l, int len);
void orc_set_max_edge_length(orc_model* m, double l);
void orc_set_model_enum(orc_model* m, int e);
void orc_set_stiffness(orc_model* m, double k);
void orc_set_compressibility(orc_model* m, double c);

void orc_initialize_neighbor_cells(orc_model* m);
void orc_update_polygon_geometry(orc_model* m);
void orc_update_neighbor_cells(orc_model* m);
int  orc_update_neighbors(orc_model* m);
void orc_update_outersections(orc_model* m);
void orc_update_force_energy(orc_model* m);
void orc_project_force(orc_model* m);
int  orc_shake_project(orc_model* m, int nIter, double tol);
int  orc_xpbd_project(orc_model* m, int nIter, double tol);
void orc_update_positions(orc_model* m, double dt);
void orc_reset_velocities(orc_model* m);
void orc_reset_areas(orc_model* m);
void orc_save_tentative_positions(orc_model* m);
double orc_get_max_effective_force(orc_model* m, double dt, int minimizerFIRE);
double orc_get_max_unbalanced_force(orc_model* m);
/* Model::minimizeFIREStep (model.cpp:405-486); out[4] = E, dt, alpha, nPos */
void orc_fire_step(orc_model* m, double dt, double alpha, int nPos, double dtMax,
                   double alphaStart, double fAlpha, double fInc, double fDec,
                   int nMin, int shakeIter, double out[4]);
/* Model::minimizeFIRE (model.cpp:488-504); out[3] = E, dt, steps */
void orc_minimize_fire(orc_model* m, double thr, double dt0, int maxSteps,
                       double dtMax, double alphaStart, double fAlpha, double fInc,
                       double fDec, int nMin, int shakeIter, double out[3]);

/* ---- getters (model.cpp:654-893); they return internal arrays ---- */
int orc_num_vertices(const orc_model* m);
int orc_num_polygons(const orc_model* m);
int orc_num_intersections(const orc_model* m);
int orc_max_neighbors(const orc_model* m);
int orc_box_size(const orc_model* m);
int orc_last_shake_iters(const orc_model* m);
int orc_fire_first_shake_iters(const orc_model* m);
double orc_energy(const orc_model* m);
double orc_max_edge_length(const orc_model* m);
const double*   orc_positions(const orc_model* m);
const double*   orc_forces(const orc_model* m);
const double*   orc_velocities(const orc_model* m);
const double*   orc_areas(const orc_model* m);
const double*   orc_com_x(const orc_model* m);
const double*   orc_com_y(const orc_model* m);
const double*   orc_edge_lengths(const orc_model* m);
const double*   orc_constraints(const orc_model* m);
const double*   orc_perimeters(const orc_model* m);
const int*      orc_shape_id(const orc_model* m);
const int*      orc_start_indices(const orc_model* m);   /* P+1 */
const int*      orc_cell_location(const orc_model* m);
const int*      orc_neighbor_indices(const orc_model* m);
const int*      orc_box_starts(const orc_model* m);
const int*      orc_neighbors(const orc_model* m);
const int*      orc_num_neighbors(const orc_model* m);
const uint8_t*  orc_inside(const orc_model* m);
const int*      orc_shape_counts(const orc_model* m);
const uint64_t* orc_intersections(const orc_model* m);
const uint64_t* orc_outersections(const orc_model* m);
const double*   orc_tu(const orc_model* m);
const double*   orc_ut(const orc_model* m);
const double*   orc_target_areas(const orc_model* m);
const double*   orc_target_edge_lengths(const orc_model* m);

/* grid-point overlap estimate (updateOverlapAreaKernel + Model::updateOverlapArea) */
double orc_update_overlap_area(orc_model* m, int pointDensity);

#ifdef __cplusplus
}
#endif
#endif
