/*
 * pcp_gb300.h -- C ABI of the GB300-native (sm_103a) polygon overlap path.
 *
 * Library: libpcp_gb300.so (built in-tree by pycudapolygon_gb300/buildlib.py).
 * Every function returns an int status (PCP_OK == 0) and never exits the
 * process; pcp_last_error() gives the message of the last failure on the
 * calling thread.  Device memory is allocated by pcp_model_create and the
 * pcp_model_set_* / pcp_model_initialize_* functions that size the model's
 * buffers (as the reference's setters do), by model calls whose contact
 * buffers must grow, and by pcp_project_force / pcp_shake_project, which
 * keep one process-wide scratch buffer that grows to the largest vertex
 * count they have seen.
 *
 * Two layers, each replacing one seam of camdennis/pyCudaPolygon:
 *
 *  1. pcp_model_*  -- a handle per simulated system.  Each call is one method
 *     of the reference's `class Model` (src/model.hpp:18-107) as bound by
 *     pybind11 (src/pybindWrapper.cpp:25-107); the citation above each
 *     declaration names the method it replaces.  Host arrays cross by copy,
 *     as the reference's std::vector setters and getters do.  The pybind11
 *     module `libpyCudaPolygon` built beside this library is a thin wrapper
 *     over this layer with the reference's exact method table.
 *
 *  2. pcp_* kernels -- stateless launchers on caller-owned device buffers
 *     (plain pointers + sizes + a cudaStream_t passed as void*).  Each one
 *     replaces an `extern "C"` wrapper of src/model.cu that the reference's
 *     C++ host code declares at src/model.cpp:17-56.
 *
 * One device per process: the library serves the device that is current
 * when it is first used (its SM count sizes the grids, and kernel launch
 * attributes are set once), as one process per GPU does.
 *
 * Data layout (identical to the reference): positions and forces are
 * interleaved FP64 [x0, y0, x1, y1, ...] in the unit periodic box; polygon p
 * owns vertices [startIndices[p], startIndices[p+1]) in counter-clockwise
 * order; contact records are packed uint64 keys
 * (sj << 48 | si << 32 | i << 16 | j, src/kernels.cuh:861-874).
 */
#ifndef PCP_GB300_H
#define PCP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PCP_OK = 0,
    PCP_ERR_ARG = 1,       /* bad argument or size */
    PCP_ERR_CUDA = 2,      /* a CUDA runtime call failed */
    PCP_ERR_CAPACITY = 3,  /* a per-pair or per-polygon size limit was exceeded */
    PCP_ERR_LIMIT = 4,     /* more than 65535 polygons or vertices per polygon */
    PCP_ERR_STATE = 5,     /* call order (e.g. no startIndices yet) */
    PCP_ERR_NUMERIC = 6    /* a kernel met non-finite input it cannot process */
};

/* simControlStruct::modelEnum (src/enumTypes.h:6) */
enum { PCP_MODEL_NORMAL = 0, PCP_MODEL_EDGE_ONLY = 1, PCP_MODEL_AREA_ONLY = 2,
       PCP_MODEL_SOFT_BODY = 3, PCP_MODEL_ABNORMAL = 4, PCP_MODEL_HYBRID = 5 };
/* minimizerEnum (src/enumTypes.h:9) */
enum { PCP_MINIMIZER_GD = 0, PCP_MINIMIZER_FIRE = 1 };

/* Output pointers of the scalar getters must not be NULL (PCP_ERR_ARG);
 * the array getters take the capacity of their output. */
/* Message of the last failed call on this thread ("" if none). */
const char* pcp_last_error(void);
/* Library version string. */
const char* pcp_version(void);

/* ======================================================================
 * 1. Model handle API
 * ====================================================================== */
typedef struct pcp_model pcp_model;

/* Model::Model(int) (model.cpp:60-101) */
int pcp_model_create(int size, pcp_model** out);
/* Model::~Model (model.cpp:103-160) */
int pcp_model_destroy(pcp_model* m);
/* Stream the model launches on (NULL = the legacy default stream). */
int pcp_model_set_stream(pcp_model* m, void* cuda_stream);

/* ---- setters ---- */
/* Model::setNumVertices (model.cpp:600-628) */
int pcp_model_set_num_vertices(pcp_model* m, int n);
/* Model::setPositions (model.cpp:522-528): len must be 2*numVertices, else
 * the reference prints and ignores the call; here PCP_ERR_ARG is returned
 * after the same message. */
int pcp_model_set_positions(pcp_model* m, const double* host, int len);
/* Model::setForces (model.cpp:530-535) */
int pcp_model_set_forces(pcp_model* m, const double* host, int len);
/* Model::setStartIndices (model.cpp:537-598) */
int pcp_model_set_start_indices(pcp_model* m, const int* host, int len);
/* Model::setTargetAreas (model.cpp:634-636) */
int pcp_model_set_target_areas(pcp_model* m, const double* host, int len);
/* Model::setTargetEdgeLengths (model.cpp:630-632) */
int pcp_model_set_target_edge_lengths(pcp_model* m, const double* host, int len);
/* Model::setMaxEdgeLength (model.cpp:513-516): boxSize = floor(1/l) */
int pcp_model_set_max_edge_length(pcp_model* m, double l);
/* Model::setModelEnum (model.cpp:518-520) */
int pcp_model_set_model_enum(pcp_model* m, int model_enum);
/* Model::setStiffness / setCompressibility (model.cpp:638-644) */
int pcp_model_set_stiffness(pcp_model* m, double k);
int pcp_model_set_compressibility(pcp_model* m, double c);
int pcp_model_get_stiffness(pcp_model* m, double* out);
int pcp_model_get_compressibility(pcp_model* m, double* out);

/* ---- initialisers and updaters ---- */
/* Model::initializeNeighborCells (model.cpp:176-229): topology */
int pcp_model_initialize_neighbor_cells(pcp_model* m);
/* Model::updatePolygonGeometry (model.cpp:313-315; model.cu:113-163) */
int pcp_model_update_polygon_geometry(pcp_model* m);
/* Model::updateNeighborCells (model.cpp:252-254; model.cu:308-385) */
int pcp_model_update_neighbor_cells(pcp_model* m);
/* Model::updateNeighbors (model.cpp:256-307; model.cu:393-411): finds every
 * edge-edge crossing the reference's 3x3 cell scan finds */
int pcp_model_update_neighbors(pcp_model* m);
/* Model::updateValidAndCounts (model.cpp:309-311) */
int pcp_model_update_valid_and_counts(pcp_model* m);
/* Model::updateCompactedIntersections (model.cpp:347-349) */
int pcp_model_update_compacted_intersections(pcp_model* m);
/* Model::updateOutersections (model.cpp:351-361) */
int pcp_model_update_outersections(pcp_model* m);
/* Model::updateForceEnergy (model.cpp:363-395) */
int pcp_model_update_force_energy(pcp_model* m);
/* Model::projectForce (model.cpp:337-344; model.cu:165-206) */
int pcp_model_project_force(pcp_model* m);
/* Model::shakeProject (model.cpp:317-322; model.cu:619-636) */
int pcp_model_shake_project(pcp_model* m, int n_iter, double tol, int* iters_out);
/* xpbdProjectCUDA (model.cu:209-278); not bound by the reference */
int pcp_model_xpbd_project(pcp_model* m, int n_iter, double tol, int* iters_out);
/* Model::updatePositions (model.cpp:397-399) */
int pcp_model_update_positions(pcp_model* m, double dt);
/* Model::resetVelocities (model.cpp:401-403) */
int pcp_model_reset_velocities(pcp_model* m);
/* Model::resetAreas (model.cpp:507-509) */
int pcp_model_reset_areas(pcp_model* m);
/* Model::saveTentativePositions (model.cpp:328-330) */
int pcp_model_save_tentative_positions(pcp_model* m);
/* Model::getMaxEffectiveForce (model.cpp:332-335) */
int pcp_model_get_max_effective_force(pcp_model* m, double dt, int minimizer, double* out);
/* Model::sortKeys (model.cpp:238-240) */
int pcp_model_sort_keys(pcp_model* m, int end_bit);
/* Model::updateOverlapArea (model.cpp:824-847) */
int pcp_model_update_overlap_area(pcp_model* m, int point_density);

/* Model::minimizeFIREStep (model.cpp:405-486); out = {E, dt, alpha, nPos} */
int pcp_model_fire_step(pcp_model* m, double dt, double alpha, int n_pos, double dt_max,
                        double alpha_start, double f_alpha, double f_inc, double f_dec,
                        int n_min, int shake_iter, double out[4]);
/* Model::minimizeFIRE (model.cpp:488-504); out = {E, dt, steps}.  Runs the
 * steps as CUDA-graph launches with the stop test on the device. */
int pcp_model_minimize_fire(pcp_model* m, double max_force_threshold, double dt_init,
                            int max_steps, double dt_max, double alpha_start, double f_alpha,
                            double f_inc, double f_dec, int n_min, int shake_iter,
                            double out[3]);

/* Device-resident FIRE driver (the loop of Model::minimizeFIRE, model.cpp:
 * 488-504, and of the Python minimizeFIRELoop, pyCudaPolygon.py:653-672,
 * without a host round trip per step).
 * pcp_model_fire_setup: reset velocities, evaluate force (+ projection for the
 *   normal model) and load the FIRE parameters; max_force_threshold is the
 *   stop test, max_steps the step limit (<= 0: none).
 * pcp_model_fire_continue: enqueue n_steps step-graph launches on the model's
 *   stream and return at once; steps after the stop test or the limit are
 *   no-ops on the device.
 * pcp_model_fire_status: wait for the stream; out = {E, dt, alpha, nPos,
 *   max|F|, steps done, converged, last SHAKE iterations}.  A contact buffer
 *   that overflowed during a step is grown here and the step is rolled back
 *   to its start; *redo_out is then 1 and the caller continues. */
int pcp_model_fire_setup(pcp_model* m, double max_force_threshold, double dt_init,
                         int max_steps, double dt_max, double alpha_start, double f_alpha,
                         double f_inc, double f_dec, int n_min, int shake_iter);
int pcp_model_fire_continue(pcp_model* m, int n_steps);
int pcp_model_fire_status(pcp_model* m, double out[8], int* redo_out);
/* The stop rule of the reference's Python FIRE driver (pyCudaPolygon.py:
 * 719-727) for the next pcp_model_fire_setup run: a step whose returned
 * energy differs from the previous step's by less than energy_tol counts as
 * stagnant (the count is never reset), and the run stops on the device once
 * the count exceeds stagnant_limit.  stagnant_limit < 0 turns the rule off
 * (the default: only |F|max and the step limit stop a run). */
int pcp_model_fire_set_stop_rule(pcp_model* m, double energy_tol, int stagnant_limit);
/* The last device-resident run: out = {stopped by the stagnation rule (0/1),
 * min, sum and max over its steps of the last SHAKE iteration count}. */
int pcp_model_fire_run_stats(pcp_model* m, double out[4]);
/* model.minimizeFIRE of the reference's Python layer (pyCudaPolygon.py:
 * 674-731; its loop minimizeFIRELoop, :653-672) as one call: the same model
 * calls before the loop (initForceEnergy, which resets the cell size to 0.5,
 * and the small gradient step), then the FIRE steps run as step-graph
 * launches stopped on the device by |F|max <= max_force_threshold, the
 * step limit or the stagnation rule (|dE| < 1e-15 counted, stop past 5).
 * out = {E, dt, steps, min, sum / max_steps, max of the per-step SHAKE
 * iterations}, the values that driver returns.  max_steps <= 0 only runs
 * the steps before the loop (out[2] = 0). */
int pcp_model_minimize_fire_driver(pcp_model* m, double max_force_threshold, double dt_init,
                                   int max_steps, double dt_max, double alpha_start,
                                   double f_alpha, double f_inc, double f_dec, int n_min,
                                   int shake_iter, double out[6]);

/* The contact search (update of the crossing records) split into its stages,
 * enqueued without waiting: 0 = per-polygon prepass and broad phase
 * (bounding circles, grid counting sort, candidate pairs), 1 = narrow phase
 * (warp-per-pair kernel, its block fallback, and the exit matching's
 * empty-group fix-up), 2 = nothing left to enqueue (kept for callers that
 * run the three stages).
 * Overflow is only detected by pcp_model_update_neighbors. */
int pcp_model_contacts_stage(pcp_model* m, int stage);

/* No reference counterpart: positions from a device buffer of 2*numVertices
 * doubles (device-to-device copy on the model's stream), for CUDA-aware
 * callers such as the PyTorch edge.  Same effect as pcp_model_set_positions. */
int pcp_model_set_positions_device(pcp_model* m, const double* d_pos, int len);
/* The overlap energy with a per-vertex output written to the device buffer
 * d_out (2*numVertices doubles, overwritten), the energy to *energy_out.
 * search = 1 runs the contact search on the current positions first (else
 * the records of the last search are used, as updateForceEnergy does).
 *   mode 0: the reference's energy and force (model.cpp:363-395;
 *           kernels.cuh:1067-1424), computed record by record -- the same
 *           values as pcp_model_update_force_energy within rounding.
 *   mode 1: the energy with the crossing points taken exactly (not from the
 *           float-rounded parameters, kernels.cuh:857-858) and its exact
 *           gradient dE/dx, including the dependence of each chain's start
 *           point that the reference's force leaves out; no reference
 *           counterpart (the backward of the PyTorch autograd function). */
int pcp_model_overlap_energy_gradient(pcp_model* m, int mode, int search, double* energy_out,
                                      double* d_out);

/* ---- getters (model.cpp:654-893; bound among pybindWrapper.cpp:35-104);
 * arrays are copied into caller memory ---- */
int pcp_model_get_num_vertices(pcp_model* m, int* out);
int pcp_model_get_num_polygons(pcp_model* m, int* out);
int pcp_model_get_num_intersections(pcp_model* m, int* out);
int pcp_model_get_max_neighbors(pcp_model* m, int* out);
int pcp_model_get_box_size(pcp_model* m, int* out);
int pcp_model_get_model_enum(pcp_model* m, int* out);
int pcp_model_get_last_shake_iters(pcp_model* m, int* out);
int pcp_model_get_energy(pcp_model* m, double* out);
/* Model::getMaxUnbalancedForce (model.cpp:881-883): max |force component|.
 * Called right after pcp_model_fire_step (no other call on the model in
 * between) it returns the maximum the step already read back with its
 * control block, without a launch: the reference's per-step Python loop
 * (pyCudaPolygon.py:666-668) asks for it after every step. */
int pcp_model_get_max_unbalanced_force(pcp_model* m, double* out);
int pcp_model_get_max_edge_length(pcp_model* m, double* out);
int pcp_model_get_overlap_area(pcp_model* m, double* out);
/* The array getters take the capacity of `out` in elements and fail with
 * PCP_ERR_ARG when it is too small; *len_out receives the element count. */
int pcp_model_get_positions(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_forces(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_velocities(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_areas(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_com(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_perimeters(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_edge_lengths(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_constraints(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_target_areas(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_target_edge_lengths(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_start_indices(pcp_model* m, int* out, int cap, int* len_out);
int pcp_model_get_shape_id(pcp_model* m, int* out, int cap, int* len_out);
int pcp_model_get_neighbor_cells(pcp_model* m, int* out, int cap, int* len_out);
int pcp_model_get_neighbor_indices(pcp_model* m, int* out, int cap, int* len_out);
int pcp_model_get_box_counts(pcp_model* m, int* out, int cap, int* len_out);
int pcp_model_get_neighbors(pcp_model* m, int* out, int cap, int* len_out);
int pcp_model_get_num_neighbors(pcp_model* m, int* out, int cap, int* len_out);
int pcp_model_get_inside_flag(pcp_model* m, uint8_t* out, int cap, int* len_out);
int pcp_model_get_shape_counts(pcp_model* m, int* out, int cap, int* len_out);
int pcp_model_get_intersections(pcp_model* m, uint64_t* out, int cap, int* len_out);
int pcp_model_get_outersections(pcp_model* m, uint64_t* out, int cap, int* len_out);
int pcp_model_get_tu(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_ut(pcp_model* m, double* out, int cap, int* len_out);
int pcp_model_get_keys(pcp_model* m, uint32_t* out, int cap, int* len_out);
int pcp_model_get_intersections_counter(pcp_model* m, int* out, int cap, int* len_out);

/* No reference counterpart: device views of the model's state (valid until
 * the next resize); for zero-copy use from CUDA-aware callers.  Interleaved FP64 [2*numVertices]. */
int pcp_model_device_positions(pcp_model* m, double** out);
int pcp_model_device_forces(pcp_model* m, double** out);
/* No reference counterpart: pair evaluations since creation, polygon pairs
 * a < b with overlapping bounding circles taken through the contact search. */
int pcp_model_get_pair_count(pcp_model* m, long long* out);
/* No reference counterpart: pairs a < b handed to the narrow phase since
 * creation (bounding circles meet and boxes within the crossing margin meet;
 * self pairs not counted) -- the pair evaluations a benchmark counts. */
int pcp_model_get_narrow_pair_total(pcp_model* m, long long* out);
/* No reference counterpart: pairs the last contact search handed to the
 * narrow phase, polygon pairs
 * a < b whose bounding boxes are within the crossing margin, and self pairs
 * (polygons not certified simple). */
int pcp_model_get_narrow_pair_count(pcp_model* m, int* pairs_out, int* self_out);
/* ======================================================================
 * Learned warm start (no counterpart in the reference): the dense products
 * and the neighbour sums of a small message-passing network over the
 * contact graph.  FIRE remains the minimiser; the network only proposes a
 * starting point.
 * ====================================================================== */
/* C[m,n] = A[m,k] B[n,k]^T (+ bias[n]) (then ReLU when relu != 0) on the
 * tensor cores: A and B BF16, row-major, k a multiple of 8; C FP32,
 * row-major; A, B and C 16-byte aligned.  splits > 1 divides k over blocks
 * that add into C (which the caller zeroes; bias added once, no ReLU).
 * Asynchronous on the stream. */
int pcp_gemm_bf16(const void* d_a, const void* d_b, float* d_c, int m, int n, int k,
                  const float* d_bias, int relu, int splits, void* stream);
/* 1 in *out when a wait inside a GEMM launched since the last call ran out
 * (its results are then not to be used); clears the flag.  Synchronises. */
int pcp_gemm_status(int* out);
/* out[i,:] = scale * sum over j in col[rowptr[i]..rowptr[i+1]) of h[j,:],
 * BF16 rows of f (even) values, FP32 sums; h and out 4-byte aligned.  The
 * device arrays are not read on the host: rowptr[0..v] must be
 * non-decreasing and every col entry a row of h. */
int pcp_graph_sum_bf16(const int* d_rowptr, const int* d_col, const void* d_h, void* d_out,
                       int v, int f, float scale, void* stream);

/* No reference counterpart: bytes of the per-model control block that a
 * FIRE step reads back to the host (counters and FIRE scalars). */
int pcp_control_block_bytes(void);
/* Kernel launches issued by the model since creation (for accounting). */
int pcp_model_get_launch_count(pcp_model* m, long long* out);

/* ======================================================================
 * 1b. Many independent systems (no reference counterpart: the reference
 *     runs one system per Model)
 * ====================================================================== */
typedef struct pcp_batch pcp_batch;
int pcp_batch_create(pcp_batch** out);
/* Destroys the batch only; the models stay with their owner. */
int pcp_batch_destroy(pcp_batch* b);
/* Adds a configured model (start indices, positions, targets, topology);
 * the batch does not take ownership. */
int pcp_batch_add(pcp_batch* b, pcp_model* m);
int pcp_batch_size(pcp_batch* b, int* out);
/* Streams the systems are spread over (default 16) and FIRE steps per
 * graph launch (default 8). */
int pcp_batch_set_streams(pcp_batch* b, int n_streams, int chunk_steps);
/* Minimises every system of the batch: each system gets a stream of the
 * batch's pool and is prepared as rule says (1: the reference's Python
 * driver, pyCudaPolygon.py:674-731, with its stagnation stop; 0:
 * Model::minimizeFIRE, model.cpp:488-504), then each launch runs
 * chunk_steps FIRE steps of one system; the control blocks are read back
 * once per chunk and stopped systems drop out.  out[4k..4k+3] = {E, dt,
 * steps, stop: 1 |F|max <= thr, 2 stagnation, 0 step limit} of system k.
 * The models get their own streams back. */
int pcp_batch_minimize_fire(pcp_batch* b, int rule, double max_force_threshold, double dt_init,
                            int max_steps, double dt_max, double alpha_start, double f_alpha,
                            double f_inc, double f_dec, int n_min, int shake_iter, double* out);
/* Launch shapes of a model's narrow phase and overlap-force pass (blocks;
 * 0 = the default of 4 per SM).  Any grid covers the work; the best one
 * depends on the system's size and on what runs beside it. */
int pcp_model_set_launch_shape(pcp_model* m, int narrow_blocks, int force_blocks);
int pcp_model_get_launch_shape(pcp_model* m, int out[2]);
/* Autotuner: systems grouped by polygon count (classes [2^k, 2^(k+1)));
 * per class, each candidate grid (SMs x {1/4, 1/2, 1, 2, 4} blocks) runs
 * `steps` FIRE steps of the class's systems together from the same start
 * positions (restored afterwards) and the fastest is set on the class's
 * models.  shapes_out (2 per system, may be NULL) receives the choices;
 * pcp_batch_autotune_report gives the timing table as JSON. */
int pcp_batch_autotune(pcp_batch* b, int steps, int* shapes_out);
int pcp_batch_autotune_report(pcp_batch* b, char* buf, int cap, int* len_out);

/* ======================================================================
 * 2. Stateless kernels on caller-owned device buffers (stream = cudaStream_t)
 * ====================================================================== */
/* A negative size, a NULL buffer for a non-empty input, or box_size < 1
 * returns PCP_ERR_ARG before any launch.  pcp_project_force and
 * pcp_shake_project read d_start back (they size their scratch from it)
 * and return PCP_ERR_ARG unless it is CSR offsets: start[0] == 0, never
 * decreasing.  The other launchers do not read device arrays on the host. */

/* topology: updateShapeIdKernel + computeNextPrevKernel
 * (model.cu:77-81, 387-391; kernels.cuh:127-135, 652-659) */
int pcp_topology(const int* d_start, int num_polygons, int num_vertices,
                 int* d_shape_id, int* d_next, int* d_prev, void* stream);

/* updatePolygonGeometryCUDA (model.cu:113-163).  One warp per polygon;
 * outputs areas, centres of mass (wrapped), perimeters, edge lengths, the
 * three normalised constraint vectors [6V] and the longest edge. */
int pcp_polygon_geometry(const double* d_pos, const int* d_start, int num_polygons,
                         int num_vertices, double* d_edge_lengths, double* d_areas,
                         double* d_com_x, double* d_com_y, double* d_perimeters,
                         double* d_constraints, double* d_max_edge_length, void* stream);

/* updateNeighborCellsKernel (kernels.cuh:661-707): cell of each edge midpoint */
int pcp_neighbor_cells(const double* d_pos, const int* d_start, const int* d_shape_id,
                       int num_vertices, int box_size, int* d_cell_location, void* stream);

/* projectForceCUDA (model.cu:165-206): removes from each polygon's force the
 * span of its edge-length gradients and of its (normalised) area gradient
 * d_constraints[6k+0..1].  Any n per polygon. */
int pcp_project_force(const double* d_pos, const int* d_start, int num_polygons,
                      const double* d_constraints, double* d_force, void* stream);

/* shakeProjectCUDA (model.cu:619-636): projects each polygon onto
 * |edge| = targetEdgeLength[p], area = targetArea[p]; *d_max_iters receives
 * the largest iteration count (failure when >= max_iter). */
int pcp_shake_project(double* d_pos, const int* d_start, int num_polygons,
                      const double* d_target_edge_lengths, const double* d_target_areas,
                      int max_iter, double tol, int* d_max_iters, void* stream);

/* No counterpart in the reference: pcp_shake_project for callers that may
 * not allocate device memory -- plugins whose host owns the device's memory
 * through its own pool and hands the plugin only the buffers it passes in,
 * and loops where the device-wide synchronisation of cudaMalloc/cudaFree is
 * not allowed.  It always runs the warp-per-polygon SHAKE kernel with its
 * workspace in global memory (pcp_shake_project runs the register-resident
 * one-vertex-per-lane form when no polygon exceeds 32 vertices); positions
 * agree with pcp_shake_project within the 1e-12 SHAKE tolerance and the
 * iteration counts are the same.  The workspace is a static device array of
 * this library sized for PCP_SHAKE_NOALLOC_MAX_VERTICES vertices (4.5 MiB);
 * the call makes no cudaMalloc, cudaFree or other allocation.
 *   - start must be CSR offsets: start[0] == 0 and start never decreasing.
 *     A one-block kernel checks that and start[num_polygons] against the
 *     array before anything else runs, and the call waits for `stream` to
 *     read its verdict: offsets that are not CSR return PCP_ERR_ARG, more
 *     than PCP_SHAKE_NOALLOC_MAX_VERTICES vertices PCP_ERR_CAPACITY, and
 *     neither launches the SHAKE kernel or touches d_max_iters.
 *   - The first call on a device looks up the array's device address (it
 *     may load the library's kernels onto that device); make that first
 *     call before any stream capture.
 *   - Every call on a device shares the one array and it keeps the last
 *     call's contents (each polygon writes its part before reading it;
 *     *d_max_iters is cleared by the call).  Calls whose kernels overlap on
 *     the GPU -- on two streams, or from two host threads -- race on it. */
#define PCP_SHAKE_NOALLOC_MAX_VERTICES 16384
int pcp_shake_project_noalloc(double* d_pos, const int* d_start, int num_polygons,
                              const double* d_target_edge_lengths,
                              const double* d_target_areas, int max_iter, double tol,
                              int* d_max_iters, void* stream);

/* updatePositionsKernel (kernels.cuh:1433-1438): x = frac(x + dt F) */
int pcp_update_positions(double* d_pos, const double* d_force, int num_vertices,
                         double dt, void* stream);

/* No reference counterpart: d_y[i] = the reciprocal the projection's
 * area-gradient removal uses in place of a division (two Newton-Raphson
 * steps from the FP32 reciprocal), for 2^-126 <= |d_x[i]| < 2^126; exposed
 * so its error bound can be tested against 1/x. */
int pcp_rcp_newton(const double* d_x, double* d_y, int n, void* stream);

#ifdef __cplusplus
}
#endif
#endif
