// pcp_internal.h -- internal launchers and device-state layout shared by the
// .cu translation units and the host-side model (model.cpp).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pcp_gb300.h"

namespace pcp {

// Largest polygon the warp-per-pair contact kernel stages in shared memory;
// bigger polygons (and pairs with more crossings than a warp buffers) take
// the block-per-pair path, which handles up to kSlowRing vertices per pair.
constexpr int kFastRing = 64;
constexpr int kFastRecords = 64;
constexpr int kSlowRing = 2048;
constexpr int kSlowRecords = 2048;
// Largest polygon the thread-per-polygon projection / SHAKE kernels accept.
constexpr int kMaxPolyN = 256;
// Largest narrow-phase grid (blocks) a launch shape may ask for; every warp
// of the narrow phase publishes its largest key once, so kMaxCand covers
// them all (4 warps per block, plus the overflow kernel's 4 per block on
// 4 blocks per SM and the block path's 16).
constexpr int kMaxNarrowBlocks = 16384;
constexpr int kMaxCand = 4 * kMaxNarrowBlocks + 4096;
// Broad-phase grid cap per axis.
constexpr int kGridMax = 256;

// Device control block of one model (contact search counters, FIRE scalars).
struct Ctrl {
    // ---- contact search (zeroed at the start of each search) ----
    int numPairs;
    int pairCursor;
    int numRecords;
    int numFix;
    int numSlow;
    int slowCursor;
    int numUnsafe;
    int numSelf;           // self pairs among the candidate pairs
    int numMaxCand;        // entries of ContactWS::maxCand
    int numOver;           // entries of ContactWS::overList
    int overCursor;
    int G;                 // broad-phase grid cells per axis
    unsigned int flags;    // kFlag* bits
    float Rmax;            // largest bounding radius of a well-formed polygon
    unsigned long long maxKey;
    // ---- energy / force ----
    double energy;
    double maxF;           // max |force component| after the last projection
    // ---- FIRE scalars (the reference keeps these on the host) ----
    double dt, alpha;
    double ePre;
    double P, vv, ff;
    double dtMax, alphaStart, fAlpha, fInc, fDec;
    double threshold;
    double outE;           // energy the step returns
    int nPos, nMin, shakeIter;
    int shakeIters1, shakeIters2;
    int shakeLast;         // iterations of the last SHAKE call
    int needRetry;
    int retryGate;         // gate: second SHAKE attempt
    int shakeFailed;
    int rollback;          // the energy-increase rollback was taken
    int rbGate;            // gate: rollback path
    int proceed;           // the step's FIRE velocity update ran
    int active;            // gate: the minimisation is still running
    int converged;
    int stepsDone;
    int stepLimit;
    int errorCode;
    int needsRecovery;     // a contact buffer overflowed during a FIRE step
    int snapNPos;
    double snapDt, snapAlpha;   // FIRE scalars at the start of the step
    unsigned long long pairEvals;   // cumulative candidate pairs (a < b) examined
    unsigned long long narrowEvals; // cumulative pairs handed to the narrow phase (self pairs too)
    unsigned long long selfEvals;   // cumulative self pairs among them
    // last-block tickets of the FIRE step's SHAKE and velocity-mixing kernels
    // (zeroed by k_fire_begin) and the kernels run inside the step graph's
    // conditional bodies (the host counts the unconditional ones)
    unsigned int shakeTicket, bendTicket;
    unsigned long long condLaunches;
    int rbBodyKernels;     // kernels in the rollback body (set by the host)
    // the velocity bend of the last step (model.cpp:471-484), applied by the
    // next step's start or before velocities are read: 0 none, 1 v <- bendA v
    // + bendS F, 2 v <- 0
    int bendMode;
    double bendA, bendS;
    // blocks of the step's force pass finished (its last one decides the
    // energy rollback)
    unsigned int forceTicket;
    // stop rule of the reference's Python driver (pyCudaPolygon.py:719-727):
    // steps whose returned energy moved by less than stagnantTol are counted
    // (never reset); the run stops once the count exceeds stagnantLimit
    // (< 0: rule off)
    double prevE, stagnantTol;
    int stagnant, stagnantLimit, stagnated;
    // per-step SHAKE iterations over the run (min, sum, max), as that driver
    // reports them
    int shakeMinRun, shakeMaxRun;
    long long shakeSumRun;
};

enum : unsigned int {
    kFlagPairOverflow = 1u,
    kFlagRecordOverflow = 2u,
    kFlagSlowOverflow = 4u,
    kFlagFixOverflow = 8u,
    kFlagCapacity = 16u,    // a pair exceeds even the block-per-pair limits
    kFlagNonFinite = 32u,
};

// Contact-search workspace (device memory owned by the model).
struct ContactWS {
    int V = 0, P = 0;
    int capPairs = 0, capRecords = 0, capFix = 0, capSlow = 0;
    double2* edgeVec = nullptr;     // [V] wrap(p_next - p)
    float4* vtx = nullptr;          // [V] (x, y) as float, cell, 0
    float4* polyInfo = nullptr;     // [P] centre x, y, radius, longest edge
    float4* polyBox = nullptr;      // [P] box (x0, x1, y0, y1) relative to vertex 0 (FP32)
    int* polyFlags = nullptr;       // [P] 1 = well formed (safe for the culls)
    int* gridCount = nullptr;       // [G*G] (G <= kGridMax)
    int* gridStart = nullptr;       // [G*G + 1]
    int* gridFill = nullptr;        // [G*G]
    int* sortedPoly = nullptr;      // [P]
    int* unsafeList = nullptr;      // [P]
    int2* pairs = nullptr;          // [capPairs] candidate pairs a <= b
    unsigned long long* recKey = nullptr;    // [capRecords]
    unsigned long long* recOuter = nullptr;  // [capRecords]
    float2* recTU = nullptr;        // [capRecords] (tu.x, tu.y) rounded to float
    float2* recUT = nullptr;        // [capRecords]
    int* fixList = nullptr;         // [capFix] records whose partner group is empty
    int* slowList = nullptr;        // [capSlow] pair indices for the block path
    int* maxCand = nullptr;         // [kMaxCand] records that raised maxKey when written
    int* overList = nullptr;        // [capPairs] pairs whose crossings overflowed a warp slot
    // launch shapes (0: the default, 4 blocks per SM): blocks of the
    // warp-per-pair narrow phase and of the overlap-force pass; both kernels
    // take their work from the record/pair counters, so any grid covers it
    int narrowBlocks = 0, forceBlocks = 0;
};

// The Verlet move of a FIRE step, done by the step-start kernel (pos == null:
// no move): x, v, F in place, and their snapshots.
struct FireMove {
    double2 *pos, *vel, *force, *save, *velSnap, *forceSnap;
    Ctrl* c;
};

// --- launchers (all asynchronous on `st`) ---
cudaError_t launch_topology(const int* start, int P, int V, int* shapeId, int* next, int* prev,
                            cudaStream_t st);
cudaError_t launch_geometry(const double2* pos, const int* start, int P, int V,
                            double* edgeLengths, double* areas, double* comX, double* comY,
                            double* perimeters, double* constraints, double* maxEdge,
                            const int* gate, cudaStream_t st);
cudaError_t launch_neighbor_cells(const double2* pos, const int* start, const int* shapeId,
                                  int V, int B, int* cellLocation, const int* gate,
                                  cudaStream_t st);
cudaError_t launch_update_positions(double* pos, const double* force, int V, double dt,
                                    cudaStream_t st);
cudaError_t launch_reset_areas(double* pos, const int* shapeId, const double* areas,
                               const double* targetAreas, const double* comX,
                               const double* comY, int V, cudaStream_t st);
cudaError_t launch_max_abs(const double* x, int n, double* out, cudaStream_t st);
cudaError_t launch_max_effective_force(const double* pos, const double* posTent,
                                       const double* force, int V, double scale,
                                       double* out, cudaStream_t st);
cudaError_t launch_soft_edge(const double2* pos, const double* targetEdgeLengths,
                             const double* edgeLengths, const int* next, const int* prev,
                             const int* shapeId, int V, double stiffness, double* force,
                             double* energy, const int* gate, cudaStream_t st);
cudaError_t launch_soft_area(const double2* pos, const int* shapeId, const int* next,
                             const int* prev, const double* areas, const double* targetAreas,
                             const int* start, int V, double compressibility, double* force,
                             double* energy, const int* gate, cudaStream_t st);
cudaError_t launch_overlap_area_mc(const double2* pos, const int* start, const int* shapeId,
                                   const int* neighborIndices, const int* boxStarts, int V,
                                   int B, int pointDensity, int* counter,
                                   unsigned long long* sum, cudaStream_t st);

// contacts
cudaError_t contacts_init();
// stages: bit 0 = reset + prepass + broad phase, bit 1 = narrow phase, bit 2 =
// skip the counter reset (done by the caller); cellOut: compute the edge
// midpoint cells in the prepass and store them there (cellLocation unused)
constexpr int kContactsNoReset = 4;
// bit 3: skip the prepass (already run by launch_prepass_move)
constexpr int kContactsNoPrepass = 8;
cudaError_t launch_contacts(const double2* pos, const int* start, const int* shapeId,
                            const int* cellLocation, int P, int V, int B, ContactWS& ws,
                            Ctrl* ctrl, const int* gate, cudaStream_t st, int stages = 3,
                            int* cellOut = nullptr);
// The start of a FIRE step fused with the contact prepass (warp per polygon):
// the control-block resets, the Verlet move of mv (positions moved in place
// and copied to `verlet`, which the search then reads), and the prepass on
// the moved positions with the cells stored in cellOut.
cudaError_t launch_prepass_move(double2* verlet, const int* start, int* cellOut, int P, int B,
                                ContactWS& ws, Ctrl* ctrl, const int* gate, cudaStream_t st,
                                const FireMove& mv);
// edge: the edge vectors wrap(x_next - x) of pos, or nullptr
// decide: the FIRE step's force pass; its last block decides the energy
// rollback (model.cpp:450-453) and sets `rbCond` of the step graph
cudaError_t launch_overlap_force(const double2* pos, const int* start,
                                 int V, ContactWS& ws, Ctrl* ctrl, double2* force,
                                 const int* gate, cudaStream_t st, const double2* edge = nullptr,
                                 int decide = 0, cudaGraphConditionalHandle rbCond = 0);

// constraints
cudaError_t constraints_init();
// nmax: largest vertex count of a polygon (decides whether the per-polygon
// scratch fits in shared memory)
// mainPass: the FIRE step's own pass after a force pass that decided the
// energy rollback (launch_overlap_force with decide): the pass reads that
// decision and does nothing when the rollback runs
// pre ([3V] double2: unit edge tangents, unit area gradients, then the edge
// vectors the overlap force loads): when non-null, the values
// launch_project_pre stored for the current positions
cudaError_t launch_project(const double2* pos, const int* start, int P, int nmax,
                           const double* constraints, double2* force, double* scratch, int V,
                           int areaFromPositions, Ctrl* fireCtrl, const int* gate, double2* vel,
                           cudaStream_t st, int mainPass = 0, const double2* pre = nullptr);
// whether launch_project runs its register (one vertex per lane) form, the
// only one that reads `pre`
bool project_uses_lanes(int P, int nmax);
// the tangents and area gradients of `pos` into pre for launch_project (a
// no-op unless project_uses_lanes(P, nmax))
cudaError_t launch_rcp_newton(const double* x, double* y, int n, cudaStream_t st);
cudaError_t launch_project_pre(const double2* pos, const int* start, int P, int nmax,
                               double2* pre, int V, const int* gate, cudaStream_t st);
// fire (device-resident FIRE step, first SHAKE attempt): the last block to
// finish decides whether the retry runs and sets `retryCond` of the step
// graph; vel (with dtc for dt): also rederive v from the SHAKE displacement
cudaError_t launch_shake(double2* pos, const int* start, int P, int nmax, const double* targetEdge,
                         const double* targetArea, int maxIter, double tol, int* maxItersOut,
                         double* scratch, int V, const int* gate, cudaStream_t st,
                         Ctrl* fire = nullptr, cudaGraphConditionalHandle retryCond = 0,
                         double2* vel = nullptr, const Ctrl* dtc = nullptr);
// scratch doubles per vertex needed by launch_project / launch_shake
constexpr int kScratchPerVertex = 36;
// pcp_shake_project_noalloc: device address of its static workspace on the
// current device, and k_shake launched with every workspace in it
cudaError_t shake_noalloc_scratch(double** out);
// pcp_shake_project_noalloc: checks start[0..P] on the device (0 valid,
// 1 not a CSR offset array, 2 beyond the static workspace) and waits for it.
cudaError_t shake_noalloc_check(const int* start, int P, int* status, cudaStream_t st);
cudaError_t launch_shake_noalloc(double2* pos, const int* start, int P, const double* targetEdge,
                                 const double* targetArea, int maxIter, double tol,
                                 int* maxItersOut, double* scratch, cudaStream_t st);
cudaError_t launch_xpbd_iteration(double2* pos, const int* start, int P,
                                  const double* targetEdge, const double* targetArea,
                                  double* devOut, cudaStream_t st);

// FIRE parameters of a run, written into Ctrl by one thread on the stream
// (no host round trip)
// Overlap energy with a per-vertex output (gradient.cu): kRefForce gives
// the reference's force and energy, kExactGrad the exact gradient of the
// energy taken at the exact crossing points.  `out` (2V doubles) and
// `energy` are added to; `bad` is set on a record outside the polygons.
enum { kRefForce = 0, kExactGrad = 1 };
cudaError_t launch_overlap_energy_grad(const double2* pos, const int* start, int V,
                                       const ContactWS& ws, const Ctrl* ctrl, int mode,
                                       double2* out, double* energy, int* bad, cudaStream_t st);

struct FireScalars {
    double dt, alpha, dtMax, alphaStart, fAlpha, fInc, fDec, threshold;
    int nPos, nMin, shakeIter, stepLimit, resetRun, rbBodyKernels;
    double stagnantTol;
    int stagnantLimit;
};
cudaError_t launch_set_fire_params(Ctrl* c, const FireScalars& f, cudaStream_t st);

// FIRE pieces (device-resident scalars in Ctrl)
cudaError_t launch_fire_begin(double2* pos, double2* vel, double2* force, double2* save,
                              double2* velSnap, double2* forceSnap, double2* verlet, int V,
                              int resetContacts, Ctrl* c, const int* gate, cudaStream_t st);
cudaError_t launch_fire_retry_outcome(double2* pos, double2* vel, const double2* save, int V,
                                      Ctrl* c, cudaStream_t st);
cudaError_t launch_fire_rollback(double2* pos, double2* vel, double2* force, const double2* save,
                                 int V, int resetContacts, Ctrl* c, cudaStream_t st);
cudaError_t launch_zero_force(double2* force, int V, Ctrl* c, const int* gate, cudaStream_t st);
cudaError_t launch_fire_velocity(double2* vel, const double2* force, int V, Ctrl* c,
                                 cudaGraphConditionalHandle rbCond, int useCond,
                                 const int* gate, cudaStream_t st);
cudaError_t launch_fire_maxf(const double2* force, int V, Ctrl* c, const int* gate,
                             cudaStream_t st);
// apply a pending velocity bend (Ctrl::bendMode) and clear it
cudaError_t launch_fire_settle(double2* vel, const double2* force, int V, Ctrl* c,
                               cudaStream_t st);

int sm_count();

// ---- warmstart.cu: tensor-core kernels of the learned warm start ----
// C[m,n] = A[m,k] B[n,k]^T (+ bias, ReLU), BF16 in, FP32 out; 0, -1 when a
// tensor map could not be encoded, else a cudaError_t
int launch_gemm_bf16(const void* a, const void* b, float* c, int m, int n, int k,
                     const float* bias, int relu, int splits, cudaStream_t st);
// reads and clears the flag a timed-out wait of the GEMM sets
cudaError_t gemm_error_flag(int* out);
cudaError_t launch_graph_sum_bf16(const int* rowptr, const int* col, const void* h, void* out,
                                  int v, int f, float scale, cudaStream_t st);

}  // namespace pcp
