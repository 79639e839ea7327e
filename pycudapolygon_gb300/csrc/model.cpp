// model.cpp -- host side of the GB300 polygon path: the model object behind
// the pcp_model_* C ABI (include/pcp_gb300.h) and the stateless pcp_*
// launchers.  It mirrors the reference's `class Model` (camdennis/
// pyCudaPolygon src/model.hpp, src/model.cpp) method by method, but
//   * never calls exit(): every failure is a status code + message;
//   * allocates once per size change (no per-call cudaMalloc/cudaFree);
//   * runs a FIRE step as one CUDA-graph launch with every scalar of the
//     reference's host loop (dt, alpha, nPos, E_pre, rollback decisions)
//     kept on the device, and one small device-to-host read per step;
//   * keeps contact records grouped by polygon pair and only restores the
//     reference's sorted (si, i, j, sj) order when a getter asks for it.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "pcp_gb300.h"
#include "pcp_internal.h"

using namespace pcp;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t _e = (call);                                                         \
        if (_e != cudaSuccess)                                                           \
            return fail(PCP_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(_e),   \
                        __FILE__, __LINE__);                                             \
    } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
    if (*p) { cudaFree(*p); *p = nullptr; }
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e == cudaSuccess) e = cudaMemset(*p, 0, n * sizeof(T));
    return e;
}
template <typename T>
void dfree(T** p) {
    if (*p) { cudaFree(*p); *p = nullptr; }
}

// Stream-ordered allocation for the contact workspace, which grows inside
// FIRE runs (the reference's resize-and-retry): cudaMalloc and cudaFree wait
// for the whole device, which stalled every other system of a batch each time
// one system's buffers grew.  The device's default pool keeps up to 8 GiB of
// freed memory for reuse.
void keep_pool_memory() {
    static bool done = false;
    if (done) return;
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long keep = 8ull << 30;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done = true;
}
template <typename T>
cudaError_t dalloc_async(T** p, size_t n, cudaStream_t st) {
    if (*p) {
        cudaError_t e = cudaFreeAsync(*p, st);
        *p = nullptr;
        if (e != cudaSuccess) return e;
    }
    if (n == 0) n = 1;
    cudaError_t e = cudaMallocAsync((void**)p, n * sizeof(T), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, n * sizeof(T), st);
    return e;
}
template <typename T>
void dfree_async(T** p, cudaStream_t st) {
    if (*p) { cudaFreeAsync(*p, st); *p = nullptr; }
}

}  // namespace

struct pcp_model {
    // host-side parameters
    int modelType = PCP_MODEL_NORMAL;
    int V = 0, P = 0;
    int nmax = 0;          // largest polygon
    int boxSize = 2;
    double maxEdgeLengthSet = 0.5;
    int maxNeighbors = 100;
    int numIntersections = 0;
    double stiffness = 0.0, compressibility = 0.0;
    int lastShakeIters = 0;
    int pointDensity = -1;
    double overlapArea = 0.0;
    bool topology = false;
    bool geometryStale = false;   // geometry of the current positions not yet computed
    bool geomFromSnapshot = false;  // ... of the positions saved in posGeom instead
    std::vector<int> startHost;
    cudaStream_t stream = nullptr;
    long long launches = 0;
    unsigned long long generation = 1;
    // every C ABI call on the model counts one; the max |F| a FIRE step
    // read back is returned by the next call if that call is
    // pcp_model_get_max_unbalanced_force (nothing ran in between)
    unsigned long long callSerial = 0;
    unsigned long long maxFSerial = 0;
    double maxFCached = 0.0;
    // stop rule of the device-resident loop (pcp_model_fire_set_stop_rule)
    double stopTol = 1e-15;
    int stopStagnant = -1;

    // device state
    double2 *pos = nullptr, *force = nullptr, *vel = nullptr;
    double2 *posTMP = nullptr, *posTMP2 = nullptr, *posTent = nullptr;
    double2* posGeom = nullptr;   // positions the pending geometry belongs to
    double2 *velSnap = nullptr, *forceSnap = nullptr;
    double *edgeLengths = nullptr, *constraints = nullptr, *scratch = nullptr;
    double *areas = nullptr, *comX = nullptr, *comY = nullptr, *perimeters = nullptr;
    double *targetAreas = nullptr, *targetEdge = nullptr;
    double *maxEdge = nullptr, *dtmp = nullptr, *xpbdDev = nullptr;
    int *start = nullptr, *shapeId = nullptr, *next = nullptr, *prev = nullptr;
    int *cellLocation = nullptr, *shakeIters = nullptr;
    int *mcCounter = nullptr, *mcNbIdx = nullptr, *mcBoxStarts = nullptr;
    unsigned long long* mcSum = nullptr;
    double* gradEnergy = nullptr;   // energy of pcp_model_overlap_energy_gradient
    int* gradBad = nullptr;
    Ctrl* ctrl = nullptr;
    Ctrl* ctrlHost = nullptr;   // pinned mirror
    ContactWS ws;

    // host views of the contact records
    enum View { VIEW_NONE, VIEW_COMPACT, VIEW_FINAL } view = VIEW_NONE;
    bool recordsCached = false;
    std::vector<unsigned long long> hKey, hOuter;   // records in the current view
    std::vector<float2> hTU, hUT;
    std::vector<uint32_t> hKeys;                    // permutation of the last sort
    bool neighborsCached = false;
    std::vector<int> hNeighbors, hNumNeighbors, hShapeCounts;
    std::vector<uint8_t> hInside;

    // FIRE graph (one step) and a graph of fireMultiSteps steps in a row
    cudaGraphExec_t fireExec = nullptr;
    cudaGraphExec_t fireExecMulti = nullptr;
    int fireMultiSteps = 0;
    unsigned long long fireGen = 0;
    int fireShakeIter = -1, fireModel = -1, fireB = -1;
    int fireKernelNodes = 0;   // kernel launches one FIRE step graph makes
    int rbBodyKernels = 0;     // kernels of its rollback body (counted on the device)
    cudaStream_t sideStream = nullptr, bodyStream = nullptr, preStream = nullptr;   // capture helpers
    cudaStream_t ifStream = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr, evPreFork = nullptr, evPreJoin = nullptr;
    cudaEvent_t evRbFork = nullptr, evRbJoin = nullptr;

    ~pcp_model() { release(); }

    void release() {
        if (fireExec) { cudaGraphExecDestroy(fireExec); fireExec = nullptr; }
        if (fireExecMulti) { cudaGraphExecDestroy(fireExecMulti); fireExecMulti = nullptr; }
        if (sideStream) { cudaStreamDestroy(sideStream); sideStream = nullptr; }
        if (bodyStream) { cudaStreamDestroy(bodyStream); bodyStream = nullptr; }
        if (evFork) { cudaEventDestroy(evFork); evFork = nullptr; }
        if (evJoin) { cudaEventDestroy(evJoin); evJoin = nullptr; }
        if (preStream) { cudaStreamDestroy(preStream); preStream = nullptr; }
        if (ifStream) { cudaStreamDestroy(ifStream); ifStream = nullptr; }
        if (evPreFork) { cudaEventDestroy(evPreFork); evPreFork = nullptr; }
        if (evPreJoin) { cudaEventDestroy(evPreJoin); evPreJoin = nullptr; }
        if (evRbFork) { cudaEventDestroy(evRbFork); evRbFork = nullptr; }
        if (evRbJoin) { cudaEventDestroy(evRbJoin); evRbJoin = nullptr; }
        dfree(&pos); dfree(&force); dfree(&vel); dfree(&posTMP); dfree(&posTMP2); dfree(&posTent);
        dfree(&posGeom);
        dfree(&velSnap); dfree(&forceSnap);
        dfree(&edgeLengths); dfree(&constraints); dfree(&scratch);
        dfree(&areas); dfree(&comX); dfree(&comY); dfree(&perimeters);
        dfree(&targetAreas); dfree(&targetEdge); dfree(&maxEdge); dfree(&dtmp); dfree(&xpbdDev);
        dfree(&start); dfree(&shapeId); dfree(&next); dfree(&prev); dfree(&cellLocation);
        dfree(&shakeIters); dfree(&mcCounter); dfree(&mcNbIdx); dfree(&mcBoxStarts); dfree(&mcSum);
        dfree(&gradEnergy); dfree(&gradBad);
        dfree(&ctrl);
        if (ctrlHost) { cudaFreeHost(ctrlHost); ctrlHost = nullptr; }
        free_ws();
    }
    void free_ws() {
        // stream-ordered, like their allocation (alloc_ws)
        cudaStream_t st = stream;
        dfree_async(&ws.edgeVec, st); dfree_async(&ws.vtx, st); dfree_async(&ws.polyInfo, st);
        dfree_async(&ws.polyBox, st); dfree_async(&ws.polyFlags, st);
        dfree_async(&ws.gridCount, st); dfree_async(&ws.gridStart, st);
        dfree_async(&ws.gridFill, st); dfree_async(&ws.sortedPoly, st);
        dfree_async(&ws.unsafeList, st); dfree_async(&ws.pairs, st); dfree_async(&ws.recKey, st);
        dfree_async(&ws.recOuter, st); dfree_async(&ws.recTU, st); dfree_async(&ws.recUT, st);
        dfree_async(&ws.fixList, st); dfree_async(&ws.slowList, st);
        dfree_async(&ws.maxCand, st); dfree_async(&ws.overList, st);
        if (st) cudaStreamSynchronize(st);
        else cudaDeviceSynchronize();
    }
    void invalidate() {
        recordsCached = false;
        neighborsCached = false;
    }
};

namespace {

int alloc_vertex(pcp_model* m) {
    size_t V = (size_t)m->V;
    CK(dalloc(&m->pos, V)); CK(dalloc(&m->force, V)); CK(dalloc(&m->vel, V));
    CK(dalloc(&m->posTMP, V)); CK(dalloc(&m->posTMP2, V)); CK(dalloc(&m->posTent, V));
    CK(dalloc(&m->posGeom, V));
    CK(dalloc(&m->velSnap, V)); CK(dalloc(&m->forceSnap, V));
    m->geometryStale = false;
    m->geomFromSnapshot = false;
    CK(dalloc(&m->edgeLengths, V)); CK(dalloc(&m->constraints, 6 * V));
    CK(dalloc(&m->scratch, (size_t)kScratchPerVertex * V));
    m->generation++;
    m->topology = false;
    return PCP_OK;
}

int alloc_ws(pcp_model* m, int capPairs, int capRecords) {
    ContactWS& w = m->ws;
    w.V = m->V; w.P = m->P;
    w.capPairs = capPairs; w.capRecords = capRecords;
    w.capFix = std::max(1024, capRecords / 16);
    w.capSlow = std::max(1024, capPairs / 4);
    size_t V = (size_t)m->V, P = (size_t)std::max(m->P, 1);
    cudaStream_t st = m->stream;
    keep_pool_memory();
    CK(dalloc_async(&w.edgeVec, V, st)); CK(dalloc_async(&w.vtx, V, st));
    CK(dalloc_async(&w.polyInfo, P, st)); CK(dalloc_async(&w.polyBox, P, st)); CK(dalloc_async(&w.polyFlags, P, st));
    CK(dalloc_async(&w.gridCount, (size_t)kGridMax * kGridMax, st));
    CK(dalloc_async(&w.gridStart, (size_t)kGridMax * kGridMax + 1, st));
    CK(dalloc_async(&w.gridFill, (size_t)kGridMax * kGridMax, st));
    CK(dalloc_async(&w.sortedPoly, P, st)); CK(dalloc_async(&w.unsafeList, P, st));
    CK(dalloc_async(&w.pairs, (size_t)capPairs, st));
    CK(dalloc_async(&w.recKey, (size_t)capRecords, st)); CK(dalloc_async(&w.recOuter, (size_t)capRecords, st));
    CK(dalloc_async(&w.recTU, (size_t)capRecords, st)); CK(dalloc_async(&w.recUT, (size_t)capRecords, st));
    CK(dalloc_async(&w.fixList, (size_t)w.capFix, st)); CK(dalloc_async(&w.slowList, (size_t)w.capSlow, st));
    if (!w.maxCand) CK(dalloc_async(&w.maxCand, (size_t)kMaxCand, st));
    CK(dalloc_async(&w.overList, (size_t)capPairs, st));
    m->generation++;
    return PCP_OK;
}

int sync(pcp_model* m) {
    CK(cudaStreamSynchronize(m->stream));
    return PCP_OK;
}

int read_ctrl(pcp_model* m) {
    CK(cudaMemcpyAsync(m->ctrlHost, m->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, m->stream));
    return sync(m);
}

int need_topology(pcp_model* m) {
    if (m->P <= 0 || m->startHost.empty())
        return fail(PCP_ERR_STATE, "setStartIndices has not been called");
    if (!m->topology) return fail(PCP_ERR_STATE, "initializeNeighborCells has not been called");
    return PCP_OK;
}

// contact search with the reference's resize-and-retry (model.cpp:256-307):
// capacities grow until the search fits, so no crossing is ever dropped
int run_contacts(pcp_model* m) {
    for (int attempt = 0; attempt < 8; ++attempt) {
        CK(launch_contacts(m->pos, m->start, m->shapeId, m->cellLocation, m->P, m->V, m->boxSize,
                           m->ws, m->ctrl, nullptr, m->stream));
        m->launches += 10;
        int rc = read_ctrl(m);
        if (rc) return rc;
        unsigned fl = m->ctrlHost->flags;
        if (fl & kFlagCapacity)
            return fail(PCP_ERR_CAPACITY,
                        "a polygon pair exceeds the contact kernel limits (%d vertices, %d "
                        "crossings per pair)", kSlowRing, kSlowRecords);
        if (!(fl & (kFlagPairOverflow | kFlagRecordOverflow | kFlagSlowOverflow |
                    kFlagFixOverflow)))
            return PCP_OK;
        int np = std::max(m->ws.capPairs, m->ctrlHost->numPairs) * 2 + 1024;
        int nr = std::max(m->ws.capRecords, m->ctrlHost->numRecords) * 2 + 4096;
        int rc2 = alloc_ws(m, np, nr);
        if (rc2) return rc2;
    }
    return fail(PCP_ERR_CAPACITY, "contact buffers could not be sized");
}

// ---- host views of the records ----------------------------------------

int fetch_records(pcp_model* m, std::vector<unsigned long long>& key,
                  std::vector<unsigned long long>& outer, std::vector<float2>& tu,
                  std::vector<float2>& ut) {
    int rc = read_ctrl(m);
    if (rc) return rc;
    int I = std::min(m->ctrlHost->numRecords, m->ws.capRecords);
    key.resize(I); outer.resize(I); tu.resize(I); ut.resize(I);
    if (I > 0) {
        CK(cudaMemcpy(key.data(), m->ws.recKey, I * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(outer.data(), m->ws.recOuter, I * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(tu.data(), m->ws.recTU, I * sizeof(float2), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(ut.data(), m->ws.recUT, I * sizeof(float2), cudaMemcpyDeviceToHost));
    }
    return PCP_OK;
}

// lower (id1) and higher (nid) vertex of a record and its inside flag
// (inverse of the packing at kernels.cuh:861-874)
inline void record_vertices(const std::vector<int>& st, unsigned long long key, int& id1,
                            int& nid, bool& inside) {
    int sj = (int)(key >> 48), si = (int)((key >> 32) & 0xFFFF);
    int i = (int)((key >> 16) & 0xFFFF), j = (int)(key & 0xFFFF);
    inside = (sj < si) || (sj == si && j < i);
    if (inside) { id1 = st[sj] + j; nid = st[si] + i; }
    else { id1 = st[si] + i; nid = st[sj] + j; }
}

// rank of cell c2 in the 3x3 scan order of updateNeighborsKernel around c1
// (kernels.cuh:737-757): dx outer, dy inner, repeated cells skipped
int visit_rank(int c1, int c2, int B) {
    int bx = c1 % B, by = c1 / B;
    int seen[9], ns = 0;
    for (int dx = -1; dx <= 1; dx++) {
        int nx = bx + dx;
        if (nx < 0) nx += B; else if (nx >= B) nx -= B;
        for (int dy = -1; dy <= 1; dy++) {
            int ny = by + dy;
            if (ny < 0) ny += B; else if (ny >= B) ny -= B;
            int nb = ny * B + nx;
            bool dup = false;
            for (int t = 0; t < ns; t++) dup |= seen[t] == nb;
            if (dup) continue;
            seen[ns++] = nb;
            if (nb == c2) return ns - 1;
        }
    }
    return 9;
}

// Records in the compaction order of the reference (by id1, then slot):
// slots fill in cell-scan order, and inside a cell by vertex id.
int build_compact(pcp_model* m, std::vector<size_t>& order,
                  const std::vector<unsigned long long>& key, std::vector<int>& id1s,
                  std::vector<int>& nids, std::vector<uint8_t>& ins) {
    size_t I = key.size();
    std::vector<int> cells(m->V);
    if (m->V > 0)
        CK(cudaMemcpy(cells.data(), m->cellLocation, m->V * sizeof(int), cudaMemcpyDeviceToHost));
    id1s.resize(I); nids.resize(I); ins.resize(I);
    std::vector<long long> sortKey(I);
    int B = std::max(1, m->boxSize);
    for (size_t r = 0; r < I; ++r) {
        int a, b; bool in;
        record_vertices(m->startHost, key[r], a, b, in);
        id1s[r] = a; nids[r] = b; ins[r] = in ? 1 : 0;
        int rank = (a < m->V && b < m->V) ? visit_rank(cells[a], cells[b], B) : 9;
        sortKey[r] = ((long long)a << 36) | ((long long)rank << 32) | (long long)(unsigned)b;
    }
    order.resize(I);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return sortKey[x] < sortKey[y]; });
    return PCP_OK;
}

// Canonical final order (model.cpp:354-360): keys sorted, then stably by the
// low 48 bits, i.e. ascending (si, i, j) with ties in ascending sj.
void final_order(const std::vector<unsigned long long>& key, std::vector<size_t>& order) {
    order.resize(key.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        unsigned long long la = key[a] & 0xFFFFFFFFFFFFull, lb = key[b] & 0xFFFFFFFFFFFFull;
        if (la != lb) return la < lb;
        return key[a] < key[b];
    });
}

int ensure_records(pcp_model* m) {
    if (m->recordsCached) return PCP_OK;
    std::vector<unsigned long long> key, outer;
    std::vector<float2> tu, ut;
    int rc = fetch_records(m, key, outer, tu, ut);
    if (rc) return rc;
    std::vector<size_t> order;
    if (m->view == pcp_model::VIEW_COMPACT) {
        std::vector<int> a, b;
        std::vector<uint8_t> in;
        rc = build_compact(m, order, key, a, b, in);
        if (rc) return rc;
    } else {
        final_order(key, order);
    }
    size_t I = key.size();
    m->hKey.resize(I); m->hOuter.resize(I); m->hTU.resize(I); m->hUT.resize(I);
    for (size_t r = 0; r < I; ++r) {
        m->hKey[r] = key[order[r]];
        m->hOuter[r] = outer[order[r]];
        m->hTU[r] = tu[order[r]];
        m->hUT[r] = ut[order[r]];
    }
    // permutation of the reference's last sort (bits [0,48) over the 64-bit order)
    std::vector<size_t> o64(I);
    std::iota(o64.begin(), o64.end(), 0);
    std::sort(o64.begin(), o64.end(), [&](size_t a, size_t b) { return key[a] < key[b]; });
    std::vector<uint32_t> perm(I);
    std::iota(perm.begin(), perm.end(), 0u);
    std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) {
        return (key[o64[a]] & 0xFFFFFFFFFFFFull) < (key[o64[b]] & 0xFFFFFFFFFFFFull);
    });
    m->hKeys = perm;
    m->recordsCached = true;
    return PCP_OK;
}

// per-vertex slot arrays of updateNeighborsKernel (kernels.cuh:792-811)
int ensure_neighbors(pcp_model* m) {
    if (m->neighborsCached) return PCP_OK;
    std::vector<unsigned long long> key, outer;
    std::vector<float2> tu, ut;
    int rc = fetch_records(m, key, outer, tu, ut);
    if (rc) return rc;
    std::vector<size_t> order;
    std::vector<int> a, b;
    std::vector<uint8_t> in;
    rc = build_compact(m, order, key, a, b, in);
    if (rc) return rc;
    std::vector<int> count(m->V, 0);
    for (size_t r = 0; r < key.size(); ++r) if (a[r] < m->V) count[a[r]]++;
    int need = 0;
    for (int c : count) need = std::max(need, c);
    if (need > m->maxNeighbors) {
        fprintf(stderr, "Warning: neighbor buffer overflow: maxNeighbors=%d required=%d. "
                        "Resizing and retrying.\n", m->maxNeighbors, need);
        m->maxNeighbors = std::max(m->maxNeighbors * 2 + 1, need);
    }
    int M = m->maxNeighbors;
    m->hNeighbors.assign((size_t)m->V * M, 0);
    m->hInside.assign((size_t)m->V * M, 0);
    m->hNumNeighbors.assign(m->V, 0);
    m->hShapeCounts.assign(m->P, 0);
    for (size_t t = 0; t < order.size(); ++t) {
        size_t r = order[t];
        int v = a[r];
        if (v >= m->V) continue;
        int s = m->hNumNeighbors[v]++;
        if (s < M) {
            m->hNeighbors[(size_t)v * M + s] = b[r];
            m->hInside[(size_t)v * M + s] = in[r];
        }
        int si = (int)((key[r] >> 32) & 0xFFFF);
        if (si < m->P) m->hShapeCounts[si]++;
    }
    m->neighborsCached = true;
    return PCP_OK;
}

template <typename T>
int copy_out(const T* src, int n, T* out, int cap, int* len_out) {
    if (len_out) *len_out = n;
    if (!out) return PCP_OK;
    if (cap < n) return fail(PCP_ERR_ARG, "output buffer holds %d elements, %d needed", cap, n);
    if (n > 0) memcpy(out, src, (size_t)n * sizeof(T));
    return PCP_OK;
}

template <typename T>
int copy_dev_out(pcp_model* m, const T* dsrc, int n, T* out, int cap, int* len_out) {
    if (len_out) *len_out = n;
    if (!out) return PCP_OK;
    if (cap < n) return fail(PCP_ERR_ARG, "output buffer holds %d elements, %d needed", cap, n);
    // ordered after the model's stream work; one wait for both
    if (n > 0) CK(cudaMemcpyAsync(out, dsrc, (size_t)n * sizeof(T), cudaMemcpyDeviceToHost, m->stream));
    return sync(m);
}

int upload(pcp_model* m, void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return PCP_OK;
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, m->stream));
    return sync(m);
}

// ---- the force evaluation (Model::updateForceEnergy, model.cpp:363-395) ----
// edgeVec: the edge vectors of the current positions when they are at hand
// decide: the FIRE step's force pass, whose last block decides the energy
// rollback and sets rbCond
int force_energy(pcp_model* m, const int* gate, bool zeroed = false,
                 const double2* edgeVec = nullptr, int decide = 0,
                 cudaGraphConditionalHandle rbCond = 0) {
    if (!zeroed) {
        CK(launch_zero_force(m->force, m->V, m->ctrl, gate, m->stream));
        m->launches++;
    }
    int t = m->modelType;
    bool overlap = (t == PCP_MODEL_NORMAL || t == PCP_MODEL_HYBRID);
    bool edge = (t == PCP_MODEL_SOFT_BODY || t == PCP_MODEL_EDGE_ONLY || t == PCP_MODEL_HYBRID);
    bool area = (t == PCP_MODEL_SOFT_BODY || t == PCP_MODEL_AREA_ONLY || t == PCP_MODEL_HYBRID);
    if (overlap) {
        CK(launch_overlap_force(m->pos, m->start, m->V, m->ws, m->ctrl, m->force, gate,
                                m->stream, edgeVec, decide, rbCond));
        m->launches++;
    }
    if (edge) {
        CK(launch_soft_edge(m->pos, m->targetEdge, m->edgeLengths, m->next, m->prev, m->shapeId,
                            m->V, m->stiffness, reinterpret_cast<double*>(m->force),
                            &m->ctrl->energy, gate, m->stream));
        m->launches++;
    }
    if (area) {
        CK(launch_soft_area(m->pos, m->shapeId, m->next, m->prev, m->areas, m->targetAreas,
                            m->start, m->V, m->compressibility, reinterpret_cast<double*>(m->force),
                            &m->ctrl->energy, gate, m->stream));
        m->launches++;
    }
    return PCP_OK;
}

int geometry(pcp_model* m, const int* gate, const double2* src = nullptr) {
    CK(launch_geometry(src ? src : m->pos, m->start, m->P, m->V, m->edgeLengths, m->areas,
                       m->comX, m->comY,
                       m->perimeters, m->constraints, m->maxEdge, gate, m->stream));
    m->launches += 2;
    return PCP_OK;
}

// Materialise geometry the FIRE graph deferred (it corresponds to the
// positions the last FIRE step ended with, as in the reference).
int ensure_geometry(pcp_model* m) {
    if (!m->geometryStale) return PCP_OK;
    m->geometryStale = false;
    bool snap = m->geomFromSnapshot;
    m->geomFromSnapshot = false;
    return geometry(m, nullptr, snap ? m->posGeom : nullptr);
}

// The positions are about to change while their geometry is still pending:
// keep a copy of them (a device-to-device copy instead of the geometry pass)
// so the getters later see the geometry the reference computed at that point.
int snapshot_geometry(pcp_model* m) {
    if (!m->geometryStale || m->geomFromSnapshot) return PCP_OK;
    CK(cudaMemcpyAsync(m->posGeom, m->pos, (size_t)m->V * sizeof(double2),
                       cudaMemcpyDeviceToDevice, m->stream));
    m->geomFromSnapshot = true;
    return PCP_OK;
}

// ---- FIRE step graph ------------------------------------------------------
// Adds an IF node with condition `h` after the work captured so far on `st`
// and starts capturing its body on `body`.
int begin_if(cudaStream_t st, cudaGraphConditionalHandle h, cudaStream_t body) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edges, &nd));
    if (cs != cudaStreamCaptureStatusActive) return fail(PCP_ERR_CUDA, "stream is not capturing");
    cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, deps, edges, nd, &p));
    CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                           cudaStreamSetCaptureDependencies));
    CK(cudaStreamBeginCaptureToGraph(body, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                     cudaStreamCaptureModeThreadLocal));
    return PCP_OK;
}

int count_kernel_nodes(cudaGraph_t g) {
    size_t nn = 0;
    if (cudaGraphGetNodes(g, nullptr, &nn) != cudaSuccess) return 0;
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
    int k = 0;
    for (size_t i = 0; i < nn; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

// One FIRE step (Model::minimizeFIREStep, model.cpp:405-486) recorded on the
// capturing stream m->stream.  Graph layout (normal model with SHAKE):
//
//   begin --+-- SHAKE (+ v) -- [IF retry: SHAKE x10 (+ v), outcome] --+-- force --
//           +-- contact search on the pre-SHAKE copy ------------------+
//   -- projection (decides the rollback) -- [IF rollback: restore, contact
//   search, force, projection] -- bend + scalar bookkeeping
//
// The contact search reads the positions the reference searches (after the
// Verlet move, before SHAKE) from their copy, so it runs beside SHAKE.  The
// two IF bodies run only when a kernel of the step sets their condition.
int record_fire_step(pcp_model* m, cudaGraphConditionalHandle retryCond,
                     cudaGraphConditionalHandle rbCond) {
    const int* gA = &m->ctrl->active;
    cudaStream_t st = m->stream;
    bool needsI = (m->modelType == PCP_MODEL_NORMAL || m->modelType == PCP_MODEL_HYBRID);
    bool rigid = (m->modelType == PCP_MODEL_NORMAL);
    bool shake = rigid && m->fireShakeIter > 0;
    int V = m->V;
    const int noReset = 3 | kContactsNoReset;
    double2* pre = reinterpret_cast<double2*>(m->scratch);
    if (needsI) {
        // the step start fused with the contact prepass: x, v, F moved in
        // place, the moved positions copied to posTMP (read by the search)
        FireMove mv = {m->pos, m->vel, m->force, m->posTMP2, m->velSnap, m->forceSnap, m->ctrl};
        CK(launch_prepass_move(shake ? m->posTMP : m->pos, m->start, m->cellLocation, m->P,
                               m->boxSize, m->ws, m->ctrl, gA, st, mv));
    } else {
        CK(launch_fire_begin(m->pos, m->vel, m->force, m->posTMP2, m->velSnap, m->forceSnap,
                             nullptr, V, 0, m->ctrl, gA, st));
    }
    if (shake) {
        CK(cudaEventRecord(m->evFork, st));
        CK(cudaStreamWaitEvent(m->sideStream, m->evFork, 0));
        CK(launch_contacts(m->posTMP, m->start, m->shapeId, m->cellLocation, m->P, V,
                           m->boxSize, m->ws, m->ctrl, gA, m->sideStream,
                           noReset | kContactsNoPrepass, m->cellLocation));
        CK(cudaEventRecord(m->evJoin, m->sideStream));
        // SHAKE rederives v from its displacement itself (model.cpp:436-438)
        CK(launch_shake(m->pos, m->start, m->P, m->nmax, m->targetEdge, m->targetAreas,
                        m->fireShakeIter, 1e-15, &m->ctrl->shakeIters1, m->scratch, V, gA, st,
                        m->ctrl, retryCond, m->vel, m->ctrl));
        int rc = begin_if(st, retryCond, m->bodyStream);
        if (rc) return rc;
        CK(launch_shake(m->pos, m->start, m->P, m->nmax, m->targetEdge, m->targetAreas,
                        m->fireShakeIter * 10, 1e-15, &m->ctrl->shakeIters2, m->scratch, V,
                        nullptr, m->bodyStream, nullptr, 0, m->vel, m->ctrl));
        CK(launch_fire_retry_outcome(m->pos, m->vel, m->posTMP2, V, m->ctrl, m->bodyStream));
        cudaGraph_t body = nullptr;
        CK(cudaStreamEndCapture(m->bodyStream, &body));
        // the projection's tangents and area gradients of the final
        // positions (restored ones after a failed SHAKE), on a third branch
        // beside the end of the contact search and the force
        CK(cudaEventRecord(m->evPreFork, st));
        CK(cudaStreamWaitEvent(m->preStream, m->evPreFork, 0));
        CK(launch_project_pre(m->pos, m->start, m->P, m->nmax, pre, V, gA, m->preStream));
        CK(cudaEventRecord(m->evPreJoin, m->preStream));
        CK(cudaStreamWaitEvent(st, m->evJoin, 0));
    } else if (needsI) {
        CK(launch_contacts(m->pos, m->start, m->shapeId, m->cellLocation, m->P, V, m->boxSize,
                           m->ws, m->ctrl, gA, st, noReset | kContactsNoPrepass,
                           m->cellLocation));
    }
    // The normal model reads nothing of the geometry inside the step (the
    // projection takes the area gradient from the positions), so the
    // geometry of the final positions is computed when a getter asks for it.
    int rc = PCP_OK;
    if (!rigid) {
        rc = geometry(m, gA);
        if (rc) return rc;
    }
    // the third branch's edge vectors (computed with the tangents) feed the
    // force when the projection takes the one-vertex-per-lane path
    const bool preEdges = shake && project_uses_lanes(m->P, m->nmax);
    if (shake) CK(cudaStreamWaitEvent(st, m->evPreJoin, 0));
    // (the rigid model's force pass decides the energy rollback itself)
    rc = force_energy(m, gA, true, preEdges ? pre + 2 * (size_t)V : nullptr, rigid ? 1 : 0,
                      rbCond);
    if (rc) return rc;
    cudaStream_t ifSt = st;
    if (rigid) {
        // the rollback's IF node beside the projection, which does nothing
        // when the body runs
        CK(cudaEventRecord(m->evRbFork, st));
        CK(cudaStreamWaitEvent(m->ifStream, m->evRbFork, 0));
        ifSt = m->ifStream;
    } else {
        CK(launch_fire_velocity(m->vel, m->force, V, m->ctrl, rbCond, 1, gA, st));
    }
    // energy-increase rollback (model.cpp:450-470) as the body of an IF node
    rc = begin_if(ifSt, rbCond, m->bodyStream);
    if (rc) return rc;
    m->stream = m->bodyStream;
    CK(launch_fire_rollback(m->pos, m->vel, m->force, m->posTMP2, V, needsI ? 1 : 0, m->ctrl,
                            m->stream));
    if (!rigid) rc = geometry(m, nullptr);
    if (!rc && needsI) {
        cudaError_t e = launch_contacts(m->pos, m->start, m->shapeId, m->cellLocation, m->P, V,
                                        m->boxSize, m->ws, m->ctrl, nullptr, m->stream, noReset,
                                        m->cellLocation);
        if (e != cudaSuccess) rc = fail(PCP_ERR_CUDA, "rollback capture: %s", cudaGetErrorString(e));
    }
    if (!rc) rc = force_energy(m, nullptr, true);
    if (!rc) {
        cudaError_t e = rigid
            ? launch_project(m->pos, m->start, m->P, m->nmax, m->constraints, m->force, m->scratch,
                             V, 1, m->ctrl, nullptr, m->vel, m->stream)
            : launch_fire_maxf(m->force, V, m->ctrl, nullptr, m->stream);
        if (e != cudaSuccess) rc = fail(PCP_ERR_CUDA, "rollback capture: %s", cudaGetErrorString(e));
    }
    m->stream = st;
    cudaGraph_t body = nullptr;
    cudaError_t e = cudaStreamEndCapture(m->bodyStream, &body);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(PCP_ERR_CUDA, "rollback capture: %s", cudaGetErrorString(e));
    m->rbBodyKernels = count_kernel_nodes(body);
    if (rigid) {
        CK(cudaEventRecord(m->evRbJoin, m->ifStream));
        CK(launch_project(m->pos, m->start, m->P, m->nmax, m->constraints, m->force, m->scratch, V, 1,
                          m->ctrl, gA, m->vel, st, 1, shake ? pre : nullptr));
        CK(cudaStreamWaitEvent(st, m->evRbJoin, 0));
    }
    // the step's scalar bookkeeping ran in the last block of the force pass
    // (or of the rollback body's pass); the velocity bend waits for the next
    // step's start kernel (or for a read of the velocities)
    return PCP_OK;
}

// Capture nSteps consecutive FIRE steps into one executable graph (each
// step with its own conditional handles); kernelNodes receives the kernel
// launches of one step.
int capture_fire_graph(pcp_model* m, int nSteps, cudaGraphExec_t* exec, int* kernelNodes) {
    const int shakeIter = m->fireShakeIter;
    if (!m->sideStream) CK(cudaStreamCreateWithFlags(&m->sideStream, cudaStreamNonBlocking));
    if (!m->bodyStream) CK(cudaStreamCreateWithFlags(&m->bodyStream, cudaStreamNonBlocking));
    if (!m->evFork) CK(cudaEventCreateWithFlags(&m->evFork, cudaEventDisableTiming));
    if (!m->evJoin) CK(cudaEventCreateWithFlags(&m->evJoin, cudaEventDisableTiming));
    if (!m->preStream) CK(cudaStreamCreateWithFlags(&m->preStream, cudaStreamNonBlocking));
    if (!m->evPreFork) CK(cudaEventCreateWithFlags(&m->evPreFork, cudaEventDisableTiming));
    if (!m->evPreJoin) CK(cudaEventCreateWithFlags(&m->evPreJoin, cudaEventDisableTiming));
    if (!m->ifStream) CK(cudaStreamCreateWithFlags(&m->ifStream, cudaStreamNonBlocking));
    if (!m->evRbFork) CK(cudaEventCreateWithFlags(&m->evRbFork, cudaEventDisableTiming));
    if (!m->evRbJoin) CK(cudaEventCreateWithFlags(&m->evRbJoin, cudaEventDisableTiming));
    cudaStream_t cap = nullptr;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaStream_t saved = m->stream;
    long long savedLaunches = m->launches;   // captured launches are not launches
    m->stream = cap;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    int rc = PCP_OK;
    if (e == cudaSuccess) {
        // the conditions are created on the graph being captured; they read
        // 0 at every launch of it until a kernel of the step sets them.  The
        // SHAKE retry exists only for the normal model with SHAKE (a handle
        // that no conditional node uses makes the instantiation fail).
        cudaStreamCaptureStatus cs;
        cudaGraph_t cg = nullptr;
        const bool retry = m->modelType == PCP_MODEL_NORMAL && shakeIter > 0;
        e = cudaStreamGetCaptureInfo(cap, &cs, nullptr, &cg);
        for (int step = 0; step < nSteps && e == cudaSuccess && rc == PCP_OK; ++step) {
            cudaGraphConditionalHandle retryCond = 0, rbCond = 0;
            if (e == cudaSuccess && retry)
                e = cudaGraphConditionalHandleCreate(&retryCond, cg, 0, cudaGraphCondAssignDefault);
            if (e == cudaSuccess)
                e = cudaGraphConditionalHandleCreate(&rbCond, cg, 0, cudaGraphCondAssignDefault);
            if (e == cudaSuccess) rc = record_fire_step(m, retryCond, rbCond);
        }
        cudaError_t e2 = cudaStreamEndCapture(cap, &g);
        if (e == cudaSuccess) e = e2;
    }
    m->stream = saved;
    m->launches = savedLaunches;
    cudaStreamDestroy(cap);
    if (rc) { if (g) cudaGraphDestroy(g); (void)cudaGetLastError(); return rc; }
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();    // not left for the next launcher's check
        return fail(PCP_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    }
    *kernelNodes = count_kernel_nodes(g) / std::max(nSteps, 1);
    e = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();    // not left for the next launcher's check
        return fail(PCP_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    }
    // the rollback kernel counts its body's launches from the control block
    m->ctrlHost->rbBodyKernels = m->rbBodyKernels;
    CK(cudaMemcpyAsync(&m->ctrl->rbBodyKernels, &m->ctrlHost->rbBodyKernels, sizeof(int),
                       cudaMemcpyHostToDevice, m->stream));
    return sync(m);
}

int build_fire_graph(pcp_model* m, int shakeIter) {
    if (m->fireExec && m->fireGen == m->generation && m->fireShakeIter == shakeIter &&
        m->fireModel == m->modelType && m->fireB == m->boxSize)
        return PCP_OK;
    if (m->fireExec) { cudaGraphExecDestroy(m->fireExec); m->fireExec = nullptr; }
    if (m->fireExecMulti) { cudaGraphExecDestroy(m->fireExecMulti); m->fireExecMulti = nullptr; }
    m->fireShakeIter = shakeIter;
    int rc = capture_fire_graph(m, 1, &m->fireExec, &m->fireKernelNodes);
    if (rc) return rc;
    m->fireGen = m->generation;
    m->fireModel = m->modelType;
    m->fireB = m->boxSize;
    return PCP_OK;
}

// The step graph and a graph of nSteps steps in a row (one launch for a
// chunk of steps), both for the current parameters.
int build_fire_graph_multi(pcp_model* m, int shakeIter, int nSteps) {
    int rc = build_fire_graph(m, shakeIter);
    if (rc) return rc;
    if (m->fireExecMulti && m->fireMultiSteps == nSteps) return PCP_OK;
    if (m->fireExecMulti) { cudaGraphExecDestroy(m->fireExecMulti); m->fireExecMulti = nullptr; }
    int nodes = 0;
    rc = capture_fire_graph(m, nSteps, &m->fireExecMulti, &nodes);
    if (rc) return rc;
    m->fireMultiSteps = nSteps;
    return PCP_OK;
}

struct FireParams {
    double dt, alpha, dtMax, alphaStart, fAlpha, fInc, fDec, threshold;
    int nPos, nMin, shakeIter, stepLimit;
    double stagnantTol = 0.0;
    int stagnantLimit = -1;     // the Python driver's stop rule (< 0: off)
};

// write the step parameters into the device control block (a one-thread
// kernel on the model's stream: no host round trip)
int set_fire_params(pcp_model* m, const FireParams& f, bool resetRun) {
    FireScalars d{f.dt, f.alpha, f.dtMax, f.alphaStart, f.fAlpha, f.fInc, f.fDec, f.threshold,
                  f.nPos, f.nMin, f.shakeIter, f.stepLimit, resetRun ? 1 : 0, m->rbBodyKernels,
                  f.stagnantTol, f.stagnantLimit};
    CK(launch_set_fire_params(m->ctrl, d, m->stream));
    m->launches++;
    return PCP_OK;
}

// A contact buffer overflowed inside a FIRE step: the step stopped itself
// (k_fire_scalars clears `active`).  Grow the buffers, put back the state
// the step started from and let the caller run it again.
int recover_fire(pcp_model* m, bool& redo) {
    redo = false;
    Ctrl c = *m->ctrlHost;
    if (c.flags & kFlagCapacity)
        return fail(PCP_ERR_CAPACITY, "a polygon pair exceeds the contact kernel limits");
    if (!c.needsRecovery) return PCP_OK;
    redo = true;
    int np = std::max(m->ws.capPairs, c.numPairs) * 2 + 1024;
    int nr = std::max(m->ws.capRecords, c.numRecords) * 2 + 4096;
    int rc = alloc_ws(m, np, nr);
    if (rc) return rc;
    size_t b = (size_t)m->V * sizeof(double2);
    CK(cudaMemcpyAsync(m->pos, m->posTMP2, b, cudaMemcpyDeviceToDevice, m->stream));
    CK(cudaMemcpyAsync(m->vel, m->velSnap, b, cudaMemcpyDeviceToDevice, m->stream));
    CK(cudaMemcpyAsync(m->force, m->forceSnap, b, cudaMemcpyDeviceToDevice, m->stream));
    c.energy = c.ePre;
    c.dt = c.snapDt; c.alpha = c.snapAlpha; c.nPos = c.snapNPos;
    c.flags = 0; c.needsRecovery = 0; c.active = 1;
    c.Rmax = 0.f;            // the step's fused start accumulates it afresh
    *m->ctrlHost = c;
    CK(cudaMemcpyAsync(m->ctrl, m->ctrlHost, sizeof(Ctrl), cudaMemcpyHostToDevice, m->stream));
    rc = sync(m);
    if (rc) return rc;
    return build_fire_graph(m, m->fireShakeIter);
}

int fire_step_once(pcp_model* m, const FireParams& fp, double out[4]) {
    int rc = build_fire_graph(m, fp.shakeIter);
    if (rc) return rc;
    rc = set_fire_params(m, fp, true);
    if (rc) return rc;
    for (int attempt = 0; attempt < 6; ++attempt) {
        CK(cudaGraphLaunch(m->fireExec, m->stream));
        m->launches += m->fireKernelNodes;
        rc = read_ctrl(m);
        if (rc) return rc;
        bool redo = false;
        rc = recover_fire(m, redo);
        if (rc) return rc;
        if (!redo) {
            const Ctrl& c = *m->ctrlHost;
            out[0] = c.outE; out[1] = c.dt; out[2] = c.alpha; out[3] = c.nPos;
            m->maxFCached = c.maxF;
            m->maxFSerial = m->callSerial;
            m->lastShakeIters = c.shakeLast;
            m->numIntersections = c.numRecords;
            m->view = pcp_model::VIEW_FINAL;
            m->invalidate();
            if (m->modelType == PCP_MODEL_NORMAL) {
                m->geometryStale = true;
                m->geomFromSnapshot = false;
            }
            return PCP_OK;
        }
    }
    return fail(PCP_ERR_CAPACITY, "FIRE step: contact buffers could not be sized");
}

}  // namespace

// =========================================================================
// C ABI
// =========================================================================
extern "C" {

const char* pcp_last_error(void) { return g_err.c_str(); }
const char* pcp_version(void) { return "pcp_gb300 0.1 (sm_103a)"; }

#define CHECK_M(m) do { if (!(m)) return fail(PCP_ERR_ARG, "null model"); ++(m)->callSerial; } while (0)
// a model call with one scalar output
#define CHECK_MO(m, o) do { CHECK_M(m); if (!(o)) return fail(PCP_ERR_ARG, "null output"); } while (0)

int pcp_model_create(int size, pcp_model** out) {
    if (!out) return fail(PCP_ERR_ARG, "null output");
    *out = nullptr;
    if (size < 0) return fail(PCP_ERR_ARG, "negative size");
    CK(cudaFree(0));
    pcp_model* m = new pcp_model();
    m->V = size;
    int rc = alloc_vertex(m);
    if (!rc) {
        cudaError_t e = dalloc(&m->ctrl, 1);
        if (e == cudaSuccess) e = cudaMallocHost((void**)&m->ctrlHost, sizeof(Ctrl));
        if (e == cudaSuccess) memset(m->ctrlHost, 0, sizeof(Ctrl));
        if (e == cudaSuccess) e = dalloc(&m->maxEdge, 1);
        if (e == cudaSuccess) e = dalloc(&m->dtmp, 1);
        if (e == cudaSuccess) e = dalloc(&m->shakeIters, 1);
        if (e == cudaSuccess) e = dalloc(&m->mcSum, 1);
        if (e != cudaSuccess) rc = fail(PCP_ERR_CUDA, "allocation failed: %s", cudaGetErrorString(e));
    }
    if (!rc) {
        cudaError_t e = contacts_init();
        if (e == cudaSuccess) e = constraints_init();
        if (e != cudaSuccess) rc = fail(PCP_ERR_CUDA, "kernel setup failed: %s", cudaGetErrorString(e));
    }
    if (rc) { delete m; return rc; }
    sm_count();
    *out = m;
    return PCP_OK;
}

int pcp_model_destroy(pcp_model* m) {
    if (!m) return PCP_OK;
    if (m->stream) cudaStreamSynchronize(m->stream);
    else cudaDeviceSynchronize();
    delete m;
    return PCP_OK;
}

int pcp_model_set_stream(pcp_model* m, void* s) {
    CHECK_M(m);
    m->stream = (cudaStream_t)s;
    return PCP_OK;
}

int pcp_model_set_num_vertices(pcp_model* m, int n) {
    CHECK_M(m);
    if (n < 0) return fail(PCP_ERR_ARG, "negative vertex count");
    int rc = sync(m);
    if (rc) return rc;
    m->V = n;
    m->invalidate();
    return alloc_vertex(m);
}

int pcp_model_set_positions(pcp_model* m, const double* host, int len) {
    if (m && m->geometryStale) { int grc = snapshot_geometry(m); if (grc) return grc; }
    CHECK_M(m);
    if (len != 2 * m->V) {
        printf("Update numVertices before setting the positions\n");   // model.cpp:524
        fflush(stdout);
        return fail(PCP_ERR_ARG, "positions hold %d values, 2*numVertices = %d", len, 2 * m->V);
    }
    return upload(m, m->pos, host, (size_t)len * sizeof(double));
}

int pcp_model_set_forces(pcp_model* m, const double* host, int len) {
    CHECK_M(m);
    if (len > 2 * m->V) len = 2 * m->V;
    return upload(m, m->force, host, (size_t)len * sizeof(double));
}

int pcp_model_set_start_indices(pcp_model* m, const int* host, int len) {
    CHECK_M(m);
    if (len < 1) return fail(PCP_ERR_ARG, "startIndices needs at least one entry");
    int P = len - 1;
    if (P > 65535) return fail(PCP_ERR_LIMIT, "%d polygons; the packed records hold 65535", P);
    for (int p = 0; p < P; ++p) {
        if (host[p + 1] < host[p]) return fail(PCP_ERR_ARG, "startIndices must not decrease");
        if (host[p + 1] - host[p] > 65535)
            return fail(PCP_ERR_LIMIT, "polygon %d has more than 65535 vertices", p);
    }
    if (host[0] < 0) return fail(PCP_ERR_ARG, "startIndices[0] < 0");
    int rc = sync(m);
    if (rc) return rc;
    m->P = P;
    m->startHost.assign(host, host + len);
    m->nmax = 0;
    for (int p = 0; p < P; ++p) m->nmax = std::max(m->nmax, host[p + 1] - host[p]);
    size_t Pn = (size_t)std::max(P, 1);
    CK(dalloc(&m->start, (size_t)len));
    CK(dalloc(&m->areas, Pn)); CK(dalloc(&m->comX, Pn)); CK(dalloc(&m->comY, Pn));
    CK(dalloc(&m->perimeters, Pn)); CK(dalloc(&m->targetAreas, Pn)); CK(dalloc(&m->targetEdge, Pn));
    CK(dalloc(&m->xpbdDev, 2 * Pn));
    CK(cudaMemcpy(m->start, host, (size_t)len * sizeof(int), cudaMemcpyHostToDevice));
    m->generation++;
    m->topology = false;
    m->invalidate();
    return PCP_OK;
}

int pcp_model_set_target_areas(pcp_model* m, const double* host, int len) {
    CHECK_M(m);
    if (len > m->P) len = m->P;
    return upload(m, m->targetAreas, host, (size_t)len * sizeof(double));
}

int pcp_model_set_target_edge_lengths(pcp_model* m, const double* host, int len) {
    CHECK_M(m);
    if (len > m->P) len = m->P;
    return upload(m, m->targetEdge, host, (size_t)len * sizeof(double));
}

int pcp_model_set_max_edge_length(pcp_model* m, double l) {
    CHECK_M(m);
    double b = std::floor(1.0 / l);
    if (!(b >= 1.0)) b = 1.0;
    if (b > 1e7) b = 1e7;   // boxSize*boxSize must stay an int
    m->boxSize = (int)b;
    m->maxEdgeLengthSet = l;
    // the reference copies the value into its device maxEdgeLength (model.cpp:515)
    CK(cudaMemcpy(m->maxEdge, &l, sizeof(double), cudaMemcpyHostToDevice));
    return PCP_OK;
}

int pcp_model_set_model_enum(pcp_model* m, int e) {
    CHECK_M(m);
    if (e < 0 || e > 5) return fail(PCP_ERR_ARG, "unknown model enum %d", e);
    m->modelType = e;
    return PCP_OK;
}

int pcp_model_set_stiffness(pcp_model* m, double k) { CHECK_M(m); m->stiffness = k; return PCP_OK; }
int pcp_model_set_compressibility(pcp_model* m, double c) { CHECK_M(m); m->compressibility = c; return PCP_OK; }
int pcp_model_get_stiffness(pcp_model* m, double* out) { CHECK_MO(m, out); *out = m->stiffness; return PCP_OK; }
int pcp_model_get_compressibility(pcp_model* m, double* out) { CHECK_MO(m, out); *out = m->compressibility; return PCP_OK; }

int pcp_model_initialize_neighbor_cells(pcp_model* m) {
    CHECK_M(m);
    if (m->P <= 0 || m->startHost.empty())
        return fail(PCP_ERR_STATE, "setStartIndices has not been called");
    if (m->startHost.back() > m->V)
        return fail(PCP_ERR_ARG, "startIndices end at %d but the model has %d vertices",
                    m->startHost.back(), m->V);
    int rc = sync(m);
    if (rc) return rc;
    size_t V = (size_t)m->V;
    CK(dalloc(&m->shapeId, V)); CK(dalloc(&m->next, V)); CK(dalloc(&m->prev, V));
    CK(dalloc(&m->cellLocation, V));
    int capPairs = 16 * m->P + 4096;
    int capRecords = 8 * m->V + 16384;
    rc = alloc_ws(m, capPairs, capRecords);
    if (rc) return rc;
    CK(launch_topology(m->start, m->P, m->V, m->shapeId, m->next, m->prev, m->stream));
    m->launches++;
    rc = sync(m);
    if (rc) return rc;
    m->topology = true;
    m->numIntersections = 0;
    m->view = pcp_model::VIEW_NONE;
    m->invalidate();
    // reset the record counters (launches counted on the device move to the
    // host count)
    rc = read_ctrl(m);
    if (rc) return rc;
    m->launches += (long long)m->ctrlHost->condLaunches;
    memset(m->ctrlHost, 0, sizeof(Ctrl));
    CK(cudaMemcpy(m->ctrl, m->ctrlHost, sizeof(Ctrl), cudaMemcpyHostToDevice));
    return PCP_OK;
}

int pcp_model_update_polygon_geometry(pcp_model* m) {
    if (m) { m->geometryStale = false; m->geomFromSnapshot = false; }
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    return geometry(m, nullptr);
}

int pcp_model_update_neighbor_cells(pcp_model* m) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    CK(launch_neighbor_cells(m->pos, m->start, m->shapeId, m->V, m->boxSize, m->cellLocation,
                             nullptr, m->stream));
    m->launches++;
    m->neighborsCached = false;
    return PCP_OK;
}

int pcp_model_update_neighbors(pcp_model* m) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    rc = run_contacts(m);
    m->view = pcp_model::VIEW_COMPACT;
    m->invalidate();
    return rc;
}

int pcp_model_update_valid_and_counts(pcp_model* m) {
    CHECK_M(m);
    int rc = read_ctrl(m);
    if (rc) return rc;
    m->numIntersections = m->ctrlHost->numRecords;
    return PCP_OK;
}

int pcp_model_update_compacted_intersections(pcp_model* m) {
    CHECK_M(m);
    int rc = read_ctrl(m);
    if (rc) return rc;
    m->numIntersections = m->ctrlHost->numRecords;
    m->view = pcp_model::VIEW_COMPACT;
    m->recordsCached = false;
    return PCP_OK;
}

int pcp_model_update_outersections(pcp_model* m) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    // (the narrow phase matched the partners, and k_fixup after it did the
    // empty-group fixup)
    rc = read_ctrl(m);
    if (rc) return rc;
    m->numIntersections = m->ctrlHost->numRecords;
    m->view = pcp_model::VIEW_FINAL;
    m->recordsCached = false;
    return PCP_OK;
}

int pcp_model_update_force_energy(pcp_model* m) {
    if (m && m->geometryStale) { int grc = ensure_geometry(m); if (grc) return grc; }
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    return force_energy(m, nullptr);
}

int pcp_model_project_force(pcp_model* m) {
    if (m && m->geometryStale) { int grc = ensure_geometry(m); if (grc) return grc; }
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    CK(launch_project(m->pos, m->start, m->P, m->nmax, m->constraints, m->force, m->scratch, m->V, 0,
                      nullptr,
                      nullptr, nullptr, m->stream));
    m->launches++;
    return PCP_OK;
}

int pcp_model_shake_project(pcp_model* m, int n_iter, double tol, int* iters_out) {
    if (m && m->geometryStale) { int grc = snapshot_geometry(m); if (grc) return grc; }
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    int it = 0;
    if (m->P > 0 && n_iter > 0) {
        CK(cudaMemsetAsync(m->shakeIters, 0, sizeof(int), m->stream));
        CK(launch_shake(m->pos, m->start, m->P, m->nmax, m->targetEdge, m->targetAreas, n_iter, tol,
                        m->shakeIters, m->scratch, m->V, nullptr, m->stream));
        m->launches++;
        CK(cudaMemcpyAsync(&it, m->shakeIters, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
        rc = sync(m);
        if (rc) return rc;
    }
    m->lastShakeIters = it;
    if (iters_out) *iters_out = it;
    return PCP_OK;
}

int pcp_model_xpbd_project(pcp_model* m, int n_iter, double tol, int* iters_out) {
    if (m && m->geometryStale) { int grc = snapshot_geometry(m); if (grc) return grc; }
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    int iter = 0;
    std::vector<double> dev(2 * (size_t)m->P);
    for (; iter < n_iter; ++iter) {
        CK(launch_xpbd_iteration(m->pos, m->start, m->P, m->targetEdge, m->targetAreas, m->xpbdDev,
                                 m->stream));
        m->launches++;
        if (tol > 0) {
            rc = sync(m);
            if (rc) return rc;
            CK(cudaMemcpy(dev.data(), m->xpbdDev, dev.size() * sizeof(double), cudaMemcpyDeviceToHost));
            double me = 0, ma = 0;
            for (int p = 0; p < m->P; ++p) { me = std::max(me, dev[2 * p]); ma = std::max(ma, dev[2 * p + 1]); }
            if (me < tol && ma < tol) break;
        }
    }
    rc = sync(m);
    if (iters_out) *iters_out = iter;
    return rc;
}

int pcp_model_update_positions(pcp_model* m, double dt) {
    if (m && m->geometryStale) { int grc = snapshot_geometry(m); if (grc) return grc; }
    CHECK_M(m);
    CK(launch_update_positions(reinterpret_cast<double*>(m->pos), reinterpret_cast<const double*>(m->force),
                               m->V, dt, m->stream));
    m->launches++;
    return PCP_OK;
}

int pcp_model_reset_velocities(pcp_model* m) {
    CHECK_M(m);
    CK(cudaMemsetAsync(m->vel, 0, (size_t)m->V * sizeof(double2), m->stream));
    CK(cudaMemsetAsync(&m->ctrl->bendMode, 0, sizeof(int), m->stream));   // nothing left to bend
    return PCP_OK;
}

int pcp_model_reset_areas(pcp_model* m) {
    if (m && m->geometryStale) { int grc = ensure_geometry(m); if (grc) return grc; }
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    CK(launch_reset_areas(reinterpret_cast<double*>(m->pos), m->shapeId, m->areas, m->targetAreas,
                          m->comX, m->comY, m->V, m->stream));
    m->launches++;
    return PCP_OK;
}

int pcp_model_save_tentative_positions(pcp_model* m) {
    CHECK_M(m);
    CK(cudaMemcpyAsync(m->posTent, m->pos, (size_t)m->V * sizeof(double2), cudaMemcpyDeviceToDevice,
                       m->stream));
    return PCP_OK;
}

int pcp_model_get_max_effective_force(pcp_model* m, double dt, int minimizer, double* out) {
    CHECK_MO(m, out);
    double scale = (minimizer == PCP_MINIMIZER_GD) ? (1.0 / dt) : (2.0 / (dt * dt));
    CK(launch_max_effective_force(reinterpret_cast<const double*>(m->pos),
                                  reinterpret_cast<const double*>(m->posTent),
                                  reinterpret_cast<const double*>(m->force), m->V, scale, m->dtmp,
                                  m->stream));
    m->launches++;
    CK(cudaMemcpyAsync(out, m->dtmp, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    return sync(m);
}

int pcp_model_sort_keys(pcp_model* m, int end_bit) {
    CHECK_M(m);
    int rc = ensure_records(m);
    if (rc) return rc;
    size_t I = m->hKey.size();
    unsigned long long mask = end_bit >= 64 ? ~0ull : ((1ull << std::max(end_bit, 0)) - 1ull);
    std::vector<uint32_t> perm(I);
    std::iota(perm.begin(), perm.end(), 0u);
    std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) {
        return (m->hKey[a] & mask) < (m->hKey[b] & mask);
    });
    std::vector<unsigned long long> k2(I);
    for (size_t i = 0; i < I; ++i) k2[i] = m->hKey[perm[i]];
    m->hKey.swap(k2);
    m->hKeys = perm;
    return PCP_OK;
}

int pcp_model_update_overlap_area(pcp_model* m, int pd) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    if (pd <= 0) return fail(PCP_ERR_ARG, "point density must be positive");
    // vertex-level sorted cell list (model.cu:308-385) for the Monte-Carlo scan
    std::vector<int> cells(m->V);
    rc = sync(m);
    if (rc) return rc;
    CK(cudaMemcpy(cells.data(), m->cellLocation, m->V * sizeof(int), cudaMemcpyDeviceToHost));
    int B = std::max(1, m->boxSize), nb = B * B;
    std::vector<int> cnt(nb + 1, 0), idx(m->V);
    for (int i = 0; i < m->V; ++i) cnt[std::min(std::max(cells[i], 0), nb - 1) + 1]++;
    for (int c = 0; c < nb; ++c) cnt[c + 1] += cnt[c];
    std::vector<int> starts(cnt.begin(), cnt.end() - 1);
    std::vector<int> fill = starts;
    for (int i = 0; i < m->V; ++i) idx[fill[std::min(std::max(cells[i], 0), nb - 1)]++] = i;
    CK(dalloc(&m->mcNbIdx, (size_t)m->V));
    CK(dalloc(&m->mcBoxStarts, (size_t)nb));
    CK(cudaMemcpy(m->mcNbIdx, idx.data(), m->V * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m->mcBoxStarts, starts.data(), nb * sizeof(int), cudaMemcpyHostToDevice));
    if (pd != m->pointDensity) {
        CK(dalloc(&m->mcCounter, (size_t)pd * pd));
        m->pointDensity = pd;
    }
    CK(launch_overlap_area_mc(m->pos, m->start, m->shapeId, m->mcNbIdx, m->mcBoxStarts, m->V, B,
                              pd, m->mcCounter, m->mcSum, m->stream));
    m->launches++;
    unsigned long long s = 0;
    CK(cudaMemcpyAsync(&s, m->mcSum, sizeof(s), cudaMemcpyDeviceToHost, m->stream));
    rc = sync(m);
    if (rc) return rc;
    m->overlapArea = (double)s / ((double)pd * (double)pd);
    return PCP_OK;
}

int pcp_model_fire_step(pcp_model* m, double dt, double alpha, int n_pos, double dt_max,
                        double alpha_start, double f_alpha, double f_inc, double f_dec, int n_min,
                        int shake_iter, double out[4]) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    FireParams fp{dt, alpha, dt_max, alpha_start, f_alpha, f_inc, f_dec, -1.0,
                  n_pos, n_min, shake_iter, 0};
    return fire_step_once(m, fp, out);
}

int pcp_model_minimize_fire(pcp_model* m, double thr, double dt0, int max_steps, double dt_max,
                            double alpha_start, double f_alpha, double f_inc, double f_dec,
                            int n_min, int shake_iter, double out[3]) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    // Model::minimizeFIRE (model.cpp:488-504)
    rc = pcp_model_reset_velocities(m);
    if (rc) return rc;
    m->geometryStale = false;
    m->geomFromSnapshot = false;
    rc = geometry(m, nullptr);
    if (rc) return rc;
    rc = force_energy(m, nullptr);
    if (rc) return rc;
    bool rigid = m->modelType == PCP_MODEL_NORMAL;
    if (rigid) {
        rc = pcp_model_project_force(m);
        if (rc) return rc;
    }
    FireParams fp{dt0, alpha_start, dt_max, alpha_start, f_alpha, f_inc, f_dec, thr,
                  0, n_min, shake_iter, max_steps};
    rc = build_fire_graph(m, shake_iter);
    if (rc) return rc;
    rc = set_fire_params(m, fp, true);
    if (rc) return rc;
    if (max_steps <= 0) {
        out[0] = m->ctrlHost->energy; out[1] = dt0; out[2] = 0;
        return PCP_OK;
    }
    // Steps are launched in chunks; a step that finds the stop test true (or
    // the step limit) clears `active`, and every later launch is a no-op.
    const int chunk = 32;
    int recoveries = 0;
    for (;;) {
        int left = max_steps - m->ctrlHost->stepsDone;
        int todo = std::min(chunk, left);
        if (todo <= 0) break;
        for (int s = 0; s < todo; ++s) CK(cudaGraphLaunch(m->fireExec, m->stream));
        m->launches += (long long)todo * m->fireKernelNodes;
        rc = read_ctrl(m);
        if (rc) return rc;
        bool redo = false;
        rc = recover_fire(m, redo);
        if (rc) return rc;
        if (redo) {
            if (++recoveries > 16) return fail(PCP_ERR_CAPACITY, "contact buffers could not be sized");
            continue;
        }
        if (!m->ctrlHost->active) break;
    }
    const Ctrl& c = *m->ctrlHost;
    m->lastShakeIters = c.shakeLast;
    m->numIntersections = c.numRecords;
    m->view = pcp_model::VIEW_FINAL;
    m->invalidate();
    if (m->modelType == PCP_MODEL_NORMAL && c.stepsDone > 0) {
        m->geometryStale = true;
        m->geomFromSnapshot = false;
    }
    out[0] = c.converged ? c.outE : c.energy;
    out[1] = c.dt;
    out[2] = c.stepsDone;
    return PCP_OK;
}

int pcp_model_fire_setup(pcp_model* m, double thr, double dt0, int max_steps, double dt_max,
                         double alpha_start, double f_alpha, double f_inc, double f_dec,
                         int n_min, int shake_iter) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    rc = pcp_model_reset_velocities(m);
    if (rc) return rc;
    m->geometryStale = false;
    m->geomFromSnapshot = false;
    rc = geometry(m, nullptr);
    if (rc) return rc;
    rc = force_energy(m, nullptr);
    if (rc) return rc;
    if (m->modelType == PCP_MODEL_NORMAL) {
        rc = pcp_model_project_force(m);
        if (rc) return rc;
    }
    FireParams fp{dt0, alpha_start, dt_max, alpha_start, f_alpha, f_inc, f_dec, thr,
                  0, n_min, shake_iter, max_steps > 0 ? max_steps : 0};
    fp.stagnantTol = m->stopTol;
    fp.stagnantLimit = m->stopStagnant;
    rc = build_fire_graph(m, shake_iter);
    if (rc) return rc;
    return set_fire_params(m, fp, true);
}

int pcp_model_fire_set_stop_rule(pcp_model* m, double energy_tol, int stagnant_limit) {
    CHECK_M(m);
    if (!(energy_tol >= 0.0)) return fail(PCP_ERR_ARG, "energy tolerance must be >= 0");
    m->stopTol = energy_tol;
    m->stopStagnant = stagnant_limit < 0 ? -1 : stagnant_limit;
    return PCP_OK;
}

int pcp_model_fire_run_stats(pcp_model* m, double out[4]) {
    CHECK_M(m);
    int rc = read_ctrl(m);
    if (rc) return rc;
    const Ctrl& c = *m->ctrlHost;
    out[0] = c.stagnated;
    out[1] = c.stepsDone > 0 ? (double)c.shakeMinRun : 1e9;
    out[2] = (double)c.shakeSumRun;
    out[3] = (double)c.shakeMaxRun;
    return PCP_OK;
}

// pyCudaPolygon.py:674-731 (the reference's Python minimizeFIRE) with its
// per-step loop (pyCudaPolygon.py:653-672) run on the device: the same calls
// before the loop, then step graphs launched in chunks without a host round
// trip per step, stopped on the device by |F|max <= thr or by the energy
// stagnation rule of pyCudaPolygon.py:723-727.
}  // extern "C"

// Everything of a device-resident run before its first step.  rule 1: the
// reference's Python driver (pyCudaPolygon.py:674-700: initForceEnergy,
// which resets the cell size to 0.5, and the small gradient step; then its
// loop's start, :658-664) with its stagnation stop rule; rule 0:
// Model::minimizeFIRE (model.cpp:488-496), stopped only by |F|max and the
// step limit.  max_steps <= 0 with rule 1 runs only the calls before the loop.
static int prepare_run(pcp_model* m, int rule, double thr, double dt0, int max_steps,
                       double dt_max, double alpha_start, double f_alpha, double f_inc,
                       double f_dec, int n_min, int shake_iter) {
    int rc = need_topology(m);
    if (rc) return rc;
    const bool normal = m->modelType == PCP_MODEL_NORMAL;
#define RUN(call) do { rc = (call); if (rc) return rc; } while (0)
    if (rule == 1) {
        RUN(pcp_model_reset_velocities(m));
        if (normal) {
            RUN(pcp_model_initialize_neighbor_cells(m));
            RUN(pcp_model_set_max_edge_length(m, 0.5));
            RUN(pcp_model_update_neighbor_cells(m));
            RUN(pcp_model_update_neighbors(m));
            RUN(pcp_model_update_outersections(m));
        }
        RUN(pcp_model_update_polygon_geometry(m));
        RUN(pcp_model_update_force_energy(m));
        if (normal) RUN(pcp_model_project_force(m));
        if (normal && max_steps > 0) {
            RUN(pcp_model_update_positions(m, dt0));
            RUN(pcp_model_update_polygon_geometry(m));
            RUN(pcp_model_update_neighbor_cells(m));
            RUN(pcp_model_update_neighbors(m));
            RUN(pcp_model_update_outersections(m));
            RUN(pcp_model_update_force_energy(m));
            RUN(pcp_model_project_force(m));
            RUN(pcp_model_reset_velocities(m));
        }
        if (max_steps <= 0) return PCP_OK;
    }
#undef RUN
    const double tol0 = m->stopTol;
    const int lim0 = m->stopStagnant;
    m->stopTol = 1e-15;
    m->stopStagnant = rule == 1 ? 5 : -1;
    rc = pcp_model_fire_setup(m, thr, dt0, max_steps, dt_max, alpha_start, f_alpha, f_inc, f_dec,
                              n_min, shake_iter);
    m->stopTol = tol0;
    m->stopStagnant = lim0;
    return rc;
}

extern "C" {

// pyCudaPolygon.py:674-731 (the reference's Python minimizeFIRE) with its
// per-step loop (pyCudaPolygon.py:653-672) run on the device: the same calls
// before the loop, then step graphs launched in chunks without a host round
// trip per step, stopped on the device by |F|max <= thr or by the energy
// stagnation rule of pyCudaPolygon.py:723-727.
int pcp_model_minimize_fire_driver(pcp_model* m, double thr, double dt0, int max_steps,
                                   double dt_max, double alpha_start, double f_alpha, double f_inc,
                                   double f_dec, int n_min, int shake_iter, double out[6]) {
    CHECK_M(m);
    const bool normal = m->modelType == PCP_MODEL_NORMAL;
    int rc = prepare_run(m, 1, thr, dt0, max_steps, dt_max, alpha_start, f_alpha, f_inc, f_dec,
                         n_min, shake_iter);
    if (rc) return rc;
    if (max_steps <= 0) {
        double e = 0.0;
        rc = pcp_model_get_energy(m, &e);
        if (rc) return rc;
        out[0] = e; out[1] = dt0; out[2] = 0; out[3] = 1e9; out[4] = 0; out[5] = 0;
        return PCP_OK;
    }
    const int chunk = 32;
    int recoveries = 0;
    for (;;) {
        int left = max_steps - m->ctrlHost->stepsDone;
        int todo = std::min(chunk, left);
        if (todo <= 0) break;
        for (int s = 0; s < todo; ++s) CK(cudaGraphLaunch(m->fireExec, m->stream));
        m->launches += (long long)todo * m->fireKernelNodes;
        rc = read_ctrl(m);
        if (rc) return rc;
        bool redo = false;
        rc = recover_fire(m, redo);
        if (rc) return rc;
        if (redo) {
            if (++recoveries > 16) return fail(PCP_ERR_CAPACITY, "contact buffers could not be sized");
            continue;
        }
        if (!m->ctrlHost->active) break;
    }
    const Ctrl& c = *m->ctrlHost;
    m->lastShakeIters = c.shakeLast;
    m->numIntersections = c.numRecords;
    m->view = pcp_model::VIEW_FINAL;
    m->invalidate();
    if (normal && c.stepsDone > 0) {
        m->geometryStale = true;
        m->geomFromSnapshot = false;
    }
    out[0] = c.outE;
    out[1] = c.dt;
    out[2] = c.stepsDone;
    out[3] = c.stepsDone > 0 ? (double)c.shakeMinRun : 1e9;
    out[4] = (double)c.shakeSumRun / (double)max_steps;
    out[5] = (double)c.shakeMaxRun;
    return PCP_OK;
}

int pcp_model_fire_continue(pcp_model* m, int n_steps) {
    CHECK_M(m);
    if (!m->fireExec) return fail(PCP_ERR_STATE, "pcp_model_fire_setup has not been called");
    for (int s = 0; s < n_steps; ++s) CK(cudaGraphLaunch(m->fireExec, m->stream));
    m->launches += (long long)n_steps * m->fireKernelNodes;
    if (n_steps > 0 && m->modelType == PCP_MODEL_NORMAL) {
        m->geometryStale = true;
        m->geomFromSnapshot = false;
    }
    return PCP_OK;
}

int pcp_model_fire_status(pcp_model* m, double out[8], int* redo_out) {
    CHECK_MO(m, out);
    int rc = read_ctrl(m);
    if (rc) return rc;
    bool redo = false;
    rc = recover_fire(m, redo);
    if (rc) return rc;
    if (redo_out) *redo_out = redo ? 1 : 0;
    const Ctrl& c = *m->ctrlHost;
    out[0] = c.converged ? c.outE : c.energy;
    out[1] = c.dt; out[2] = c.alpha; out[3] = c.nPos; out[4] = c.maxF;
    out[5] = c.stepsDone; out[6] = c.converged; out[7] = c.shakeLast;
    m->lastShakeIters = c.shakeLast;
    m->numIntersections = c.numRecords;
    m->view = pcp_model::VIEW_FINAL;
    m->invalidate();
    return PCP_OK;
}

int pcp_model_set_positions_device(pcp_model* m, const double* d_pos, int len) {
    CHECK_M(m);
    if (len != 2 * m->V) return fail(PCP_ERR_ARG, "positions must hold 2*numVertices values");
    if (len > 0 && !d_pos) return fail(PCP_ERR_ARG, "null device buffer");
    if (len > 0)
        CK(cudaMemcpyAsync(m->pos, d_pos, (size_t)len * sizeof(double), cudaMemcpyDeviceToDevice,
                           m->stream));
    // the same state changes as the host setter
    m->geometryStale = false;
    m->geomFromSnapshot = false;
    m->invalidate();
    return PCP_OK;
}

int pcp_model_overlap_energy_gradient(pcp_model* m, int mode, int search, double* energy_out,
                                      double* d_out) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    if (mode != kRefForce && mode != kExactGrad) return fail(PCP_ERR_ARG, "unknown mode %d", mode);
    if (!d_out || !energy_out) return fail(PCP_ERR_ARG, "null output");
    if (search) {
        rc = run_contacts(m);
        if (rc) return rc;
        m->view = pcp_model::VIEW_COMPACT;
        m->invalidate();
    }
    if (!m->gradEnergy) CK(dalloc(&m->gradEnergy, 1));
    if (!m->gradBad) CK(dalloc(&m->gradBad, 1));
    CK(cudaMemsetAsync(d_out, 0, (size_t)m->V * 2 * sizeof(double), m->stream));
    CK(cudaMemsetAsync(m->gradEnergy, 0, sizeof(double), m->stream));
    CK(cudaMemsetAsync(m->gradBad, 0, sizeof(int), m->stream));
    CK(launch_overlap_energy_grad(m->pos, m->start, m->V, m->ws, m->ctrl, mode,
                                  reinterpret_cast<double2*>(d_out), m->gradEnergy, m->gradBad,
                                  m->stream));
    m->launches++;
    int bad = 0;
    CK(cudaMemcpyAsync(energy_out, m->gradEnergy, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    CK(cudaMemcpyAsync(&bad, m->gradBad, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    rc = sync(m);
    if (rc) return rc;
    if (bad) return fail(PCP_ERR_NUMERIC, "a crossing record names a vertex outside its polygon");
    return PCP_OK;
}

int pcp_model_contacts_stage(pcp_model* m, int stage) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    if (stage == 0 || stage == 1) {
        CK(launch_contacts(m->pos, m->start, m->shapeId, m->cellLocation, m->P, m->V, m->boxSize,
                           m->ws, m->ctrl, nullptr, m->stream, stage == 0 ? 1 : 2));
        m->launches += stage == 0 ? 6 : 4;
    } else if (stage == 2) {
        // nothing left to launch: the fixup runs at the end of stage 1
    } else {
        return fail(PCP_ERR_ARG, "unknown contact stage %d", stage);
    }
    m->view = pcp_model::VIEW_FINAL;
    m->invalidate();
    return PCP_OK;
}

// ---- scalar getters ----
int pcp_model_get_num_vertices(pcp_model* m, int* out) { CHECK_MO(m, out); *out = m->V; return PCP_OK; }
int pcp_model_get_num_polygons(pcp_model* m, int* out) { CHECK_MO(m, out); *out = m->P; return PCP_OK; }
int pcp_model_get_num_intersections(pcp_model* m, int* out) { CHECK_MO(m, out); *out = m->numIntersections; return PCP_OK; }
int pcp_model_get_max_neighbors(pcp_model* m, int* out) {
    CHECK_MO(m, out);
    if (m->topology && m->view != pcp_model::VIEW_NONE) {
        int rc = ensure_neighbors(m);
        if (rc) return rc;
    }
    *out = m->maxNeighbors;
    return PCP_OK;
}
int pcp_model_get_box_size(pcp_model* m, int* out) { CHECK_MO(m, out); *out = m->boxSize; return PCP_OK; }
int pcp_model_get_model_enum(pcp_model* m, int* out) { CHECK_MO(m, out); *out = m->modelType; return PCP_OK; }
int pcp_model_get_last_shake_iters(pcp_model* m, int* out) { CHECK_MO(m, out); *out = m->lastShakeIters; return PCP_OK; }
int pcp_model_get_energy(pcp_model* m, double* out) {
    CHECK_MO(m, out);
    int rc = read_ctrl(m);
    if (rc) return rc;
    *out = m->ctrlHost->energy;
    return PCP_OK;
}
int pcp_model_get_max_unbalanced_force(pcp_model* m, double* out) {
    CHECK_MO(m, out);
    if (m->maxFSerial != 0 && m->maxFSerial + 1 == m->callSerial) {
        // the FIRE step just before read it back with its control block (the
        // same maximum over the same forces); the reference's per-step loop
        // (pyCudaPolygon.py:666-668) asks for it after every step
        *out = m->maxFCached;
        return PCP_OK;
    }
    CK(launch_max_abs(reinterpret_cast<const double*>(m->force), 2 * m->V, m->dtmp, m->stream));
    m->launches++;
    CK(cudaMemcpyAsync(out, m->dtmp, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    return sync(m);
}
int pcp_model_get_max_edge_length(pcp_model* m, double* out) {
    if (m && m->geometryStale) { int grc = ensure_geometry(m); if (grc) return grc; }
    CHECK_MO(m, out);
    CK(cudaMemcpyAsync(out, m->maxEdge, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    return sync(m);
}
int pcp_model_get_overlap_area(pcp_model* m, double* out) { CHECK_MO(m, out); *out = m->overlapArea; return PCP_OK; }

// ---- array getters ----
int pcp_model_get_positions(pcp_model* m, double* out, int cap, int* len) {
    CHECK_M(m); return copy_dev_out(m, reinterpret_cast<const double*>(m->pos), 2 * m->V, out, cap, len);
}
int pcp_model_get_forces(pcp_model* m, double* out, int cap, int* len) {
    CHECK_M(m); return copy_dev_out(m, reinterpret_cast<const double*>(m->force), 2 * m->V, out, cap, len);
}
int pcp_model_get_velocities(pcp_model* m, double* out, int cap, int* len) {
    CHECK_M(m);
    if (m->V > 0) {
        // the last FIRE step's bend, if the next step has not applied it yet
        CK(launch_fire_settle(m->vel, m->force, m->V, m->ctrl, m->stream));
        CK(cudaMemsetAsync(&m->ctrl->bendMode, 0, sizeof(int), m->stream));
    }
    return copy_dev_out(m, reinterpret_cast<const double*>(m->vel), 2 * m->V, out, cap, len);
}
int pcp_model_get_areas(pcp_model* m, double* out, int cap, int* len) {
    if (m && m->geometryStale) { int grc = ensure_geometry(m); if (grc) return grc; }
    CHECK_M(m); return copy_dev_out(m, (const double*)m->areas, m->P, out, cap, len);
}
int pcp_model_get_com(pcp_model* m, double* out, int cap, int* len) {
    if (m && m->geometryStale) { int grc = ensure_geometry(m); if (grc) return grc; }
    CHECK_M(m);
    if (len) *len = 2 * m->P;
    if (!out) return PCP_OK;
    if (cap < 2 * m->P) return fail(PCP_ERR_ARG, "output buffer too small");
    int rc = copy_dev_out(m, (const double*)m->comX, m->P, out, cap, nullptr);
    if (rc) return rc;
    return copy_dev_out(m, (const double*)m->comY, m->P, out + m->P, cap - m->P, nullptr);
}
int pcp_model_get_perimeters(pcp_model* m, double* out, int cap, int* len) {
    if (m && m->geometryStale) { int grc = ensure_geometry(m); if (grc) return grc; }
    CHECK_M(m); return copy_dev_out(m, (const double*)m->perimeters, m->P, out, cap, len);
}
int pcp_model_get_edge_lengths(pcp_model* m, double* out, int cap, int* len) {
    if (m && m->geometryStale) { int grc = ensure_geometry(m); if (grc) return grc; }
    CHECK_M(m); return copy_dev_out(m, (const double*)m->edgeLengths, m->V, out, cap, len);
}
int pcp_model_get_constraints(pcp_model* m, double* out, int cap, int* len) {
    if (m && m->geometryStale) { int grc = ensure_geometry(m); if (grc) return grc; }
    CHECK_M(m); return copy_dev_out(m, (const double*)m->constraints, 6 * m->V, out, cap, len);
}
int pcp_model_get_target_areas(pcp_model* m, double* out, int cap, int* len) {
    CHECK_M(m); return copy_dev_out(m, (const double*)m->targetAreas, m->P, out, cap, len);
}
int pcp_model_get_target_edge_lengths(pcp_model* m, double* out, int cap, int* len) {
    CHECK_M(m); return copy_dev_out(m, (const double*)m->targetEdge, m->P, out, cap, len);
}
int pcp_model_get_start_indices(pcp_model* m, int* out, int cap, int* len) {
    CHECK_M(m); return copy_out(m->startHost.data(), (int)m->startHost.size(), out, cap, len);
}
int pcp_model_get_shape_id(pcp_model* m, int* out, int cap, int* len) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    return copy_dev_out(m, (const int*)m->shapeId, m->V, out, cap, len);
}
int pcp_model_get_neighbor_cells(pcp_model* m, int* out, int cap, int* len) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    return copy_dev_out(m, (const int*)m->cellLocation, m->V, out, cap, len);
}

static int sorted_cells(pcp_model* m, std::vector<int>& idx, std::vector<int>& starts) {
    int rc = sync(m);
    if (rc) return rc;
    std::vector<int> cells(m->V);
    if (m->V) CK(cudaMemcpy(cells.data(), m->cellLocation, m->V * sizeof(int), cudaMemcpyDeviceToHost));
    int B = std::max(1, m->boxSize), nb = B * B;
    // stable sort of vertex ids by cell + lower bound per cell (model.cu:308-377)
    idx.resize(m->V);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cells[a] < cells[b]; });
    starts.assign(nb, 0);
    for (int c = 0; c < nb; ++c)
        starts[c] = (int)(std::lower_bound(idx.begin(), idx.end(), c,
                                           [&](int v, int cc) { return cells[v] < cc; }) - idx.begin());
    return PCP_OK;
}

int pcp_model_get_neighbor_indices(pcp_model* m, int* out, int cap, int* len) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    std::vector<int> idx, starts;
    rc = sorted_cells(m, idx, starts);
    if (rc) return rc;
    return copy_out(idx.data(), (int)idx.size(), out, cap, len);
}
int pcp_model_get_box_counts(pcp_model* m, int* out, int cap, int* len) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    std::vector<int> idx, starts;
    rc = sorted_cells(m, idx, starts);
    if (rc) return rc;
    return copy_out(starts.data(), (int)starts.size(), out, cap, len);
}
int pcp_model_get_neighbors(pcp_model* m, int* out, int cap, int* len) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    rc = ensure_neighbors(m);
    if (rc) return rc;
    return copy_out(m->hNeighbors.data(), (int)m->hNeighbors.size(), out, cap, len);
}
int pcp_model_get_num_neighbors(pcp_model* m, int* out, int cap, int* len) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    rc = ensure_neighbors(m);
    if (rc) return rc;
    return copy_out(m->hNumNeighbors.data(), (int)m->hNumNeighbors.size(), out, cap, len);
}
int pcp_model_get_inside_flag(pcp_model* m, uint8_t* out, int cap, int* len) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    rc = ensure_neighbors(m);
    if (rc) return rc;
    return copy_out(m->hInside.data(), (int)m->hInside.size(), out, cap, len);
}
int pcp_model_get_shape_counts(pcp_model* m, int* out, int cap, int* len) {
    CHECK_M(m);
    int rc = need_topology(m);
    if (rc) return rc;
    rc = ensure_neighbors(m);
    if (rc) return rc;
    return copy_out(m->hShapeCounts.data(), (int)m->hShapeCounts.size(), out, cap, len);
}

static int records_or_empty(pcp_model* m) {
    if (!m->topology || m->view == pcp_model::VIEW_NONE) {
        m->hKey.clear(); m->hOuter.clear(); m->hTU.clear(); m->hUT.clear(); m->hKeys.clear();
        return PCP_OK;
    }
    return ensure_records(m);
}

int pcp_model_get_intersections(pcp_model* m, uint64_t* out, int cap, int* len) {
    CHECK_M(m);
    int rc = records_or_empty(m);
    if (rc) return rc;
    return copy_out(reinterpret_cast<const uint64_t*>(m->hKey.data()), (int)m->hKey.size(), out, cap, len);
}
int pcp_model_get_outersections(pcp_model* m, uint64_t* out, int cap, int* len) {
    CHECK_M(m);
    int rc = records_or_empty(m);
    if (rc) return rc;
    return copy_out(reinterpret_cast<const uint64_t*>(m->hOuter.data()), (int)m->hOuter.size(), out, cap, len);
}
static int tu_out(const std::vector<float2>& v, double* out, int cap, int* len) {
    int n = 2 * (int)v.size();
    if (len) *len = n;
    if (!out) return PCP_OK;
    if (cap < n) return fail(PCP_ERR_ARG, "output buffer too small");
    for (size_t i = 0; i < v.size(); ++i) { out[2 * i] = (double)v[i].x; out[2 * i + 1] = (double)v[i].y; }
    return PCP_OK;
}
int pcp_model_get_tu(pcp_model* m, double* out, int cap, int* len) {
    CHECK_M(m);
    int rc = records_or_empty(m);
    if (rc) return rc;
    return tu_out(m->hTU, out, cap, len);
}
int pcp_model_get_ut(pcp_model* m, double* out, int cap, int* len) {
    CHECK_M(m);
    int rc = records_or_empty(m);
    if (rc) return rc;
    return tu_out(m->hUT, out, cap, len);
}
int pcp_model_get_keys(pcp_model* m, uint32_t* out, int cap, int* len) {
    CHECK_M(m);
    int rc = records_or_empty(m);
    if (rc) return rc;
    return copy_out(m->hKeys.data(), (int)m->hKeys.size(), out, cap, len);
}
int pcp_model_get_intersections_counter(pcp_model* m, int* out, int cap, int* len) {
    CHECK_M(m);
    int n = m->pointDensity > 0 ? m->pointDensity * m->pointDensity : 0;
    if (n == 0) { if (len) *len = 0; return PCP_OK; }
    return copy_dev_out(m, (const int*)m->mcCounter, n, out, cap, len);
}

int pcp_model_device_positions(pcp_model* m, double** out) {
    CHECK_MO(m, out); *out = reinterpret_cast<double*>(m->pos); return PCP_OK;
}
int pcp_model_device_forces(pcp_model* m, double** out) {
    CHECK_MO(m, out); *out = reinterpret_cast<double*>(m->force); return PCP_OK;
}
int pcp_model_get_pair_count(pcp_model* m, long long* out) {
    CHECK_MO(m, out);
    int rc = read_ctrl(m);
    if (rc) return rc;
    *out = (long long)m->ctrlHost->pairEvals;
    return PCP_OK;
}
// ---- tensor-core kernels of the learned warm start (warmstart.cu) ----
int pcp_gemm_bf16(const void* d_a, const void* d_b, float* d_c, int m, int n, int k,
                  const float* d_bias, int relu, int splits, void* stream) {
    if (m < 0 || n < 0 || k < 0 || splits < 1)
        return fail(PCP_ERR_ARG, "pcp_gemm_bf16: negative size or splits < 1");
    if (m == 0 || n == 0) return PCP_OK;
    if (!d_a || !d_b || !d_c) return fail(PCP_ERR_ARG, "pcp_gemm_bf16: null buffer");
    if (k == 0 || k % 8 != 0)
        return fail(PCP_ERR_ARG, "pcp_gemm_bf16: K must be a positive multiple of 8");
    // A and B: the tensor maps' base addresses; C: the epilogue's 16-byte
    // row stores
    if ((reinterpret_cast<uintptr_t>(d_a) | reinterpret_cast<uintptr_t>(d_b) |
         reinterpret_cast<uintptr_t>(d_c)) % 16 != 0)
        return fail(PCP_ERR_ARG, "pcp_gemm_bf16: A, B and C must be 16-byte aligned");
    if (splits > 1 && relu)
        return fail(PCP_ERR_ARG, "pcp_gemm_bf16: ReLU needs the whole K sum (splits = 1)");
    int rc = launch_gemm_bf16(d_a, d_b, d_c, m, n, k, d_bias, relu, splits,
                              static_cast<cudaStream_t>(stream));
    if (rc == -1) return fail(PCP_ERR_CUDA, "pcp_gemm_bf16: tensor map encoding failed");
    if (rc != 0)
        return fail(PCP_ERR_CUDA, "pcp_gemm_bf16: %s", cudaGetErrorString((cudaError_t)rc));
    return PCP_OK;
}

int pcp_gemm_status(int* out) {
    if (!out) return fail(PCP_ERR_ARG, "pcp_gemm_status: null output");
    CK(gemm_error_flag(out));
    return PCP_OK;
}

int pcp_graph_sum_bf16(const int* d_rowptr, const int* d_col, const void* d_h, void* d_out, int v,
                       int f, float scale, void* stream) {
    if (v < 0 || f <= 0 || f % 2 != 0)
        return fail(PCP_ERR_ARG, "pcp_graph_sum_bf16: bad sizes (f must be positive and even)");
    if (v == 0) return PCP_OK;
    if (!d_rowptr || !d_col || !d_h || !d_out)
        return fail(PCP_ERR_ARG, "pcp_graph_sum_bf16: null buffer");
    if ((reinterpret_cast<uintptr_t>(d_h) | reinterpret_cast<uintptr_t>(d_out)) % 4 != 0)
        return fail(PCP_ERR_ARG, "pcp_graph_sum_bf16: h and out must be 4-byte aligned");
    CK(launch_graph_sum_bf16(d_rowptr, d_col, d_h, d_out, v, f, scale,
                             static_cast<cudaStream_t>(stream)));
    return PCP_OK;
}

int pcp_control_block_bytes(void) { return (int)sizeof(Ctrl); }
int pcp_model_get_narrow_pair_total(pcp_model* m, long long* out) {
    CHECK_MO(m, out);
    int rc = read_ctrl(m);
    if (rc) return rc;
    *out = (long long)(m->ctrlHost->narrowEvals - m->ctrlHost->selfEvals);
    return PCP_OK;
}
int pcp_model_get_narrow_pair_count(pcp_model* m, int* pairs_out, int* self_out) {
    CHECK_M(m);
    int rc = read_ctrl(m);
    if (rc) return rc;
    if (pairs_out) *pairs_out = m->ctrlHost->numPairs - m->ctrlHost->numSelf;
    if (self_out) *self_out = m->ctrlHost->numSelf;
    return PCP_OK;
}
int pcp_model_get_launch_count(pcp_model* m, long long* out) {
    CHECK_MO(m, out);
    int rc = read_ctrl(m);
    if (rc) return rc;
    *out = m->launches + (long long)m->ctrlHost->condLaunches;
    return PCP_OK;
}

// ---- stateless launchers ----
int pcp_topology(const int* d_start, int P, int V, int* d_shape_id, int* d_next, int* d_prev,
                 void* stream) {
    if (P < 0 || V < 0) return fail(PCP_ERR_ARG, "pcp_topology: negative size");
    if (P > 0 && (!d_start || !d_shape_id || !d_next || !d_prev))
        return fail(PCP_ERR_ARG, "pcp_topology: null device buffer");
    CK(launch_topology(d_start, P, V, d_shape_id, d_next, d_prev, (cudaStream_t)stream));
    return PCP_OK;
}

int pcp_polygon_geometry(const double* d_pos, const int* d_start, int P, int V,
                         double* d_edge_lengths, double* d_areas, double* d_com_x, double* d_com_y,
                         double* d_perimeters, double* d_constraints, double* d_max_edge,
                         void* stream) {
    if (P < 0 || V < 0) return fail(PCP_ERR_ARG, "pcp_polygon_geometry: negative size");
    if (P > 0 && (!d_pos || !d_start || !d_edge_lengths || !d_areas || !d_com_x || !d_com_y ||
                  !d_perimeters || !d_constraints || !d_max_edge))
        return fail(PCP_ERR_ARG, "pcp_polygon_geometry: null device buffer");
    CK(launch_geometry(reinterpret_cast<const double2*>(d_pos), d_start, P, V, d_edge_lengths,
                       d_areas, d_com_x, d_com_y, d_perimeters, d_constraints, d_max_edge, nullptr,
                       (cudaStream_t)stream));
    return PCP_OK;
}

int pcp_neighbor_cells(const double* d_pos, const int* d_start, const int* d_shape_id, int V,
                       int B, int* d_cell, void* stream) {
    if (V < 0 || B < 1)
        return fail(PCP_ERR_ARG, "pcp_neighbor_cells: negative size or box_size < 1");
    if (V > 0 && (!d_pos || !d_start || !d_shape_id || !d_cell))
        return fail(PCP_ERR_ARG, "pcp_neighbor_cells: null device buffer");
    CK(launch_neighbor_cells(reinterpret_cast<const double2*>(d_pos), d_start, d_shape_id, V, B,
                             d_cell, nullptr, (cudaStream_t)stream));
    return PCP_OK;
}

// The stateless projection and SHAKE launchers need per-vertex scratch; the
// caller's stream gets a scratch buffer of kScratchPerVertex doubles per
// vertex that is allocated on first use and kept until the process ends.
static double* stateless_scratch(int V) {
    static double* buf = nullptr;
    static size_t cap = 0;
    size_t need = (size_t)kScratchPerVertex * (size_t)std::max(V, 1);
    if (need > cap) {
        if (buf) cudaFree(buf);
        buf = nullptr;
        if (cudaMalloc((void**)&buf, need * sizeof(double)) != cudaSuccess) { cap = 0; return nullptr; }
        cap = need;
    }
    return buf;
}

// Reads the CSR offsets back and checks them: the kernels index positions
// and scratch by them, and the scratch is sized from start[P].
static int start_info(const int* d_start, int P, int& V, int& nmax) {
    if (P < 0) return fail(PCP_ERR_ARG, "negative polygon count");
    if (P > 0 && !d_start) return fail(PCP_ERR_ARG, "null start array");
    std::vector<int> h(P + 1, 0);
    if (P > 0) CK(cudaMemcpy(h.data(), d_start, (P + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    if (h[0] != 0) return fail(PCP_ERR_ARG, "start must begin at 0 and never decrease");
    V = h[P];
    nmax = 0;
    for (int p = 0; p < P; ++p) {
        if (h[p + 1] < h[p]) return fail(PCP_ERR_ARG, "start must begin at 0 and never decrease");
        nmax = std::max(nmax, h[p + 1] - h[p]);
    }
    return PCP_OK;
}

int pcp_project_force(const double* d_pos, const int* d_start, int P, const double* d_constraints,
                      double* d_force, void* stream) {
    if (P > 0 && (!d_pos || !d_constraints || !d_force))
        return fail(PCP_ERR_ARG, "pcp_project_force: null device buffer");
    int V = 0, nmax = 0;
    int rc = start_info(d_start, P, V, nmax);
    if (rc) return rc;
    if (constraints_init() != cudaSuccess) return fail(PCP_ERR_CUDA, "kernel setup failed");
    double* s = stateless_scratch(V);
    if (!s) return fail(PCP_ERR_CUDA, "scratch allocation failed");
    CK(launch_project(reinterpret_cast<const double2*>(d_pos), d_start, P, nmax, d_constraints,
                      reinterpret_cast<double2*>(d_force), s, V, 0, nullptr, nullptr, nullptr,
                      (cudaStream_t)stream));
    return PCP_OK;
}

int pcp_shake_project(double* d_pos, const int* d_start, int P, const double* d_tl,
                      const double* d_ta, int max_iter, double tol, int* d_max_iters, void* stream) {
    if (!d_max_iters) return fail(PCP_ERR_ARG, "pcp_shake_project: null d_max_iters");
    if (P > 0 && (!d_pos || !d_tl || !d_ta))
        return fail(PCP_ERR_ARG, "pcp_shake_project: null device buffer");
    int V = 0, nmax = 0;
    int rc = start_info(d_start, P, V, nmax);
    if (rc) return rc;
    if (constraints_init() != cudaSuccess) return fail(PCP_ERR_CUDA, "kernel setup failed");
    double* s = stateless_scratch(V);
    if (!s) return fail(PCP_ERR_CUDA, "scratch allocation failed");
    CK(cudaMemsetAsync(d_max_iters, 0, sizeof(int), (cudaStream_t)stream));
    CK(launch_shake(reinterpret_cast<double2*>(d_pos), d_start, P, nmax, d_tl, d_ta, max_iter, tol,
                    d_max_iters, s, V, nullptr, (cudaStream_t)stream));
    return PCP_OK;
}

int pcp_rcp_newton(const double* d_x, double* d_y, int n, void* stream) {
    if (n < 0) return fail(PCP_ERR_ARG, "negative count");
    if (n > 0 && (!d_x || !d_y)) return fail(PCP_ERR_ARG, "null buffer");
    CK(launch_rcp_newton(d_x, d_y, n, (cudaStream_t)stream));
    return PCP_OK;
}

// SHAKE with its workspace in a static device array of this library: no
// cudaMalloc, cudaFree or other allocation.  A one-block kernel checks the
// CSR offsets against the array first and the call waits for its verdict, so
// a start array that would reach past the array launches nothing.
int pcp_shake_project_noalloc(double* d_pos, const int* d_start, int P, const double* d_tl,
                              const double* d_ta, int max_iter, double tol, int* d_max_iters,
                              void* stream) {
    if (P < 0) return fail(PCP_ERR_ARG, "negative polygon count");
    if (!d_max_iters) return fail(PCP_ERR_ARG, "null d_max_iters");
    if (P > 0 && (!d_pos || !d_start || !d_tl || !d_ta))
        return fail(PCP_ERR_ARG, "null device buffer");
    cudaStream_t st = (cudaStream_t)stream;
    double* scratch = nullptr;
    CK(shake_noalloc_scratch(&scratch));
    if (P > 0) {
        int status = 0;
        CK(shake_noalloc_check(d_start, P, &status, st));
        if (status == 1)
            return fail(PCP_ERR_ARG,
                        "pcp_shake_project_noalloc: start must begin at 0 and never decrease");
        if (status == 2)
            return fail(PCP_ERR_CAPACITY,
                        "pcp_shake_project_noalloc: more vertices than its static workspace of %d "
                        "vertices; use pcp_shake_project",
                        PCP_SHAKE_NOALLOC_MAX_VERTICES);
    }
    CK(cudaMemsetAsync(d_max_iters, 0, sizeof(int), st));
    CK(launch_shake_noalloc(reinterpret_cast<double2*>(d_pos), d_start, P, d_tl, d_ta, max_iter,
                            tol, d_max_iters, scratch, st));
    return PCP_OK;
}

int pcp_update_positions(double* d_pos, const double* d_force, int V, double dt, void* stream) {
    if (V < 0) return fail(PCP_ERR_ARG, "pcp_update_positions: negative size");
    if (V > 0 && (!d_pos || !d_force))
        return fail(PCP_ERR_ARG, "pcp_update_positions: null device buffer");
    CK(launch_update_positions(d_pos, d_force, V, dt, (cudaStream_t)stream));
    return PCP_OK;
}

}  // extern "C"

// ======================================================================
// Many independent systems minimised together (no reference counterpart;
// the reference runs one system per Model).  Every system keeps its own
// model, buffers and step graph; the batch gives each a stream of a pool of
// streams, launches each system's graph of `chunk` consecutive FIRE steps
// on its stream, reads all control blocks back once per chunk and drops the
// systems that have stopped.  Systems on different streams run at the same
// time, so small systems fill the GPU together.
// ======================================================================
struct pcp_batch {
    std::vector<pcp_model*> models;
    std::vector<cudaStream_t> streams;
    int nStreams = 16;
    int chunk = 8;
    std::string report;          // the last autotune table (JSON)
    ~pcp_batch() {
        for (cudaStream_t s : streams) cudaStreamDestroy(s);
    }
};

namespace {

int batch_streams(pcp_batch* b) {
    while ((int)b->streams.size() < b->nStreams) {
        cudaStream_t s = nullptr;
        CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        b->streams.push_back(s);
    }
    return PCP_OK;
}

struct RunArgs {
    int rule;
    double thr, dt0;
    int maxSteps;
    double dtMax, alphaStart, fAlpha, fInc, fDec;
    int nMin, shakeIter;
};

// Prepare every system (on its own stream), then launch chunks of steps
// until every system has stopped.  `which` lists the systems to run.
int batch_run(pcp_batch* b, const std::vector<int>& which, const RunArgs& a) {
    int rc = batch_streams(b);
    if (rc) return rc;
    const int K = b->nStreams;
    for (size_t q = 0; q < which.size(); ++q) {
        pcp_model* m = b->models[which[q]];
        m->stream = b->streams[q % K];
        rc = prepare_run(m, a.rule, a.thr, a.dt0, a.maxSteps, a.dtMax, a.alphaStart, a.fAlpha,
                         a.fInc, a.fDec, a.nMin, a.shakeIter);
        if (rc) return rc;
        rc = build_fire_graph_multi(m, a.shakeIter, b->chunk);
        if (rc) return rc;
    }
    std::vector<int> active = which;
    int recoveries = 0;
    while (!active.empty()) {
        for (int i : active) {
            pcp_model* m = b->models[i];
            CK(cudaGraphLaunch(m->fireExecMulti, m->stream));
            m->launches += (long long)b->chunk * m->fireKernelNodes;
            CK(cudaMemcpyAsync(m->ctrlHost, m->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost,
                               m->stream));
        }
        for (cudaStream_t s : b->streams) CK(cudaStreamSynchronize(s));
        std::vector<int> next;
        for (int i : active) {
            pcp_model* m = b->models[i];
            bool redo = false;
            rc = recover_fire(m, redo);
            if (rc) return rc;
            if (redo) {
                if (++recoveries > 16 * (int)b->models.size())
                    return fail(PCP_ERR_CAPACITY, "contact buffers could not be sized");
                rc = build_fire_graph_multi(m, a.shakeIter, b->chunk);
                if (rc) return rc;
                next.push_back(i);
            } else if (m->ctrlHost->active) {
                next.push_back(i);
            }
        }
        active.swap(next);
    }
    for (int i : which) {
        pcp_model* m = b->models[i];
        const Ctrl& c = *m->ctrlHost;
        m->lastShakeIters = c.shakeLast;
        m->numIntersections = c.numRecords;
        m->view = pcp_model::VIEW_FINAL;
        m->invalidate();
        if (m->modelType == PCP_MODEL_NORMAL && c.stepsDone > 0) {
            m->geometryStale = true;
            m->geomFromSnapshot = false;
        }
    }
    return PCP_OK;
}

}  // namespace

extern "C" {

int pcp_batch_create(pcp_batch** out) {
    if (!out) return fail(PCP_ERR_ARG, "null output");
    *out = new pcp_batch();
    return PCP_OK;
}

int pcp_batch_destroy(pcp_batch* b) {
    delete b;
    return PCP_OK;
}

int pcp_batch_add(pcp_batch* b, pcp_model* m) {
    if (!b || !m) return fail(PCP_ERR_ARG, "null batch or model");
    int rc = need_topology(m);
    if (rc) return rc;
    b->models.push_back(m);
    return PCP_OK;
}

int pcp_batch_size(pcp_batch* b, int* out) {
    if (!b || !out) return fail(PCP_ERR_ARG, "null argument");
    *out = (int)b->models.size();
    return PCP_OK;
}

int pcp_batch_set_streams(pcp_batch* b, int n_streams, int chunk_steps) {
    if (!b) return fail(PCP_ERR_ARG, "null batch");
    if (n_streams < 1 || n_streams > 256 || chunk_steps < 1 || chunk_steps > 256)
        return fail(PCP_ERR_ARG, "streams and chunk steps must be in 1..256");
    b->nStreams = n_streams;
    b->chunk = chunk_steps;
    return PCP_OK;
}

int pcp_model_set_launch_shape(pcp_model* m, int narrow_blocks, int force_blocks) {
    CHECK_M(m);
    if (narrow_blocks < 0 || force_blocks < 0) return fail(PCP_ERR_ARG, "negative block count");
    if (narrow_blocks > kMaxNarrowBlocks)
        return fail(PCP_ERR_ARG, "at most %d narrow-phase blocks", kMaxNarrowBlocks);
    if (m->ws.narrowBlocks != narrow_blocks || m->ws.forceBlocks != force_blocks) {
        m->ws.narrowBlocks = narrow_blocks;
        m->ws.forceBlocks = force_blocks;
        m->generation++;          // the step graphs bake the grids in: rebuild them
    }
    return PCP_OK;
}

int pcp_model_get_launch_shape(pcp_model* m, int out[2]) {
    CHECK_M(m);
    out[0] = m->ws.narrowBlocks > 0 ? m->ws.narrowBlocks : sm_count() * 4;
    out[1] = m->ws.forceBlocks > 0 ? m->ws.forceBlocks : sm_count() * 4;
    return PCP_OK;
}

int pcp_batch_minimize_fire(pcp_batch* b, int rule, double thr, double dt0, int max_steps,
                            double dt_max, double alpha_start, double f_alpha, double f_inc,
                            double f_dec, int n_min, int shake_iter, double* out) {
    if (!b || !out) return fail(PCP_ERR_ARG, "null argument");
    if (rule != 0 && rule != 1) return fail(PCP_ERR_ARG, "rule must be 0 or 1");
    if (max_steps <= 0) return fail(PCP_ERR_ARG, "max_steps must be positive");
    std::vector<int> all(b->models.size());
    for (size_t i = 0; i < all.size(); ++i) all[i] = (int)i;
    RunArgs a{rule, thr, dt0, max_steps, dt_max, alpha_start, f_alpha, f_inc, f_dec, n_min,
              shake_iter};
    std::vector<cudaStream_t> saved;
    for (pcp_model* m : b->models) saved.push_back(m->stream);
    int rc = batch_run(b, all, a);
    for (size_t i = 0; i < b->models.size(); ++i) b->models[i]->stream = saved[i];
    if (rc) return rc;
    for (size_t i = 0; i < b->models.size(); ++i) {
        const Ctrl& c = *b->models[i]->ctrlHost;
        out[4 * i + 0] = c.outE;
        out[4 * i + 1] = c.dt;
        out[4 * i + 2] = c.stepsDone;
        out[4 * i + 3] = c.converged ? 1 : (c.stagnated ? 2 : 0);
    }
    return PCP_OK;
}

// Autotuner of the launch shapes: systems are grouped by polygon count
// (classes [2^k, 2^(k+1))); for each class every candidate grid (SMs x {1/4,
// 1/2, 1, 2, 4} blocks for both the narrow phase and the force pass) runs
// `steps` FIRE steps of all the class's systems at once on the batch's
// streams from the same start positions, and the fastest is kept for the
// class.  Positions are restored after each trial.  shapes_out (2 per
// system, may be null) receives the chosen (narrow, force) blocks; the table
// of timings is kept as JSON for pcp_batch_autotune_report.
int pcp_batch_autotune(pcp_batch* b, int steps, int* shapes_out) {
    if (!b) return fail(PCP_ERR_ARG, "null batch");
    if (steps < 1) return fail(PCP_ERR_ARG, "steps must be positive");
    const int n = (int)b->models.size();
    std::map<int, std::vector<int>> classes;
    for (int i = 0; i < n; ++i) {
        int p = std::max(1, b->models[i]->P), k = 0;
        while ((2 << k) <= p) ++k;
        classes[k].push_back(i);
    }
    const int sm = sm_count();
    const int cand[5] = {std::max(1, sm / 4), std::max(1, sm / 2), sm, 2 * sm, 4 * sm};
    std::vector<cudaStream_t> saved;
    for (pcp_model* m : b->models) saved.push_back(m->stream);
    std::vector<double2*> keep(n, nullptr);
    int rc = PCP_OK;
    std::string rep = "{\"candidates_blocks\": [";
    for (int c = 0; c < 5; ++c) rep += (c ? ", " : "") + std::to_string(cand[c]);
    rep += "], \"classes\": [";
    bool firstClass = true;
    for (int i = 0; i < n && rc == PCP_OK; ++i) {
        pcp_model* m = b->models[i];
        if (dalloc(&keep[i], (size_t)m->V) != cudaSuccess) rc = fail(PCP_ERR_CUDA, "autotune buffer");
        else if (cudaMemcpy(keep[i], m->pos, (size_t)m->V * sizeof(double2),
                            cudaMemcpyDeviceToDevice) != cudaSuccess)
            rc = fail(PCP_ERR_CUDA, "autotune copy");
    }
    RunArgs a{0, -1.0, 1e-3, steps, 0.1, 0.1, 0.99, 1.1, 0.5, 5, 5};
    for (auto& kv : classes) {
        if (rc) break;
        const std::vector<int>& which = kv.second;
        double best = 1e300;
        int bestC = 2;
        std::string row = "{\"polygons_from\": " + std::to_string(1 << kv.first) +
                          ", \"systems\": " + std::to_string(which.size()) + ", \"ms\": [";
        for (int c = 0; c < 5 && rc == PCP_OK; ++c) {
            for (int i : which) {
                rc = pcp_model_set_launch_shape(b->models[i], cand[c], cand[c]);
                if (rc) break;
                if (cudaMemcpy(b->models[i]->pos, keep[i], (size_t)b->models[i]->V * sizeof(double2),
                               cudaMemcpyDeviceToDevice) != cudaSuccess)
                    rc = fail(PCP_ERR_CUDA, "autotune copy");
                b->models[i]->geometryStale = true;
                b->models[i]->geomFromSnapshot = false;
            }
            if (rc) break;
            // a first run builds the graphs and warms up; the second is timed
            rc = batch_run(b, which, a);
            if (rc) break;
            for (int i : which)
                cudaMemcpy(b->models[i]->pos, keep[i], (size_t)b->models[i]->V * sizeof(double2),
                           cudaMemcpyDeviceToDevice);
            CK(cudaDeviceSynchronize());
            auto t0 = std::chrono::steady_clock::now();
            rc = batch_run(b, which, a);
            CK(cudaDeviceSynchronize());
            double ms = std::chrono::duration<double, std::milli>(
                std::chrono::steady_clock::now() - t0).count();
            row += (c ? ", " : "") + std::to_string(ms);
            if (ms < best) { best = ms; bestC = c; }
        }
        row += "], \"chosen_blocks\": " + std::to_string(cand[bestC]) + "}";
        rep += (firstClass ? "" : ", ") + row;
        firstClass = false;
        for (int i : which) {
            if (rc) break;
            rc = pcp_model_set_launch_shape(b->models[i], cand[bestC], cand[bestC]);
        }
    }
    rep += "], \"steps_per_trial\": " + std::to_string(steps) + "}";
    for (int i = 0; i < n; ++i) {
        if (keep[i]) {
            cudaMemcpy(b->models[i]->pos, keep[i], (size_t)b->models[i]->V * sizeof(double2),
                       cudaMemcpyDeviceToDevice);
            b->models[i]->geometryStale = true;
            b->models[i]->geomFromSnapshot = false;
            cudaFree(keep[i]);
        }
        b->models[i]->stream = saved[i];
    }
    if (rc) return rc;
    b->report = rep;
    if (shapes_out)
        for (int i = 0; i < n; ++i) {
            shapes_out[2 * i] = b->models[i]->ws.narrowBlocks;
            shapes_out[2 * i + 1] = b->models[i]->ws.forceBlocks;
        }
    return PCP_OK;
}

int pcp_batch_autotune_report(pcp_batch* b, char* buf, int cap, int* len_out) {
    if (!b) return fail(PCP_ERR_ARG, "null batch");
    if (len_out) *len_out = (int)b->report.size();
    if (buf && cap > 0) {
        int k = std::min(cap - 1, (int)b->report.size());
        std::memcpy(buf, b->report.data(), (size_t)k);
        buf[k] = 0;
    }
    return PCP_OK;
}

}  // extern "C"
