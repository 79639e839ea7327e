/*
 * pcp_oracle.c -- CPU oracle (TEST INFRASTRUCTURE) for the pyCudaPolygon hot
 * path.  Plain C11, FP64, compiled with -ffp-contract=off so that every
 * product and sum is rounded exactly as written (no fused multiply-adds).
 *
 * It restates the reference's algorithm, function by function; each block
 * cites the reference lines it follows (paths inside camdennis/pyCudaPolygon).
 * Atomic accumulations of the reference become sequential sums here, so
 * floating-point sums may differ from the GPU in the last bits; integer work
 * (cells, crossing decisions, packing, ordering, matching) is bit-exact.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this.
 *
 * Pinning: the testSaver neighbour known answer, getDf, the variable-n
 * projection, centres of mass and shoelace areas are checked against
 * fixtures generated from the reference's own Python (tests/golden/).
 * Parity unpinned for SHAKE and FIRE: the reference ships neither
 * src/shake.h nor src/FIRE.h, so those parts restate the call contract
 * (model.cpp:405-504, model.cu:576-636) and velocity-Verlet FIRE (Bitzek
 * et al., PRL 97, 170201, 2006), and nothing of the reference pins them.
 */
#include "pcp_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* small helpers                                                              */
/* ------------------------------------------------------------------------ */

static void* xcalloc(size_t n, size_t sz) {
    void* p = calloc(n ? n : 1, sz);
    if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    return p;
}
#define FREE(p) do { free(p); (p) = NULL; } while (0)

void orc_set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* wrap (kernels.cuh:115-119): minimum image into [-0.5, 0.5) */
double orc_wrap(double x) {
    double y = x + 1.5;
    y = y - floor(y);
    return y - 0.5;
}

/* The reference's `while` wrap loops (kernels.cuh:670-699).  They run at most
 * one pass for positions inside [0,1]; the cap only stops corrupt input
 * (|x| > 64 or Inf) from spinning, where the reference would not return. */
static double loop_wrap_unit(double x) {
    int it = 0;
    while (x < 0.0 && it < 64) { x += 1.0; ++it; }
    while (x >= 1.0 && it < 128) { x -= 1.0; ++it; }
    if (it >= 64 && isfinite(x) && (x < 0.0 || x >= 1.0)) x = x - floor(x);
    return x;
}

/* (int)floor(v * B) with the clamp of kernels.cuh:700-704.  NaN and -Inf go
 * to cell 0, +Inf to B-1, as CUDA's saturating float->int conversion does. */
static int cell_coord(double v, int B) {
    double f = floor(v * (double)B);
    if (!(f >= 0.0)) return 0;
    if (f >= (double)B) return B - 1;
    return (int)f;
}

/* h (kernels.cuh:139-146) */
double orc_h(const double pt1[2], const double pt2[2], const double sp[2]) {
    double r1x = orc_wrap(pt1[0] - sp[0]), r1y = orc_wrap(pt1[1] - sp[1]);
    double r2x = orc_wrap(pt2[0] - sp[0]), r2y = orc_wrap(pt2[1] - sp[1]);
    double dy = orc_wrap(r2y - r1y);
    return (r1x + r2x) * dy;
}

/* g12 (kernels.cuh:148-159) */
void orc_g12(const double pt1[2], const double pt2[2], const double sp[2],
             double g1[2], double g2[2]) {
    double r1x = orc_wrap(pt1[0] - sp[0]);
    double r2x = orc_wrap(pt2[0] - sp[0]);
    double dy = orc_wrap(pt2[1] - pt1[1]);
    g1[0] = dy; g1[1] = -(r1x + r2x);
    g2[0] = dy; g2[1] = (r1x + r2x);
}

/* getDf (kernels.cuh:161-222): 2x8 Jacobian of the crossing point
 * f = vi + u (vzi - vi) with respect to (vi, vzi, vj, vzj); df[col*2+row]. */
void orc_getDf(const double vi[2], const double vzi[2], const double vj[2],
               const double vzj[2], double df[16]) {
    double djx = orc_wrap(vzj[0] - vj[0]), djy = orc_wrap(vzj[1] - vj[1]);
    double dix = orc_wrap(vzi[0] - vi[0]), diy = orc_wrap(vzi[1] - vi[1]);
    double dijx = orc_wrap(vj[0] - vi[0]), dijy = orc_wrap(vj[1] - vi[1]);
    double w = djx * diy - djy * dix;
    double diN = dix * dix + diy * diy;
    double djN = djx * djx + djy * djy;
    int i;
    for (i = 0; i < 16; ++i) df[i] = 0.0;
    if (w * w < 1e-12 * diN * djN || diN < 1e-28 || djN < 1e-28) return;
    double k = djx * dijy - djy * dijx;
    double u = k / w;
    double dk[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    dk[0] = djy;           dk[1] = -djx;
    dk[4] = -dijy - djy;   dk[5] = djx + dijx;
    dk[6] = dijy;          dk[7] = -dijx;
    double dw[8];
    dw[0] = djy;  dw[1] = -djx;
    dw[2] = -djy; dw[3] = djx;
    dw[4] = -diy; dw[5] = dix;
    dw[6] = diy;  dw[7] = -dix;
    for (int a = 0; a < 2; ++a) {
        double dia = a == 0 ? dix : diy;
        for (int b = 0; b < 2; ++b) {
            for (int p = 0; p < 4; ++p) {
                double du = dk[p * 2 + b] / w - u * dw[p * 2 + b] / w;
                int col = 2 * p + b;
                df[col * 2 + a] += dia * du;
            }
            if (a == b) {
                df[b * 2 + a] += 1.0 - u;
                df[(2 + b) * 2 + a] += u;
            }
        }
    }
}

/* crossing predicate (kernels.cuh:778-791) */
int orc_cross(const double p[2], const double p2[2], const double q[2],
              const double q2[2], double* tt, double* uu, double* denom) {
    double rx = orc_wrap(p2[0] - p[0]);
    double ry = orc_wrap(p2[1] - p[1]);
    double sx = orc_wrap(q2[0] - q[0]);
    double sy = orc_wrap(q2[1] - q[1]);
    double gx = orc_wrap(q[0] - p[0]);
    double gy = orc_wrap(q[1] - p[1]);
    double d = rx * sy - ry * sx;
    *denom = d;
    if (fabs(d) < 1e-12) return 0;
    double t = (gx * sy - gy * sx) / d;
    double u = (gx * ry - gy * rx) / d;
    *tt = t; *uu = u;
    return (t > 0.0 && t < 1.0 && u > 0.0 && u < 1.0) ? 1 : 0;
}

/* ------------------------------------------------------------------------ */
/* model state (src/model.hpp:112-184)                                        */
/* ------------------------------------------------------------------------ */

struct orc_model {
    int modelType;
    int size, numPolygons;
    int boxSize;
    int maxNeighbors;
    int numIntersections;
    int lastShakeIters;
    int fireFirstShakeIters;   /* first SHAKE call of the last FIRE step (test use) */
    double stiffness, compressibility;
    double energy;
    double maxEdgeLength;
    double* positions;      /* 2V */
    double* force;          /* 2V */
    double* velocities;     /* 2V */
    double* positionsTMP;   /* 2V */
    double* positionsTMP2;  /* 2V */
    double* edgeLengths;    /* V */
    double* comParts;       /* 2V */
    double* areaParts;      /* V */
    double* constraints;    /* 6V */
    int* startIndices;      /* P+1 */
    double* areas;          /* P */
    double* targetAreas;    /* P */
    double* targetEdgeLengths; /* P */
    double* comX; double* comY; double* perimeters; /* P */
    double* constraintNormSq;  /* 3P */
    int* shapeId; int* next; int* prev;        /* V */
    int* cellLocation; int* neighborIndices;   /* V */
    int* countPerBox; int countPerBoxLen;      /* B*B */
    int* neighbors; uint8_t* inside; double* tuSlots; int* numNeighbors;
    int* shapeCounts;                          /* P */
    int capRecords;
    uint64_t* intersections; uint64_t* outersections;
    double* tu; double* ut;
};

static void ensure_records(orc_model* m, int n) {
    if (n <= m->capRecords) return;
    int cap = n + n / 2 + 16;
    m->intersections = (uint64_t*)realloc(m->intersections, (size_t)cap * 8);
    m->outersections = (uint64_t*)realloc(m->outersections, (size_t)cap * 8);
    m->tu = (double*)realloc(m->tu, (size_t)cap * 16);
    m->ut = (double*)realloc(m->ut, (size_t)cap * 16);
    if (!m->intersections || !m->outersections || !m->tu || !m->ut) abort();
    m->capRecords = cap;
}

static void alloc_vertex_arrays(orc_model* m) {
    size_t V = (size_t)m->size;
    FREE(m->positions); FREE(m->force); FREE(m->velocities);
    FREE(m->positionsTMP); FREE(m->positionsTMP2); FREE(m->edgeLengths);
    FREE(m->comParts); FREE(m->areaParts); FREE(m->constraints);
    m->positions = (double*)xcalloc(2 * V, 8);
    m->force = (double*)xcalloc(2 * V, 8);
    m->velocities = (double*)xcalloc(2 * V, 8);
    m->positionsTMP = (double*)xcalloc(2 * V, 8);
    m->positionsTMP2 = (double*)xcalloc(2 * V, 8);
    m->edgeLengths = (double*)xcalloc(V, 8);
    m->comParts = (double*)xcalloc(2 * V, 8);
    m->areaParts = (double*)xcalloc(V, 8);
    m->constraints = (double*)xcalloc(6 * V, 8);
}

/* Model::Model (model.cpp:60-101) */
orc_model* orc_create(int size) {
    orc_model* m = (orc_model*)xcalloc(1, sizeof(orc_model));
    m->size = size < 0 ? 0 : size;
    m->maxNeighbors = 100;
    m->boxSize = 1;
    alloc_vertex_arrays(m);
    return m;
}

void orc_destroy(orc_model* m) {
    if (!m) return;
    free(m->positions); free(m->force); free(m->velocities);
    free(m->positionsTMP); free(m->positionsTMP2); free(m->edgeLengths);
    free(m->comParts); free(m->areaParts); free(m->constraints);
    free(m->startIndices); free(m->areas); free(m->targetAreas);
    free(m->targetEdgeLengths); free(m->comX); free(m->comY);
    free(m->perimeters); free(m->constraintNormSq);
    free(m->shapeId); free(m->next); free(m->prev);
    free(m->cellLocation); free(m->neighborIndices); free(m->countPerBox);
    free(m->neighbors); free(m->inside); free(m->tuSlots); free(m->numNeighbors);
    free(m->shapeCounts);
    free(m->intersections); free(m->outersections); free(m->tu); free(m->ut);
    free(m);
}

/* ---- setters (model.cpp:513-636) ---- */
void orc_set_num_vertices(orc_model* m, int n) {
    m->size = n < 0 ? 0 : n;
    alloc_vertex_arrays(m);
}

int orc_set_positions(orc_model* m, const double* pos, int len) {
    if (len != 2 * m->size) return -1;     /* model.cpp:523-526 */
    memcpy(m->positions, pos, (size_t)len * 8);
    return 0;
}

void orc_set_forces(orc_model* m, const double* f, int len) {
    if (len > 2 * m->size) len = 2 * m->size;
    memcpy(m->force, f, (size_t)len * 8);
}

/* State setters for tests that start the oracle from another
 * implementation's FIRE state (no counterpart in the reference). */
void orc_set_velocities(orc_model* m, const double* v, int len) {
    if (len > 2 * m->size) len = 2 * m->size;
    memcpy(m->velocities, v, (size_t)len * 8);
}

void orc_set_energy(orc_model* m, double e) { m->energy = e; }

void orc_set_start_indices(orc_model* m, const int* si, int len) {
    int P = len - 1;
    if (P < 0) P = 0;
    m->numPolygons = P;
    FREE(m->startIndices); FREE(m->areas); FREE(m->targetAreas);
    FREE(m->targetEdgeLengths); FREE(m->comX); FREE(m->comY);
    FREE(m->perimeters); FREE(m->constraintNormSq); FREE(m->shapeCounts);
    m->startIndices = (int*)xcalloc((size_t)P + 1, sizeof(int));
    if (len > 0) memcpy(m->startIndices, si, (size_t)len * sizeof(int));
    m->areas = (double*)xcalloc(P, 8);
    m->targetAreas = (double*)xcalloc(P, 8);
    m->targetEdgeLengths = (double*)xcalloc(P, 8);
    m->comX = (double*)xcalloc(P, 8);
    m->comY = (double*)xcalloc(P, 8);
    m->perimeters = (double*)xcalloc(P, 8);
    m->constraintNormSq = (double*)xcalloc(3 * (size_t)P, 8);
    m->shapeCounts = (int*)xcalloc(P, sizeof(int));
}

void orc_set_target_areas(orc_model* m, const double* a, int len) {
    if (len > m->numPolygons) len = m->numPolygons;
    memcpy(m->targetAreas, a, (size_t)len * 8);
}
void orc_set_target_edge_lengths(orc_model* m, const double* l, int len) {
    if (len > m->numPolygons) len = m->numPolygons;
    memcpy(m->targetEdgeLengths, l, (size_t)len * 8);
}
/* Model::setMaxEdgeLength (model.cpp:513-516) */
void orc_set_max_edge_length(orc_model* m, double l) {
    m->boxSize = (int)floor(1.0 / l);
    m->maxEdgeLength = l;
}
void orc_set_model_enum(orc_model* m, int e) { m->modelType = e; }
void orc_set_stiffness(orc_model* m, double k) { m->stiffness = k; }
void orc_set_compressibility(orc_model* m, double c) { m->compressibility = c; }

/* Model::initializeNeighborCells (model.cpp:176-229): topology
 * (updateShapeIdKernel kernels.cuh:652-659, computeNextPrevKernel :127-135) */
void orc_initialize_neighbor_cells(orc_model* m) {
    int V = m->size, P = m->numPolygons;
    FREE(m->shapeId); FREE(m->next); FREE(m->prev);
    FREE(m->cellLocation); FREE(m->neighborIndices); FREE(m->numNeighbors);
    FREE(m->neighbors); FREE(m->inside); FREE(m->tuSlots);
    m->shapeId = (int*)xcalloc(V, sizeof(int));
    m->next = (int*)xcalloc(V, sizeof(int));
    m->prev = (int*)xcalloc(V, sizeof(int));
    m->cellLocation = (int*)xcalloc(V, sizeof(int));
    m->neighborIndices = (int*)xcalloc(V, sizeof(int));
    m->numNeighbors = (int*)xcalloc(V, sizeof(int));
    size_t slots = (size_t)V * (size_t)m->maxNeighbors;
    m->neighbors = (int*)xcalloc(slots, sizeof(int));
    m->inside = (uint8_t*)xcalloc(slots, 1);
    m->tuSlots = (double*)xcalloc(2 * slots, 8);
    for (int p = 0; p < P; ++p)
        for (int i = m->startIndices[p]; i < m->startIndices[p + 1]; ++i)
            if (i >= 0 && i < V) m->shapeId[i] = p;
    for (int i = 0; i < V; ++i) {
        int s = m->shapeId[i];
        int st = m->startIndices[s], en = m->startIndices[s + 1];
        m->next[i] = (i + 1 == en) ? st : i + 1;
        m->prev[i] = (i == st) ? en - 1 : i - 1;
    }
    m->numIntersections = 0;
}

/* ------------------------------------------------------------------------ */
/* geometry: updatePolygonGeometryKernel (kernels.cuh:295-333), the CUB      */
/* segmented sums and max (model.cu:113-152), normalizeKernel                */
/* (kernels.cuh:635-650), normalizeConstraintsKernel (kernels.cuh:335-345)   */
/* ------------------------------------------------------------------------ */
void orc_update_polygon_geometry(orc_model* m) {
    int V = m->size, P = m->numPolygons;
    const double* pos = m->positions;
    memset(m->constraintNormSq, 0, 3 * (size_t)P * 8);
    #pragma omp parallel for schedule(static)
    for (int p = 0; p < P; ++p) {
        for (int k = m->startIndices[p]; k < m->startIndices[p + 1]; ++k) {
            int nx = m->next[k], pv = m->prev[k];
            int startIndex = m->startIndices[m->shapeId[k]];
            for (int alpha = 0; alpha < 2; ++alpha) {
                int idx = 2 * k + alpha;
                double x1 = orc_wrap(pos[idx] - pos[startIndex * 2 + alpha]);
                double x4 = orc_wrap(pos[pv * 2 + 1 - alpha] - pos[nx * 2 + 1 - alpha]);
                double dxPrev = orc_wrap(pos[2 * k] - pos[pv * 2]);
                double dyPrev = orc_wrap(pos[2 * k + 1] - pos[pv * 2 + 1]);
                double dxNext = orc_wrap(pos[2 * k] - pos[nx * 2]);
                double dyNext = orc_wrap(pos[2 * k + 1] - pos[nx * 2 + 1]);
                m->comParts[k + V * alpha] = x1;
                double lenPrev = sqrt(dxPrev * dxPrev + dyPrev * dyPrev);
                double lenNext = sqrt(dxNext * dxNext + dyNext * dyNext);
                double areaComp = (2 * alpha - 1) * x4;
                double edge2Comp = alpha ? (dyNext + dyPrev) : (dxNext + dxPrev);
                double edgeComp = alpha ? (dyNext / lenNext) + (dyPrev / lenPrev)
                                        : (dxNext / lenNext) + (dxPrev / lenPrev);
                m->constraints[6 * k + alpha] = areaComp;
                m->constraints[6 * k + 2 + alpha] = edge2Comp;
                m->constraints[6 * k + 4 + alpha] = edgeComp;
                m->constraintNormSq[3 * p + 0] += areaComp * areaComp;
                m->constraintNormSq[3 * p + 1] += edge2Comp * edge2Comp;
                m->constraintNormSq[3 * p + 2] += edgeComp * edgeComp;
                if (alpha) continue;
                double dx = orc_wrap(pos[2 * nx] - pos[2 * k]);
                double dy = orc_wrap(pos[2 * nx + 1] - pos[2 * k + 1]);
                m->edgeLengths[k] = sqrt(dx * dx + dy * dy);
                double dy2 = orc_wrap(pos[nx * 2 + 1] - pos[idx + 1]);
                double x2 = orc_wrap(pos[nx * 2] - pos[startIndex * 2]);
                m->areaParts[k] = dy2 * (x2 + x1) / 2.0;
            }
        }
    }
    double mx = -DBL_MAX;
    for (int p = 0; p < P; ++p) {
        int st = m->startIndices[p], en = m->startIndices[p + 1];
        double a = 0.0, cx = 0.0, cy = 0.0, per = 0.0;
        for (int k = st; k < en; ++k) {
            a += m->areaParts[k];
            cx += m->comParts[k];
            cy += m->comParts[V + k];
            per += m->edgeLengths[k];
        }
        m->areas[p] = a;
        m->perimeters[p] = per;
        int n = en - st;
        double comx = cx / (double)n + pos[2 * st];
        comx -= floor(comx);
        double comy = cy / (double)n + pos[2 * st + 1];
        comy -= floor(comy);
        m->comX[p] = comx;
        m->comY[p] = comy;
    }
    for (int k = 0; k < V; ++k) if (m->edgeLengths[k] > mx) mx = m->edgeLengths[k];
    if (V > 0) m->maxEdgeLength = mx;
    #pragma omp parallel for schedule(static)
    for (int k = 0; k < V; ++k) {
        int p = m->shapeId[k];
        for (int c = 0; c < 3; ++c) {
            double ns = m->constraintNormSq[3 * p + c];
            if (ns > 0.0) {
                double r = sqrt(ns);
                m->constraints[6 * k + 2 * c + 0] /= r;
                m->constraints[6 * k + 2 * c + 1] /= r;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* cell list: updateNeighborCellsKernel (kernels.cuh:661-707), the stable    */
/* CUB sort of (cell, vertex) and lowerBoundKernel (model.cu:308-385)        */
/* ------------------------------------------------------------------------ */
int orc_midpoint_cell(const double* pos, const int* startIndices, const int* shapeId,
                      int size, int idx, int B) {
    int v2 = idx + 1;
    if (idx == size - 1 || shapeId[idx] != shapeId[idx + 1]) v2 = startIndices[shapeId[idx]];
    double x = pos[v2 * 2] - pos[idx * 2] + 0.5;
    double y = pos[v2 * 2 + 1] - pos[idx * 2 + 1] + 0.5;
    x = loop_wrap_unit(x);
    y = loop_wrap_unit(y);
    x -= 0.5; y -= 0.5;
    x /= 2.0; y /= 2.0;
    x += pos[idx * 2];
    y += pos[idx * 2 + 1];
    x = loop_wrap_unit(x);
    y = loop_wrap_unit(y);
    int ix = cell_coord(x, B), iy = cell_coord(y, B);
    return iy * B + ix;
}

void orc_update_neighbor_cells(orc_model* m) {
    int V = m->size, B = m->boxSize;
    if (B < 1) B = 1;
    int nb = B * B;
    for (int i = 0; i < V; ++i)
        m->cellLocation[i] = orc_midpoint_cell(m->positions, m->startIndices, m->shapeId, V, i, B);
    /* stable counting sort by cell == CUB radix SortPairs with iota values */
    if (m->countPerBoxLen != nb) {
        FREE(m->countPerBox);
        m->countPerBox = (int*)xcalloc(nb, sizeof(int));
        m->countPerBoxLen = nb;
    }
    int* cnt = (int*)xcalloc((size_t)nb + 1, sizeof(int));
    for (int i = 0; i < V; ++i) cnt[m->cellLocation[i] + 1]++;
    for (int c = 0; c < nb; ++c) cnt[c + 1] += cnt[c];
    for (int c = 0; c < nb; ++c) m->countPerBox[c] = cnt[c];  /* lower bound */
    for (int i = 0; i < V; ++i) m->neighborIndices[cnt[m->cellLocation[i]]++] = i;
    free(cnt);
}

/* ------------------------------------------------------------------------ */
/* narrow phase: updateNeighborsKernel (kernels.cuh:709-812) and the resize  */
/* and retry of Model::updateNeighbors (model.cpp:256-307)                   */
/* ------------------------------------------------------------------------ */
static int neighbors_pass(orc_model* m) {
    int V = m->size, B = m->boxSize, M = m->maxNeighbors;
    if (B < 1) B = 1;
    int boxCount = B * B;
    const double* pos = m->positions;
    int maxCount = 0;
    #pragma omp parallel for schedule(dynamic, 64) reduction(max:maxCount)
    for (int id1 = 0; id1 < V; ++id1) {
        int shape = m->shapeId[id1];
        int st = m->startIndices[shape + 1] - 1;
        int id2 = (id1 == st) ? m->startIndices[shape] : id1 + 1;
        double px = pos[2 * id1], py = pos[2 * id1 + 1];
        double rx = orc_wrap(pos[2 * id2] - px);
        double ry = orc_wrap(pos[2 * id2 + 1] - py);
        int box = m->cellLocation[id1];
        int bx = box % B, by = box / B;
        int count = 0;
        int processed[16], nproc = 0;
        for (int dx = -1; dx <= 1; dx++) {
            int nx = bx + dx;
            if (nx < 0) nx += B; else if (nx >= B) nx -= B;
            for (int dy = -1; dy <= 1; dy++) {
                int ny = by + dy;
                if (ny < 0) ny += B; else if (ny >= B) ny -= B;
                int newBox = ny * B + nx;
                int seen = 0;
                for (int b = 0; b < nproc; b++) if (processed[b] == newBox) { seen = 1; break; }
                if (seen) continue;
                if (nproc < 16) processed[nproc++] = newBox;
                if (newBox < 0 || newBox >= m->countPerBoxLen) continue;
                int si = m->countPerBox[newBox];
                int sf = (newBox + 1 < boxCount) ? m->countPerBox[newBox + 1] : V;
                for (int idx = si; idx < sf; idx++) {
                    int nid = m->neighborIndices[idx];
                    if (nid <= id1) continue;
                    int shape2 = m->shapeId[nid];
                    int st2 = m->startIndices[shape2 + 1] - 1;
                    int nid2 = (nid == st2) ? m->startIndices[shape2] : nid + 1;
                    if (nid == id1 || nid == id2 || nid2 == id1 || nid2 == id2) continue;
                    double qx = pos[2 * nid], qy = pos[2 * nid + 1];
                    double sx = orc_wrap(pos[2 * nid2] - qx);
                    double sy = orc_wrap(pos[2 * nid2 + 1] - qy);
                    double gx = orc_wrap(qx - px);
                    double gy = orc_wrap(qy - py);
                    double denom = rx * sy - ry * sx;
                    if (fabs(denom) < 1e-12) continue;
                    double tt = (gx * sy - gy * sx) / denom;
                    double uu = (gx * ry - gy * rx) / denom;
                    if (tt > 0.0 && tt < 1.0 && uu > 0.0 && uu < 1.0) {
                        if (count < M) {
                            size_t s = (size_t)id1 * M + count;
                            m->neighbors[s] = nid;
                            if (denom > 0) {
                                m->inside[s] = 1; m->tuSlots[2 * s] = tt; m->tuSlots[2 * s + 1] = uu;
                            } else {
                                m->inside[s] = 0; m->tuSlots[2 * s] = uu; m->tuSlots[2 * s + 1] = tt;
                            }
                        }
                        count++;
                    }
                }
            }
        }
        m->numNeighbors[id1] = count;
        if (count > maxCount) maxCount = count;
    }
    return maxCount;
}

int orc_update_neighbors(orc_model* m) {
    int newMax = neighbors_pass(m);
    if (newMax > m->maxNeighbors) {
        int nm = m->maxNeighbors * 2 + 1;
        if (newMax > nm) nm = newMax;
        m->maxNeighbors = nm;
        size_t slots = (size_t)m->size * (size_t)nm;
        FREE(m->neighbors); FREE(m->inside); FREE(m->tuSlots);
        m->neighbors = (int*)xcalloc(slots, sizeof(int));
        m->inside = (uint8_t*)xcalloc(slots, 1);
        m->tuSlots = (double*)xcalloc(2 * slots, 8);
        newMax = neighbors_pass(m);
    }
    return newMax;
}

/* ------------------------------------------------------------------------ */
/* contact records: updateValidAndCountsKernel (kernels.cuh:814-836), the    */
/* exclusive scan (model.cu:413-450), updateCompactedIntersectionsKernel     */
/* (kernels.cuh:838-877), sortKeysCUDA (model.cu:50-75), gathers, and        */
/* updateOutersectionsKernel (kernels.cuh:981-1065), as orchestrated by      */
/* Model::updateOutersections (model.cpp:351-361)                            */
/* ------------------------------------------------------------------------ */

/* stable LSD sort of keys by bits [0, endBit), returning the permutation */
static void stable_sort_bits(uint64_t* keys, uint32_t* perm, int n, int endBit) {
    uint64_t* k2 = (uint64_t*)xcalloc(n, 8);
    uint32_t* p2 = (uint32_t*)xcalloc(n, 4);
    int* cnt = (int*)xcalloc(65537, sizeof(int));
    for (int i = 0; i < n; ++i) perm[i] = (uint32_t)i;
    for (int shift = 0; shift < endBit; shift += 16) {
        int bits = endBit - shift < 16 ? endBit - shift : 16;
        uint64_t mask = (bits == 16) ? 0xFFFFu : ((1u << bits) - 1u);
        memset(cnt, 0, 65537 * sizeof(int));
        for (int i = 0; i < n; ++i) cnt[((keys[i] >> shift) & mask) + 1]++;
        for (int c = 0; c < 65536; ++c) cnt[c + 1] += cnt[c];
        for (int i = 0; i < n; ++i) {
            int d = cnt[(keys[i] >> shift) & mask]++;
            k2[d] = keys[i]; p2[d] = perm[i];
        }
        memcpy(keys, k2, (size_t)n * 8);
        memcpy(perm, p2, (size_t)n * 4);
    }
    free(k2); free(p2); free(cnt);
}

/* updateOutersectionsKernel (kernels.cuh:981-1065) for one record */
static void outersection_one(const uint64_t* inter, const double* tu, double* ut,
                             const int* startIndices, int I, uint64_t* outer, int idx) {
    uint64_t it = inter[idx];
    int sj = (int)((it >> 48) & 0xFFFF);
    int si = (int)((it >> 32) & 0xFFFF);
    int i = (int)((it >> 16) & 0xFFFF);
    int ni = startIndices[si + 1] - startIndices[si];
    uint64_t sij = ((uint64_t)si << 48) | ((uint64_t)sj << 32);
    float tVal = (float)tu[2 * idx + 1];
    int start = 0, end = I - 1;
    while (end > start) {
        int mid = (end + start) / 2;
        if (inter[mid] < sij) start = mid + 1; else end = mid;
    }
    uint64_t ub = ((uint64_t)si << 48) | ((uint64_t)(sj + 1) << 32);
    int bestDist = -1; float bestU = FLT_MAX; int bestIdx = -1;
    float fallbackU = FLT_MAX; int fallbackIdx = -1;
    int k = start;
    while (k < I && inter[k] < ub) {
        uint64_t kk = inter[k];
        int l = (int)(kk & 0xFFFF);
        float uVal = (float)tu[2 * k];
        int d = (l - i + ni) % ni;
        if (l == i && tVal >= uVal) { k++; continue; }
        if (bestDist == -1 || d < bestDist) {
            bestDist = d; bestU = FLT_MAX; bestIdx = -1; fallbackU = FLT_MAX; fallbackIdx = -1;
        }
        if (d == bestDist) {
            if (d == 0) {
                if (uVal >= tVal && uVal < bestU) { bestU = uVal; bestIdx = k; }
                if (uVal < fallbackU) { fallbackU = uVal; fallbackIdx = k; }
            } else {
                if (uVal < bestU) { bestU = uVal; bestIdx = k; }
            }
        }
        k++;
    }
    int player = (bestIdx != -1) ? bestIdx : fallbackIdx;
    if (player == -1) {
        outer[idx] = inter[idx];
        ut[2 * idx] = tu[2 * idx]; ut[2 * idx + 1] = tu[2 * idx + 1];
        return;
    }
    outer[idx] = inter[player];
    ut[2 * idx] = tu[2 * player]; ut[2 * idx + 1] = tu[2 * player + 1];
}

void orc_update_outersections(orc_model* m) {
    int V = m->size, M = m->maxNeighbors, P = m->numPolygons;
    /* valid mask, per-shape counts and compaction in slot order */
    memset(m->shapeCounts, 0, (size_t)P * sizeof(int));
    int I = 0;
    for (int n1 = 0; n1 < V; ++n1) {
        int c = m->numNeighbors[n1] < M ? m->numNeighbors[n1] : M;
        I += c;
    }
    ensure_records(m, I);
    int out = 0;
    for (int n1 = 0; n1 < V; ++n1) {
        int c = m->numNeighbors[n1] < M ? m->numNeighbors[n1] : M;
        for (int i = 0; i < c; ++i) {
            size_t s = (size_t)n1 * M + i;
            int n2 = m->neighbors[s];
            int s1 = m->shapeId[n1], s2 = m->shapeId[n2];
            int ins = m->inside[s];
            m->shapeCounts[ins ? s2 : s1]++;
            int l1 = n1 - m->startIndices[s1];
            int l2 = n2 - m->startIndices[s2];
            float tVal = (float)m->tuSlots[2 * s];
            float uVal = (float)m->tuSlots[2 * s + 1];
            uint64_t packed;
            if (ins)
                packed = ((uint64_t)(uint16_t)s1 << 48) | ((uint64_t)(uint16_t)s2 << 32) |
                         ((uint64_t)(uint16_t)l2 << 16) | (uint64_t)(uint16_t)l1;
            else
                packed = ((uint64_t)(uint16_t)s2 << 48) | ((uint64_t)(uint16_t)s1 << 32) |
                         ((uint64_t)(uint16_t)l1 << 16) | (uint64_t)(uint16_t)l2;
            m->intersections[out] = packed;
            m->tu[2 * out] = (double)tVal;
            m->tu[2 * out + 1] = (double)uVal;
            out++;
        }
    }
    m->numIntersections = I;
    if (I == 0) return;
    uint32_t* perm = (uint32_t*)xcalloc(I, 4);
    double* tuTMP = (double*)xcalloc(2 * (size_t)I, 8);
    double* utTMP = (double*)xcalloc(2 * (size_t)I, 8);
    uint64_t* outTMP = (uint64_t*)xcalloc(I, 8);
    /* sortKeys(0, 64) + gather tu -> tuTMP (model.cpp:354-355) */
    stable_sort_bits(m->intersections, perm, I, 64);
    for (int i = 0; i < I; ++i) {
        tuTMP[2 * i] = m->tu[2 * perm[i]];
        tuTMP[2 * i + 1] = m->tu[2 * perm[i] + 1];
    }
    #pragma omp parallel for schedule(static)
    for (int idx = 0; idx < I; ++idx)
        outersection_one(m->intersections, tuTMP, utTMP, m->startIndices, I, outTMP, idx);
    /* sortKeys(0, 48) + gathers (model.cpp:357-360) */
    stable_sort_bits(m->intersections, perm, I, 48);
    for (int i = 0; i < I; ++i) {
        uint32_t p = perm[i];
        m->tu[2 * i] = tuTMP[2 * p]; m->tu[2 * i + 1] = tuTMP[2 * p + 1];
        m->ut[2 * i] = utTMP[2 * p]; m->ut[2 * i + 1] = utTMP[2 * p + 1];
        m->outersections[i] = outTMP[p];
    }
    free(perm); free(tuTMP); free(utTMP); free(outTMP);
}

/* ------------------------------------------------------------------------ */
/* overlap energy and force                                                  */
/* ------------------------------------------------------------------------ */
static inline void add_force(double* F, int v, double fx, double fy) {
    F[2 * v] += fx; F[2 * v + 1] += fy;
}

/* updateForceEnergyExteriorKernel (kernels.cuh:1067-1273) for one record;
 * returns the record's un-halved energy */
static double exterior_one(const orc_model* m, int idx, double* F) {
    uint64_t inter = m->intersections[idx], outer = m->outersections[idx];
    if (inter == outer) return 0.0;
    const double* pos = m->positions;
    int s1 = (int)((inter >> 32) & 0xFFFF);
    int s2 = (int)((inter >> 48) & 0xFFFF);
    int iLoc = (int)((inter >> 16) & 0xFFFF);
    int jLoc = (int)(inter & 0xFFFF);
    int kLoc = (int)((outer >> 16) & 0xFFFF);
    int lLoc = (int)(outer & 0xFFFF);
    int start1 = m->startIndices[s1], start2 = m->startIndices[s2];
    int i = start1 + iLoc, j = start2 + jLoc, k = start2 + kLoc, l = start1 + lLoc;
    int V = m->size;
    if (i >= V || j >= V || k >= V || l >= V) return 0.0;  /* out-of-range partner */
    int zi = m->next[i], zj = m->next[j], zk = m->next[k], zl = m->next[l];
    const double *pi = pos + 2 * i, *pj = pos + 2 * j, *pk = pos + 2 * k, *pl = pos + 2 * l;
    const double *pzi = pos + 2 * zi, *pzj = pos + 2 * zj, *pzk = pos + 2 * zk, *pzl = pos + 2 * zl;
    double r1[2] = {orc_wrap(pzi[0] - pi[0]), orc_wrap(pzi[1] - pi[1])};
    double r2[2] = {orc_wrap(pzk[0] - pk[0]), orc_wrap(pzk[1] - pk[1])};
    double t1 = m->tu[2 * idx + 1];
    double t2 = m->ut[2 * idx + 1];
    double fij[2] = {orc_wrap(pi[0] + t1 * r1[0]), orc_wrap(pi[1] + t1 * r1[1])};
    double fkl[2] = {orc_wrap(pk[0] + t2 * r2[0]), orc_wrap(pk[1] + t2 * r2[1])};
    double sp[2] = {fij[0], fij[1]};
    double e = 0.0;
    double df1[16], df2[16];
    if (i == l) {
        e += orc_h(fij, fkl, sp);
        double g1[2], g2[2];
        orc_g12(fij, fkl, sp, g1, g2);
        orc_getDf(pi, pzi, pj, pzj, df1);
        orc_getDf(pk, pzk, pi, pzi, df2);
        const int va[4] = {i, zi, j, zj};
        for (int c = 0; c < 4; ++c) {
            double ix = g1[0] * df1[(2 * c) * 2 + 0] + g1[1] * df1[(2 * c) * 2 + 1];
            double iy = g1[0] * df1[(2 * c + 1) * 2 + 0] + g1[1] * df1[(2 * c + 1) * 2 + 1];
            add_force(F, va[c], -ix, -iy);
        }
        const int vb[4] = {k, zk, i, zi};
        for (int c = 0; c < 4; ++c) {
            double ix = g2[0] * df2[(2 * c) * 2 + 0] + g2[1] * df2[(2 * c) * 2 + 1];
            double iy = g2[0] * df2[(2 * c + 1) * 2 + 0] + g2[1] * df2[(2 * c + 1) * 2 + 1];
            add_force(F, vb[c], -ix, -iy);
        }
    } else {
        e += orc_h(fij, pzi, sp);
        e += orc_h(pl, fkl, sp);
        double g1a[2], g2a[2], g1b[2], g2b[2];
        orc_g12(fij, pzi, sp, g1a, g2a);
        orc_getDf(pi, pzi, pj, pzj, df1);
        orc_getDf(pk, pzk, pl, pzl, df2);
        /* i, j, zj from dfij with g1a; zi gets dfij(g1a) + g2a */
        {
            double ix = g1a[0] * df1[0] + g1a[1] * df1[1];
            double iy = g1a[0] * df1[2] + g1a[1] * df1[3];
            add_force(F, i, -ix, -iy);
        }
        {
            double ix = g1a[0] * df1[8] + g1a[1] * df1[9];
            double iy = g1a[0] * df1[10] + g1a[1] * df1[11];
            add_force(F, j, -ix, -iy);
        }
        {
            double ix = g1a[0] * df1[4] + g1a[1] * df1[5] + g2a[0];
            double iy = g1a[0] * df1[6] + g1a[1] * df1[7] + g2a[1];
            add_force(F, zi, -ix, -iy);
        }
        {
            double ix = g1a[0] * df1[12] + g1a[1] * df1[13];
            double iy = g1a[0] * df1[14] + g1a[1] * df1[15];
            add_force(F, zj, -ix, -iy);
        }
        orc_g12(pl, fkl, sp, g1b, g2b);
        {
            double ix = g1b[0] + (g2b[0] * df2[8] + g2b[1] * df2[9]);
            double iy = g1b[1] + (g2b[0] * df2[10] + g2b[1] * df2[11]);
            add_force(F, l, -ix, -iy);
        }
        {
            double ix = g2b[0] * df2[0] + g2b[1] * df2[1];
            double iy = g2b[0] * df2[2] + g2b[1] * df2[3];
            add_force(F, k, -ix, -iy);
        }
        {
            double ix = g2b[0] * df2[12] + g2b[1] * df2[13];
            double iy = g2b[0] * df2[14] + g2b[1] * df2[15];
            add_force(F, zl, -ix, -iy);
        }
        {
            double ix = g2b[0] * df2[4] + g2b[1] * df2[5];
            double iy = g2b[0] * df2[6] + g2b[1] * df2[7];
            add_force(F, zk, -ix, -iy);
        }
    }
    return e;
}

/* updateForceEnergyEdgeKernel (kernels.cuh:1284-1335) */
static void edge_energy(orc_model* m) {
    const double* pos = m->positions;
    for (int mm = 0; mm < m->size; ++mm) {
        int prv = m->prev[mm], nxt = m->next[mm];
        double l0 = m->targetEdgeLengths[m->shapeId[mm]];
        double l0prv = m->targetEdgeLengths[m->shapeId[prv]];
        double l = m->edgeLengths[mm], prvl = m->edgeLengths[prv];
        double ax = pos[2 * mm] - pos[2 * nxt] + 1.5, ay = pos[2 * mm + 1] - pos[2 * nxt + 1] + 1.5;
        double bx = pos[2 * prv] - pos[2 * mm] + 1.5, by = pos[2 * prv + 1] - pos[2 * mm + 1] + 1.5;
        int it = 0;
        while (ax >= 1.0 && it++ < 64) ax -= 1.0;
        it = 0; while (ay >= 1.0 && it++ < 64) ay -= 1.0;
        it = 0; while (bx >= 1.0 && it++ < 64) bx -= 1.0;
        it = 0; while (by >= 1.0 && it++ < 64) by -= 1.0;
        ax -= 0.5; ay -= 0.5; bx -= 0.5; by -= 0.5;
        double c1 = (l > 1e-14) ? (1.0 - l0 / l) : 0.0;
        double c2 = (prvl > 1e-14) ? (1.0 - l0prv / prvl) : 0.0;
        double le = m->stiffness * (l - l0) * (l - l0) / 2.0;
        double fx = -(c1 * ax - c2 * bx) * m->stiffness;
        double fy = -(c1 * ay - c2 * by) * m->stiffness;
        if (le != 0.0) m->energy += le;
        if (fx != 0.0 || fy != 0.0) add_force(m->force, mm, fx, fy);
    }
}

/* updateForceEnergyAreaKernel (kernels.cuh:1337-1352) */
static void area_energy(orc_model* m) {
    const double* pos = m->positions;
    for (int mm = 0; mm < m->size; ++mm) {
        int s = m->shapeId[mm];
        double A = m->areas[s], A0 = m->targetAreas[s];
        if (A0 < 1e-14) continue;
        double coeff = 0.5 * m->compressibility * (A - A0);
        double fx = -coeff * orc_wrap(pos[2 * m->next[mm] + 1] - pos[2 * m->prev[mm] + 1]);
        double fy = -coeff * orc_wrap(pos[2 * m->prev[mm]] - pos[2 * m->next[mm]]);
        add_force(m->force, mm, fx, fy);
        if (m->startIndices[s] == mm)
            m->energy += m->compressibility * (A - A0) * (A - A0) / 2.0;
    }
}

/* overlap part: exterior + updateShapeRangesKernel + interior
 * (model.cpp:369-371; kernels.cuh:1275-1282, 1354-1424) */
static void overlap_energy(orc_model* m) {
    int I = m->numIntersections, P = m->numPolygons, V = m->size;
    double eExt = 0.0;
    for (int idx = 0; idx < I; ++idx) eExt += exterior_one(m, idx, m->force);
    m->energy += eExt / 2.0;
    int* shapeStart = (int*)xcalloc(P, sizeof(int));
    int* shapeEnd = (int*)xcalloc(P, sizeof(int));
    for (int p = 0; p < P; ++p) { shapeStart[p] = I; shapeEnd[p] = -1; }
    for (int idx = 0; idx < I; ++idx) {
        int s = (int)((m->intersections[idx] >> 32) & 0xFFFF);
        if (s >= P) continue;
        if (idx < shapeStart[s]) shapeStart[s] = idx;
        if (idx > shapeEnd[s]) shapeEnd[s] = idx;
    }
    if (I == 0) { free(shapeStart); free(shapeEnd); return; }
    const double* pos = m->positions;
    double eInt = 0.0;
    for (int mm = 0; mm < V; ++mm) {
        int s = m->shapeId[mm];
        int a = shapeStart[s], b = shapeEnd[s];
        if (a > b) continue;
        int n = m->startIndices[s + 1] - m->startIndices[s];
        int mLoc = mm - m->startIndices[s];
        const double* pm = pos + 2 * mm;
        int nxt = m->next[mm];
        const double* pn = pos + 2 * nxt;
        double le = 0.0, fmx = 0.0, fmy = 0.0, fnx = 0.0, fny = 0.0;
        for (int k = a; k <= b; ++k) {
            uint64_t inter = m->intersections[k], outer = m->outersections[k];
            if (inter == outer) continue;
            int si = (int)((inter >> 32) & 0xFFFF);
            int iLoc = (int)((inter >> 16) & 0xFFFF);
            int lLoc = (int)(outer & 0xFFFF);
            int iDist = (mLoc - iLoc + n) % n;
            int lDist = (lLoc - iLoc + n) % n;
            if (iDist > 0 && iDist < lDist) {
                int ik = m->startIndices[si] + iLoc;
                const double* pik = pos + 2 * ik;
                const double* pzik = pos + 2 * m->next[ik];
                double rik[2] = {orc_wrap(pzik[0] - pik[0]), orc_wrap(pzik[1] - pik[1])};
                double t1 = m->tu[2 * k + 1];
                double sp[2] = {orc_wrap(pik[0] + t1 * rik[0]), orc_wrap(pik[1] + t1 * rik[1])};
                le += orc_h(pm, pn, sp);
                double g1[2], g2[2];
                orc_g12(pm, pn, sp, g1, g2);
                fmx -= g1[0]; fmy -= g1[1];
                fnx -= g2[0]; fny -= g2[1];
            }
        }
        if (le != 0.0) eInt += le / 2.0;
        if (fmx != 0.0 || fmy != 0.0) add_force(m->force, mm, fmx, fmy);
        if (fnx != 0.0 || fny != 0.0) add_force(m->force, nxt, fnx, fny);
    }
    m->energy += eInt;
    free(shapeStart); free(shapeEnd);
}

/* Model::updateForceEnergy (model.cpp:363-395) */
void orc_update_force_energy(orc_model* m) {
    memset(m->force, 0, 2 * (size_t)m->size * 8);
    m->energy = 0.0;
    switch (m->modelType) {
        case ORC_NORMAL: overlap_energy(m); break;
        case ORC_SOFT_BODY: edge_energy(m); area_energy(m); break;
        case ORC_EDGE_ONLY: edge_energy(m); break;
        case ORC_AREA_ONLY: area_energy(m); break;
        case ORC_HYBRID: overlap_energy(m); edge_energy(m); area_energy(m); break;
        default: break;
    }
}

/* ------------------------------------------------------------------------ */
/* projectForce (model.cu:165-206; kernels.cuh:389-523).  The reference      */
/* builds the 2n x n edge-length Jacobian per polygon, takes an orthonormal  */
/* basis U of its columns (cuSOLVER gesvda), Gram-Schmidts the normalised    */
/* area gradient against U, normalises it (guard 1e-14) and removes both     */
/* from the force.  The result depends only on the column span, so this      */
/* restatement takes the basis from a Householder QR; it also accepts a      */
/* different n per polygon (the reference's Python twin does, the CUDA path  */
/* assumes one n, model.cpp:570).                                            */
/* ------------------------------------------------------------------------ */
static void project_polygon(const orc_model* m, int p, double* A, double* Q,
                            double* v, double* f) {
    int st = m->startIndices[p], n = m->startIndices[p + 1] - st;
    int rows = 2 * n, cols = n;
    const double* pos = m->positions;
    /* buildEdgeGradMatrixKernel (kernels.cuh:389-406); column-major rows x n */
    memset(A, 0, (size_t)rows * cols * 8);
    for (int kl = 0; kl < n; ++kl) {
        int k = st + kl, nk = m->next[k];
        double dx = orc_wrap(pos[2 * nk] - pos[2 * k]);
        double dy = orc_wrap(pos[2 * nk + 1] - pos[2 * k + 1]);
        double len = sqrt(dx * dx + dy * dy);
        if (len < 1e-14) continue;
        double tx = dx / len, ty = dy / len;
        double* col = A + (size_t)kl * rows;
        col[2 * kl] = -tx; col[2 * kl + 1] = -ty;
        col[2 * ((kl + 1) % n)] = tx; col[2 * ((kl + 1) % n) + 1] = ty;
    }
    /* Householder QR; Q holds the first `cols` columns of the orthogonal factor */
    double* R = A;
    double* vs = (double*)xcalloc((size_t)rows * cols, 8);
    double* betas = (double*)xcalloc(cols, 8);
    int rank = 0;
    for (int c = 0; c < cols; ++c) {
        double nrm = 0.0;
        for (int r = c; r < rows; ++r) nrm += R[(size_t)c * rows + r] * R[(size_t)c * rows + r];
        nrm = sqrt(nrm);
        double* hv = vs + (size_t)c * rows;
        memset(hv, 0, (size_t)rows * 8);
        if (nrm == 0.0) { betas[c] = 0.0; continue; }
        double x0 = R[(size_t)c * rows + c];
        double alpha = x0 > 0 ? -nrm : nrm;
        for (int r = c; r < rows; ++r) hv[r] = R[(size_t)c * rows + r];
        hv[c] -= alpha;
        double vn = 0.0;
        for (int r = c; r < rows; ++r) vn += hv[r] * hv[r];
        betas[c] = vn > 0 ? 2.0 / vn : 0.0;
        for (int cc = c; cc < cols; ++cc) {
            double* col = R + (size_t)cc * rows;
            double d = 0.0;
            for (int r = c; r < rows; ++r) d += hv[r] * col[r];
            d *= betas[c];
            for (int r = c; r < rows; ++r) col[r] -= d * hv[r];
        }
        rank++;
    }
    for (int c = 0; c < cols; ++c) {
        double* q = Q + (size_t)c * rows;
        memset(q, 0, (size_t)rows * 8);
        q[c] = 1.0;
        for (int h = cols - 1; h >= 0; --h) {
            double* hv = vs + (size_t)h * rows;
            if (betas[h] == 0.0) continue;
            double d = 0.0;
            for (int r = h; r < rows; ++r) d += hv[r] * q[r];
            d *= betas[h];
            for (int r = h; r < rows; ++r) q[r] -= d * hv[r];
        }
    }
    free(vs); free(betas);
    (void)rank;
    /* gramSchmidtAreaKernel (kernels.cuh:411-467) */
    for (int i = 0; i < rows; ++i) v[i] = m->constraints[6 * (st + i / 2) + (i % 2)];
    for (int j = 0; j < cols; ++j) {
        const double* q = Q + (size_t)j * rows;
        double dot = 0.0;
        for (int i = 0; i < rows; ++i) dot += q[i] * v[i];
        for (int i = 0; i < rows; ++i) v[i] -= dot * q[i];
    }
    double mag = 0.0;
    for (int i = 0; i < rows; ++i) mag += v[i] * v[i];
    mag = sqrt(mag);
    double inv = (mag > 1e-14) ? 1.0 / mag : 0.0;
    for (int i = 0; i < rows; ++i) v[i] *= inv;
    /* forceProjectFullKernel (kernels.cuh:471-523) */
    for (int i = 0; i < rows; ++i) f[i] = m->force[2 * st + i];
    for (int j = 0; j < cols; ++j) {
        const double* q = Q + (size_t)j * rows;
        double dot = 0.0;
        for (int i = 0; i < rows; ++i) dot += q[i] * f[i];
        for (int i = 0; i < rows; ++i) f[i] -= dot * q[i];
    }
    double dot = 0.0;
    for (int i = 0; i < rows; ++i) dot += v[i] * f[i];
    for (int i = 0; i < rows; ++i) f[i] -= dot * v[i];
    for (int i = 0; i < rows; ++i) m->force[2 * st + i] = f[i];
}

void orc_project_force(orc_model* m) {
    int P = m->numPolygons;
    int nmax = 0;
    for (int p = 0; p < P; ++p) {
        int n = m->startIndices[p + 1] - m->startIndices[p];
        if (n > nmax) nmax = n;
    }
    if (nmax == 0) return;
    #pragma omp parallel
    {
        double* A = (double*)xcalloc((size_t)2 * nmax * nmax, 8);
        double* Q = (double*)xcalloc((size_t)2 * nmax * nmax, 8);
        double* v = (double*)xcalloc((size_t)2 * nmax, 8);
        double* f = (double*)xcalloc((size_t)2 * nmax, 8);
        #pragma omp for schedule(dynamic, 16)
        for (int p = 0; p < P; ++p) project_polygon(m, p, A, Q, v, f);
        free(A); free(Q); free(v); free(f);
    }
}

/* ------------------------------------------------------------------------ */
/* SHAKE (restated; the reference's src/shake.h is absent).  Launch contract */
/* model.cu:616-636: one polygon per block, constraints = n edge lengths     */
/* (scalar target per polygon) + 1 area, an (n+1)x(n+1) matrix per polygon,  */
/* returns the largest iteration count over polygons; failure = count >=     */
/* maxIter.  Restatement (matrix SHAKE, Newton in the multipliers, the       */
/* correction solved in single precision):                                   */
/*   s_k = (|e_k|^2 - L^2)/2, e_k = u_{k+1} - u_k;  s_A = A - A0;             */
/*   u_k = wrap(x_k - x_0), local coordinates taken once at the start;       */
/*   stop when max(max_k |s_k|/L, |s_A|) < tol;                               */
/*   x <- x + G_ref^T l,  (G(x) G_ref^T) l = -s,                              */
/* G_ref the constraint gradients where SHAKE starts (rows -+e_k, grad A).    */
/* The matrix is a cyclic tridiagonal block bordered by the area row and      */
/* column; it is formed in float and solved by parallel cyclic reduction      */
/* (after a Sherman-Morrison split of the cyclic corners), exactly the steps  */
/* of the CUDA kernel, row by row.  Residuals and updates are double.        */
/* ------------------------------------------------------------------------ */
static int pow2_at_least(int n) { int N = 4; while (N < n) N <<= 1; return N; }

/* parallel cyclic reduction, sequential form; arrays [2][N], 3 rhs */
static void pcr3_f(float* pa, float* pb, float* pc, float* p0, float* p1, float* p2, int N) {
    int cur = 0;
    for (int d = 1; d < N; d <<= 1) {
        int nx = cur ^ 1;
        float *a = pa + cur * N, *b = pb + cur * N, *c = pc + cur * N;
        float *r0 = p0 + cur * N, *r1 = p1 + cur * N, *r2 = p2 + cur * N;
        float *a2 = pa + nx * N, *b2 = pb + nx * N, *c2 = pc + nx * N;
        float *s0 = p0 + nx * N, *s1 = p1 + nx * N, *s2 = p2 + nx * N;
        for (int i = 0; i < N; ++i) {
            int im = i - d, ip = i + d;
            float na = 0.f, nc = 0.f;
            float nb = b[i], n0 = r0[i], n1 = r1[i], n2 = r2[i];
            if (im >= 0) {
                float k1 = a[i] / b[im];
                na = -k1 * a[im];
                nb -= k1 * c[im];
                n0 -= k1 * r0[im]; n1 -= k1 * r1[im]; n2 -= k1 * r2[im];
            }
            if (ip < N) {
                float k2 = c[i] / b[ip];
                nc = -k2 * c[ip];
                nb -= k2 * a[ip];
                n0 -= k2 * r0[ip]; n1 -= k2 * r1[ip]; n2 -= k2 * r2[ip];
            }
            a2[i] = na; b2[i] = nb; c2[i] = nc; s0[i] = n0; s1[i] = n1; s2[i] = n2;
        }
        cur = nx;
    }
    float *b = pb + cur * N, *r0 = p0 + cur * N, *r1 = p1 + cur * N, *r2 = p2 + cur * N;
    for (int i = 0; i < N; ++i) {
        float ib = 1.0f / b[i];
        float x0 = r0[i] * ib, x1 = r1[i] * ib, x2 = r2[i] * ib;
        p0[i] = x0; p1[i] = x1; p2[i] = x2;
    }
}

static int shake_polygon(orc_model* m, int p, int maxIter, double tol, double* work) {
    int st = m->startIndices[p], n = m->startIndices[p + 1] - st;
    if (n < 3) return 0;
    double L = m->targetEdgeLengths[p], A0 = m->targetAreas[p];
    double invL = L > 0.0 ? 1.0 / L : 1.0;
    int N = pow2_at_least(n);
    double* x = work;              /* 2n */
    double* r = x + 2 * n;         /* 2n reference edges */
    double* ar = r + 2 * n;        /* 2n reference area gradient */
    float* f = (float*)(ar + 2 * n);
    float *rf = f, *arf = rf + 2 * n, *ef = arf + 2 * n, *acf = ef + 2 * n;
    float *vr = acf + 2 * n, *lam = vr + n;
    float *pa = lam + n, *pb = pa + 2 * N, *pc = pb + 2 * N;
    float *p0 = pc + 2 * N, *p1 = p0 + 2 * N, *p2 = p1 + 2 * N;
    /* local coordinates u_k = wrap(x_k - x_0): the iterations need no
       minimum images (a polygon spans far less than half the box) */
    const double ox = m->positions[2 * st], oy = m->positions[2 * st + 1];
    for (int k = 0; k < n; ++k) {
        x[2 * k] = orc_wrap(m->positions[2 * (st + k)] - ox);
        x[2 * k + 1] = orc_wrap(m->positions[2 * (st + k) + 1] - oy);
    }
    for (int k = 0; k < n; ++k) {
        int kn = (k + 1) % n, kp = (k + n - 1) % n;
        r[2 * k] = x[2 * kn] - x[2 * k];
        r[2 * k + 1] = x[2 * kn + 1] - x[2 * k + 1];
        ar[2 * k] = 0.5 * (x[2 * kn + 1] - x[2 * kp + 1]);
        ar[2 * k + 1] = 0.5 * (x[2 * kp] - x[2 * kn]);
        rf[2 * k] = (float)r[2 * k]; rf[2 * k + 1] = (float)r[2 * k + 1];
        arf[2 * k] = (float)ar[2 * k]; arf[2 * k + 1] = (float)ar[2 * k + 1];
    }
    int it = 0;
    for (; it < maxIter; ++it) {
        double worst = 0.0, area = 0.0;
        int nonfinite = 0;
        for (int k = 0; k < n; ++k) {
            int kn = (k + 1) % n, kp = (k + n - 1) % n;
            double ex = x[2 * kn] - x[2 * k], ey = x[2 * kn + 1] - x[2 * k + 1];
            double sk = 0.5 * (ex * ex + ey * ey - L * L);
            double q = fabs(sk) * invL;
            if (!(q <= worst)) { worst = q; if (!isfinite(q)) nonfinite = 1; }
            area += ey * (x[2 * kn] + x[2 * k]) / 2.0;
            ef[2 * k] = (float)ex; ef[2 * k + 1] = (float)ey;
            acf[2 * k] = (float)(0.5 * (x[2 * kn + 1] - x[2 * kp + 1]));
            acf[2 * k + 1] = (float)(0.5 * (x[2 * kp] - x[2 * kn]));
            lam[k] = (float)(-sk);
        }
        double sA = area - A0;
        if (!(fabs(sA) <= worst)) worst = fabs(sA);
        if (nonfinite || !isfinite(worst)) { it = maxIter; break; }
        if (worst < tol) break;
        float dc = 0.f;
        for (int k = 0; k < n; ++k) {
            int kn = (k + 1) % n, kp = (k + n - 1) % n;
            float ex = ef[2 * k], ey = ef[2 * k + 1];
            pb[k] = 2.0f * (ex * rf[2 * k] + ey * rf[2 * k + 1]);
            pc[k] = -(ex * rf[2 * kn] + ey * rf[2 * kn + 1]);
            pa[k] = -(ex * rf[2 * kp] + ey * rf[2 * kp + 1]);
            p0[k] = lam[k];
            p1[k] = ex * (arf[2 * kn] - arf[2 * k]) + ey * (arf[2 * kn + 1] - arf[2 * k + 1]);
            p2[k] = 0.f;
            vr[k] = (acf[2 * kn] - acf[2 * k]) * rf[2 * k] + (acf[2 * kn + 1] - acf[2 * k + 1]) * rf[2 * k + 1];
            dc += acf[2 * k] * arf[2 * k] + acf[2 * k + 1] * arf[2 * k + 1];
        }
        for (int k = n; k < N; ++k) { pa[k] = 0.f; pb[k] = 1.f; pc[k] = 0.f; p0[k] = 0.f; p1[k] = 0.f; p2[k] = 0.f; }
        float gamma = -pb[0], beta = pa[0], alpha = pc[n - 1];
        if (!(gamma != 0.f)) { it = maxIter; break; }
        pb[0] = pb[0] - gamma;
        pb[n - 1] = pb[n - 1] - alpha * beta / gamma;
        pa[0] = 0.f; pc[n - 1] = 0.f;
        p2[0] = gamma; p2[n - 1] = alpha;
        pcr3_f(pa, pb, pc, p0, p1, p2, N);
        float den = 1.f + p2[0] + beta * p2[n - 1] / gamma;
        float fy = (p0[0] + beta * p0[n - 1] / gamma) / den;
        float fz = (p1[0] + beta * p1[n - 1] / gamma) / den;
        float vy = 0.f, vz = 0.f;
        for (int k = 0; k < n; ++k) {
            float sv = p2[k];
            float yk = p0[k] - fy * sv, zk = p1[k] - fz * sv;
            p0[k] = yk; p1[k] = zk;
            vy += vr[k] * yk; vz += vr[k] * zk;
        }
        float mu = (-(float)sA - vy) / (dc - vz);
        int finite = isfinite(mu);
        for (int k = 0; k < n; ++k) {
            lam[k] = p0[k] - mu * p1[k];
            finite = finite && isfinite(lam[k]);
        }
        if (!finite) { it = maxIter; break; }
        double mu64 = (double)mu;
        for (int k = 0; k < n; ++k) {
            int kp = (k + n - 1) % n;
            double lk = (double)lam[k], lp = (double)lam[kp];
            x[2 * k] += -lk * r[2 * k] + lp * r[2 * kp] + mu64 * ar[2 * k];
            x[2 * k + 1] += -lk * r[2 * k + 1] + lp * r[2 * kp + 1] + mu64 * ar[2 * k + 1];
        }
    }
    for (int k = 0; k < n; ++k) {
        double vx = ox + x[2 * k], vy = oy + x[2 * k + 1];
        m->positions[2 * (st + k)] = vx - floor(vx);
        m->positions[2 * (st + k) + 1] = vy - floor(vy);
    }
    return it;
}

int orc_shake_project(orc_model* m, int nIter, double tol) {
    int P = m->numPolygons;
    if (P == 0 || nIter == 0) { m->lastShakeIters = 0; return 0; }
    int nmax = 0;
    for (int p = 0; p < P; ++p) {
        int n = m->startIndices[p + 1] - m->startIndices[p];
        if (n > nmax) nmax = n;
    }
    int worst = 0;
    #pragma omp parallel reduction(max:worst)
    {
        double* work = (double*)xcalloc((size_t)40 * nmax + 64, 8);
        #pragma omp for schedule(dynamic, 16)
        for (int p = 0; p < P; ++p) {
            int it = shake_polygon(m, p, nIter, tol, work);
            if (it > worst) worst = it;
        }
        free(work);
    }
    m->lastShakeIters = worst;
    return worst;
}

/* ------------------------------------------------------------------------ */
/* XPBD (model.cu:209-278; kernels.cuh:532-623).  Not bound by the           */
/* reference.  Edges of even local index, then odd ones, move both ends     */
/* half-way to the target length; then one area correction along grad A.    */
/* For odd n the reference races on the shared vertex of the last and first */
/* edge (kernels.cuh:529-531); here the last edge runs after the odd colour.*/
/* ------------------------------------------------------------------------ */
static void xpbd_edge(orc_model* m, int k) {
    int p = m->shapeId[k], nk = m->next[k];
    double* pos = m->positions;
    double ex = orc_wrap(pos[2 * nk] - pos[2 * k]);
    double ey = orc_wrap(pos[2 * nk + 1] - pos[2 * k + 1]);
    double len = sqrt(ex * ex + ey * ey);
    if (len < 1e-14) return;
    double c = 0.5 * (len - m->targetEdgeLengths[p]) / len;
    pos[2 * k] += c * ex; pos[2 * k + 1] += c * ey;
    pos[2 * nk] -= c * ex; pos[2 * nk + 1] -= c * ey;
}

int orc_xpbd_project(orc_model* m, int nIter, double tol) {
    int P = m->numPolygons, V = m->size;
    double* area = (double*)xcalloc(P, 8);
    double* g2 = (double*)xcalloc(P, 8);
    double* gx = (double*)xcalloc(2 * (size_t)V, 8);
    int iter = 0;
    for (; iter < nIter; ++iter) {
        for (int color = 0; color < 3; ++color)
            for (int p = 0; p < P; ++p) {
                int st = m->startIndices[p], n = m->startIndices[p + 1] - st;
                for (int kl = 0; kl < n; ++kl) {
                    int c = kl % 2;
                    if ((n % 2) && kl == n - 1) c = 2;
                    if (c == color) xpbd_edge(m, st + kl);
                }
            }
        const double* pos = m->positions;
        memset(area, 0, (size_t)P * 8); memset(g2, 0, (size_t)P * 8);
        for (int k = 0; k < V; ++k) {
            int p = m->shapeId[k], s = m->startIndices[p];
            int nk = m->next[k], pk = m->prev[k];
            double xs = pos[2 * s], ys = pos[2 * s + 1];
            double xk = orc_wrap(pos[2 * k] - xs), yk = orc_wrap(pos[2 * k + 1] - ys);
            double xnk = orc_wrap(pos[2 * nk] - xs), ynk = orc_wrap(pos[2 * nk + 1] - ys);
            double xpk = orc_wrap(pos[2 * pk] - xs), ypk = orc_wrap(pos[2 * pk + 1] - ys);
            area[p] += 0.5 * (xk * ynk - xnk * yk);
            double a = 0.5 * (ynk - ypk), b = 0.5 * (xpk - xnk);
            g2[p] += a * a + b * b;
            gx[2 * k] = a; gx[2 * k + 1] = b;
        }
        for (int k = 0; k < V; ++k) {
            int p = m->shapeId[k];
            double al = (area[p] - m->targetAreas[p]) / fmax(g2[p], 1e-24);
            m->positions[2 * k] -= al * gx[2 * k];
            m->positions[2 * k + 1] -= al * gx[2 * k + 1];
        }
        if (tol > 0) {
            double me = 0.0, ma = 0.0;
            for (int k = 0; k < V; ++k) {
                int p = m->shapeId[k], nk = m->next[k];
                double ex = orc_wrap(pos[2 * nk] - pos[2 * k]);
                double ey = orc_wrap(pos[2 * nk + 1] - pos[2 * k + 1]);
                double d = fabs(sqrt(ex * ex + ey * ey) - m->targetEdgeLengths[p]);
                if (d > me) me = d;
            }
            for (int p = 0; p < P; ++p) {
                double d = fabs(area[p] - m->targetAreas[p]);
                if (d > ma) ma = d;
            }
            if (me < tol && ma < tol) break;
        }
    }
    free(area); free(g2); free(gx);
    return iter;
}

/* ------------------------------------------------------------------------ */
/* integrators                                                                */
/* ------------------------------------------------------------------------ */
/* updatePositionsKernel (kernels.cuh:1433-1438) */
void orc_update_positions(orc_model* m, double dt) {
    for (int i = 0; i < 2 * m->size; ++i) {
        double p = m->positions[i] + m->force[i] * dt;
        m->positions[i] = p - floor(p);
    }
}

void orc_reset_velocities(orc_model* m) { memset(m->velocities, 0, 2 * (size_t)m->size * 8); }

/* resetAreasKernel (kernels.cuh:1440-1455) */
void orc_reset_areas(orc_model* m) {
    for (int idx = 0; idx < 2 * m->size; ++idx) {
        double x = m->positions[idx];
        int s = m->shapeId[idx / 2];
        double cur = m->areas[s], tgt = m->targetAreas[s];
        if (!(cur > 0.0)) continue;
        double rescale = sqrt(tgt / cur);
        double u = (idx % 2) ? orc_wrap(x - m->comY[s]) : orc_wrap(x - m->comX[s]);
        u *= rescale;
        double p = (idx % 2) ? u + m->comY[s] : u + m->comX[s];
        m->positions[idx] = p - floor(p);
    }
}

void orc_save_tentative_positions(orc_model* m) {
    memcpy(m->positionsTMP, m->positions, 2 * (size_t)m->size * 8);
}

/* getMaxEffectiveForceCUDA (model.cu:284-306; kernels.cuh:625-633) */
double orc_get_max_effective_force(orc_model* m, double dt, int minimizerFIRE) {
    double scale = minimizerFIRE ? 2.0 / (dt * dt) : 1.0 / dt;
    double mx = -DBL_MAX;
    for (int k = 0; k < m->size; ++k) {
        double fx = m->force[2 * k] + scale * (m->positions[2 * k] - m->positionsTMP[2 * k]);
        double fy = m->force[2 * k + 1] + scale * (m->positions[2 * k + 1] - m->positionsTMP[2 * k + 1]);
        double v = sqrt(fx * fx + fy * fy);
        if (v > mx) mx = v;
    }
    return mx;
}

/* getMaxUnbalancedForceCUDA (model.cu:91-109, 612-614): max |component| */
double orc_get_max_unbalanced_force(orc_model* m) {
    double mx = -DBL_MAX;
    for (int i = 0; i < 2 * m->size; ++i) {
        double a = fabs(m->force[i]);
        if (a > mx) mx = a;
    }
    return mx;
}

/* FIRE pieces (restated; src/FIRE.h is absent).  Velocity-Verlet FIRE of
 * Bitzek et al., PRL 97, 170201 (2006):
 *   updatePositionAndVelocity: v += dt/2 F;  x = frac(x + dt v)
 *   updateVelocity:            v += dt/2 F
 *   bend (P = F.v first):      v = (1-a) v + a |v| F/|F|   (|F| > 0)
 *   rederive after SHAKE:      v += wrap(x_shake - x_verlet) / dt          */
static void fire_pos_vel(orc_model* m, double dt) {
    for (int i = 0; i < 2 * m->size; ++i) {
        double v = m->velocities[i] + 0.5 * dt * m->force[i];
        m->velocities[i] = v;
        double p = m->positions[i] + dt * v;
        m->positions[i] = p - floor(p);
    }
}
static void fire_vel(orc_model* m, double dt) {
    for (int i = 0; i < 2 * m->size; ++i) m->velocities[i] += 0.5 * dt * m->force[i];
}
static double fire_bend(orc_model* m, double alpha) {
    double P = 0.0, vv = 0.0, ff = 0.0;
    for (int i = 0; i < 2 * m->size; ++i) {
        P += m->force[i] * m->velocities[i];
        vv += m->velocities[i] * m->velocities[i];
        ff += m->force[i] * m->force[i];
    }
    double vn = sqrt(vv), fn = sqrt(ff);
    if (fn > 0.0) {
        double s = alpha * vn / fn;
        for (int i = 0; i < 2 * m->size; ++i)
            m->velocities[i] = (1.0 - alpha) * m->velocities[i] + s * m->force[i];
    }
    return P;
}
static void fire_rederive(orc_model* m, double dt) {
    for (int i = 0; i < 2 * m->size; ++i)
        m->velocities[i] += orc_wrap(m->positions[i] - m->positionsTMP[i]) / dt;
}

/* Model::minimizeFIREStep (model.cpp:405-486) */
void orc_fire_step(orc_model* m, double dt, double alpha, int nPos, double dtMax,
                   double alphaStart, double fAlpha, double fInc, double fDec,
                   int nMin, int shakeIter, double out[4]) {
    int needsI = (m->modelType == ORC_NORMAL || m->modelType == ORC_HYBRID);
    int rigid = (m->modelType == ORC_NORMAL);
    int shakeFailed = 0;
    size_t nb = 2 * (size_t)m->size * 8;
    memcpy(m->positionsTMP2, m->positions, nb);
    double ePre = m->energy;
    fire_pos_vel(m, dt);
    orc_update_polygon_geometry(m);
    if (needsI) {
        orc_update_neighbor_cells(m);
        orc_update_neighbors(m);
        if (rigid && shakeIter > 0) {
            memcpy(m->positionsTMP, m->positions, nb);
            orc_shake_project(m, shakeIter, 1e-15);
            orc_update_polygon_geometry(m);
            m->fireFirstShakeIters = m->lastShakeIters;
            if (m->lastShakeIters >= shakeIter) {
                orc_shake_project(m, shakeIter * 10, 1e-15);
                orc_update_polygon_geometry(m);
                if (m->lastShakeIters >= shakeIter * 10) shakeFailed = 1;
            }
            if (shakeFailed) {
                memcpy(m->positions, m->positionsTMP2, nb);
                orc_update_polygon_geometry(m);
                orc_reset_velocities(m);
            } else {
                fire_rederive(m, dt);
            }
        }
        orc_update_outersections(m);
    }
    orc_update_force_energy(m);
    if (rigid) orc_project_force(m);
    if (shakeFailed) {
        out[0] = m->energy; out[1] = dt * fDec; out[2] = alphaStart; out[3] = 0;
        return;
    }
    double ePost = m->energy;
    if (ePost > ePre + fmax(fabs(ePre) * 1e-10, 1e-14)) {
        memcpy(m->positions, m->positionsTMP2, nb);
        orc_update_polygon_geometry(m);
        if (needsI) {
            orc_update_neighbor_cells(m);
            orc_update_neighbors(m);
            orc_update_outersections(m);
            orc_update_force_energy(m);
            if (rigid) orc_project_force(m);
        } else {
            orc_update_force_energy(m);
        }
        orc_reset_velocities(m);
        out[0] = ePre; out[1] = dt * fDec; out[2] = alphaStart; out[3] = 0;
        return;
    }
    fire_vel(m, dt);
    double P = fire_bend(m, alpha);
    if (P > 0.0) {
        if (++nPos >= nMin) {
            double nd = fmin(dt * fInc, dtMax);
            if (nd > dt) alpha = alpha * fAlpha;
            dt = nd;
        }
    } else {
        orc_reset_velocities(m);
        dt = dt * fDec;
        alpha = alphaStart;
        nPos = 0;
    }
    out[0] = m->energy; out[1] = dt; out[2] = alpha; out[3] = nPos;
}

/* Model::minimizeFIRE (model.cpp:488-504) */
void orc_minimize_fire(orc_model* m, double thr, double dt0, int maxSteps,
                       double dtMax, double alphaStart, double fAlpha, double fInc,
                       double fDec, int nMin, int shakeIter, double out[3]) {
    orc_reset_velocities(m);
    double dt = dt0, alpha = alphaStart;
    int nPos = 0;
    int rigid = (m->modelType == ORC_NORMAL);
    orc_update_polygon_geometry(m);
    orc_update_force_energy(m);
    if (rigid) orc_project_force(m);
    double r[4];
    for (int step = 0; step < maxSteps; ++step) {
        orc_fire_step(m, dt, alpha, nPos, dtMax, alphaStart, fAlpha, fInc, fDec, nMin, shakeIter, r);
        dt = r[1]; alpha = r[2]; nPos = (int)r[3];
        if (orc_get_max_unbalanced_force(m) <= thr) {
            out[0] = r[0]; out[1] = dt; out[2] = step + 1;
            return;
        }
    }
    out[0] = m->energy; out[1] = dt; out[2] = maxSteps;
}

/* ---- getters ---- */
int orc_num_vertices(const orc_model* m) { return m->size; }
int orc_num_polygons(const orc_model* m) { return m->numPolygons; }
int orc_num_intersections(const orc_model* m) { return m->numIntersections; }
int orc_max_neighbors(const orc_model* m) { return m->maxNeighbors; }
int orc_box_size(const orc_model* m) { return m->boxSize; }
int orc_last_shake_iters(const orc_model* m) { return m->lastShakeIters; }
/* iterations of the first SHAKE call of the last FIRE step: at the limit,
 * the step retried (no counterpart in the reference; test use) */
int orc_fire_first_shake_iters(const orc_model* m) { return m->fireFirstShakeIters; }
double orc_energy(const orc_model* m) { return m->energy; }
double orc_max_edge_length(const orc_model* m) { return m->maxEdgeLength; }
const double* orc_positions(const orc_model* m) { return m->positions; }
const double* orc_forces(const orc_model* m) { return m->force; }
const double* orc_velocities(const orc_model* m) { return m->velocities; }
const double* orc_areas(const orc_model* m) { return m->areas; }
const double* orc_com_x(const orc_model* m) { return m->comX; }
const double* orc_com_y(const orc_model* m) { return m->comY; }
const double* orc_edge_lengths(const orc_model* m) { return m->edgeLengths; }
const double* orc_constraints(const orc_model* m) { return m->constraints; }
const double* orc_perimeters(const orc_model* m) { return m->perimeters; }
const int* orc_shape_id(const orc_model* m) { return m->shapeId; }
const int* orc_start_indices(const orc_model* m) { return m->startIndices; }
const int* orc_cell_location(const orc_model* m) { return m->cellLocation; }
/* ------------------------------------------------------------------------ */
/* Grid-point overlap estimate: updateOverlapAreaKernel (kernels.cuh:879-979) */
/* and Model::updateOverlapArea (model.cpp:824-847).  Point (ix+.5, iy+.5)/d; */
/* the polygons owning a vertex in the 3x3 cells around it (each once, at    */
/* most 512 of them), an angle-sum inside test with the loop form of the     */
/* minimum image (wrapPeriodic, kernels.cuh:108-113), c(c-1)/2 per point,    */
/* the sum divided by d^2.  Uses the current cell list.                       */
/* ------------------------------------------------------------------------ */
static double orc_wrap_periodic(double x) {
    x += 1.5;
    while (x > 1.0) x -= 1.0;
    return x - 0.5;
}

double orc_update_overlap_area(orc_model* m, int d) {
    const double eps = 1e-12, PI = 3.141592653589793238462643383279;
    const double* pos = m->positions;
    const int B = m->boxSize, boxCount = B * B;
    long long total = 0;
    for (int idx = 0; idx < d * d; ++idx) {
        int ix = idx % d, iy = idx / d;
        double px = (ix + 0.5) / d, py = (iy + 0.5) / d;
        int cellX = (int)(px * B), cellY = (int)(py * B);
        int tracked[512], nt = 0, hits = 0, full = 0;
        for (int dx = -1; dx <= 1 && !full; ++dx) {
            int nx = cellX + dx;
            if (nx < 0) nx += B; else if (nx >= B) nx -= B;
            for (int dy = -1; dy <= 1 && !full; ++dy) {
                int ny = cellY + dy;
                if (ny < 0) ny += B; else if (ny >= B) ny -= B;
                int box = ny * B + nx;
                int si = m->countPerBox[box];
                int sf = (box + 1 < boxCount) ? m->countPerBox[box + 1] : m->size;
                for (int q = si; q < sf; ++q) {
                    int poly = m->shapeId[m->neighborIndices[q]], seen = 0;
                    for (int t = 0; t < nt; ++t) if (tracked[t] == poly) { seen = 1; break; }
                    if (seen) continue;
                    int s0 = m->startIndices[poly], s1 = m->startIndices[poly + 1];
                    if (s1 - s0 < 3) continue;
                    double ang = 0.0;
                    double vxp = orc_wrap_periodic(pos[2 * s0] - px);
                    double vyp = orc_wrap_periodic(pos[2 * s0 + 1] - py);
                    double vx0 = vxp, vy0 = vyp;
                    /* The reference's build (nvcc, default contraction)
                     * evaluates a*b - c*d as fma(a, b, -(c*d)) and a*b + c*d
                     * as fma(a, b, c*d).  At grid points on an edge the cross
                     * product is zero only without the fused rounding, and
                     * its sign picks atan2's +pi or -pi, i.e. the count:
                     * tests/golden/ref_gpu_odd_shapes.npz pins this form. */
                    for (int e = s0 + 1; e < s1; ++e) {
                        double vx = vxp + orc_wrap_periodic(pos[2 * e] - pos[2 * e - 2]);
                        double vy = vyp + orc_wrap_periodic(pos[2 * e + 1] - pos[2 * e - 1]);
                        ang += atan2(fma(vxp, vy, -(vyp * vx)), fma(vxp, vx, vyp * vy));
                        vxp = vx; vyp = vy;
                    }
                    ang += atan2(fma(vxp, vy0, -(vyp * vx0)), fma(vxp, vx0, vyp * vy0));
                    if (fabs(ang - 2.0 * PI) < eps) hits++;
                    if (nt < 512) tracked[nt++] = poly;
                    else { full = 1; break; }
                }
            }
        }
        total += (long long)hits * (hits - 1) / 2;
    }
    return (double)total / ((double)d * (double)d);
}

const int* orc_neighbor_indices(const orc_model* m) { return m->neighborIndices; }
const int* orc_box_starts(const orc_model* m) { return m->countPerBox; }
const int* orc_neighbors(const orc_model* m) { return m->neighbors; }
const int* orc_num_neighbors(const orc_model* m) { return m->numNeighbors; }
const uint8_t* orc_inside(const orc_model* m) { return m->inside; }
const int* orc_shape_counts(const orc_model* m) { return m->shapeCounts; }
const uint64_t* orc_intersections(const orc_model* m) { return m->intersections; }
const uint64_t* orc_outersections(const orc_model* m) { return m->outersections; }
const double* orc_tu(const orc_model* m) { return m->tu; }
const double* orc_ut(const orc_model* m) { return m->ut; }
const double* orc_target_areas(const orc_model* m) { return m->targetAreas; }
const double* orc_target_edge_lengths(const orc_model* m) { return m->targetEdgeLengths; }
