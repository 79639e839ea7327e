// Golden-vector driver around the reference's own C++ Model (TEST
// INFRASTRUCTURE).
//
// Built by oracle/ref_build.py against the reference's src/model.cpp and
// src/model.cu (compiled for sm_103a with the shims in oracle/ref_shim/) and
// run on a GPU by tests/golden/make_ref_gpu_golden.py.  It loads one polygon
// system, runs the reference's evaluation path through its public Model
// methods in the order its Python layer uses them (pyCudaPolygon.py:54-65,
// model.cpp:252-395), and writes every intermediate the Model exposes.  The
// outputs become tests/golden/ref_gpu_*.npz, the fixtures the CPU oracle is
// checked against.
//
// Input (little-endian, written by make_ref_gpu_golden.py):
//   int32  magic 0x47504350 ('PCPG'), version 1
//   int32  V, P, flags, point_density
//   double max_edge_length, stiffness, compressibility
//   int32  start[P+1]; double pos[2V]; double target_areas[P];
//   double target_edge_lengths[P]
// flags: 1 overlap energy/force (normal model), 2 projectForce after it,
//        4 grid overlap estimate, 8 softBody energy/force, 16 hybrid.
// Output: records {int32 name length, name, int32 type (0 f64, 1 i32, 2 u64,
//         3 u8), int64 count, raw data}.
//
// Timing mode, `ref_golden --time <input.bin> <reps> <output.json>`: after
// one warm-up evaluation, <reps> evaluations of the same path (geometry,
// cells, neighbours, outersections, and with flag 1 the overlap force, with
// flag 2 the projection), each method timed on the host around the call and
// a device synchronisation; the mean milliseconds per stage go to a JSON
// object.  The reference's methods allocate, copy and synchronise inside,
// so the host clock is the honest one for them.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "model.hpp"

namespace {

FILE* g_out = nullptr;

void emit(const char* name, int type, const void* data, int64_t count, size_t elem) {
    int32_t len = (int32_t)std::string(name).size();
    std::fwrite(&len, 4, 1, g_out);
    std::fwrite(name, 1, (size_t)len, g_out);
    int32_t t = type;
    std::fwrite(&t, 4, 1, g_out);
    std::fwrite(&count, 8, 1, g_out);
    if (count > 0) std::fwrite(data, elem, (size_t)count, g_out);
}
void emit(const char* name, const std::vector<double>& v) { emit(name, 0, v.data(), (int64_t)v.size(), 8); }
void emit(const char* name, const std::vector<int>& v) { emit(name, 1, v.data(), (int64_t)v.size(), 4); }
void emit(const char* name, const std::vector<uint64_t>& v) { emit(name, 2, v.data(), (int64_t)v.size(), 8); }
void emit(const char* name, const std::vector<uint32_t>& v) {
    std::vector<int> w(v.begin(), v.end());
    emit(name, w);
}
void emit(const char* name, const std::vector<bool>& v) {
    std::vector<uint8_t> w(v.size());
    for (size_t i = 0; i < v.size(); ++i) w[i] = v[i] ? 1 : 0;
    emit(name, 3, w.data(), (int64_t)w.size(), 1);
}
void emit(const char* name, double x) { emit(name, 0, &x, 1, 8); }
void emit(const char* name, int x) { emit(name, 1, &x, 1, 4); }

template <typename T>
void read_into(FILE* f, T* dst, size_t n) {
    if (std::fread(dst, sizeof(T), n, f) != n) {
        std::fprintf(stderr, "ref_golden: short input\n");
        std::exit(2);
    }
}

int time_stages(Model& m, int reps, int flags, const char* path) {
    static const char* kNames[6] = {"updatePolygonGeometry", "updateNeighborCells",
                                    "updateNeighbors", "updateOutersections",
                                    "updateForceEnergy", "projectForce"};
    const int stages = (flags & 1) ? ((flags & 2) ? 6 : 5) : 4;
    auto run = [&m](int s) {
        switch (s) {
            case 0: m.updatePolygonGeometry(); break;
            case 1: m.updateNeighborCells(); break;
            case 2: m.updateNeighbors(); break;
            case 3: m.updateOutersections(); break;
            case 4: m.updateForceEnergy(); break;
            default: m.projectForce(); break;
        }
    };
    for (int s = 0; s < stages; ++s) run(s);
    if (cudaDeviceSynchronize() != cudaSuccess) return 3;
    double total[6] = {0, 0, 0, 0, 0, 0};
    for (int r = 0; r < reps; ++r) {
        for (int s = 0; s < stages; ++s) {
            auto t0 = std::chrono::steady_clock::now();
            run(s);
            if (cudaDeviceSynchronize() != cudaSuccess) return 3;
            total[s] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
    }
    FILE* f = std::fopen(path, "w");
    if (!f) { std::perror(path); return 2; }
    std::fprintf(f, "{\"reps\": %d, \"records\": %d, \"energy\": %.17g, \"stage_ms\": {",
                 reps, m.getNumIntersections(), (flags & 1) ? m.getEnergy() : 0.0);
    for (int s = 0; s < stages; ++s)
        std::fprintf(f, "%s\"%s\": %.6f", s ? ", " : "", kNames[s], 1e3 * total[s] / reps);
    std::fprintf(f, "}}\n");
    std::fclose(f);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    const bool timing = argc == 5 && std::string(argv[1]) == "--time";
    if (argc != 3 && !timing) {
        std::fprintf(stderr, "usage: ref_golden <input.bin> <output.bin>\n"
                             "       ref_golden --time <input.bin> <reps> <output.json>\n");
        return 2;
    }
    const char* inPath = timing ? argv[2] : argv[1];
    FILE* in = std::fopen(inPath, "rb");
    if (!in) { std::perror(inPath); return 2; }
    int32_t hdr[6];
    read_into(in, hdr, 6);
    if (hdr[0] != 0x47504350 || hdr[1] != 1) {
        std::fprintf(stderr, "ref_golden: bad header\n");
        return 2;
    }
    const int V = hdr[2], P = hdr[3], flags = hdr[4], point_density = hdr[5];
    double scal[3];
    read_into(in, scal, 3);
    std::vector<int> start(P + 1);
    std::vector<double> pos(2 * (size_t)V), ta(P), tl(P);
    read_into(in, start.data(), start.size());
    read_into(in, pos.data(), pos.size());
    read_into(in, ta.data(), ta.size());
    read_into(in, tl.data(), tl.size());
    std::fclose(in);
    if (V <= 0 || P <= 0 || start[0] != 0 || start[P] != V) {
        std::fprintf(stderr, "ref_golden: inconsistent sizes\n");
        return 2;
    }
    Model m(V);
    // The constructor leaves the model type unset (model.cpp:99 passes the
    // member's own indeterminate value); the Python model sets it right after
    // construction (pyCudaPolygon.py:40-41), and so does this driver.
    m.setModelEnum(simControlStruct::modelEnum::normal);
    m.setStartIndices(start);
    m.setPositions(pos);
    m.setTargetAreas(ta);
    m.setTargetEdgeLengths(tl);
    // The cell grid is sized by initializeNeighborCells from boxSize, so the
    // cell size is set first (the Python wrapper's own order sets 0.5 after
    // it, pyCudaPolygon.py:54-57, and would leave a 2x2 grid).
    m.setMaxEdgeLength(scal[0]);
    m.initializeNeighborCells();
    if (timing) {
        const int reps = std::atoi(argv[3]);
        if (reps < 1) { std::fprintf(stderr, "ref_golden: reps must be positive\n"); return 2; }
        return time_stages(m, reps, flags, argv[4]);
    }
    g_out = std::fopen(argv[2], "wb");
    if (!g_out) { std::perror(argv[2]); return 2; }

    m.updatePolygonGeometry();
    emit("areas", m.getAreas());
    emit("com", m.getCOM());
    emit("constraints", m.getConstraints());
    emit("edge_lengths", m.getEdgeLengths());
    emit("max_edge_length", m.getMaxEdgeLength());
    emit("shape_id", m.getShapeId());

    m.updateNeighborCells();
    emit("cell_location", m.getNeighborCells());
    emit("neighbor_indices", m.getNeighborIndices());
    emit("box_counts", m.getBoxCounts());

    m.updateNeighbors();
    emit("num_neighbors", m.getNumNeighbors());
    emit("neighbors", m.getNeighbors());
    emit("inside", m.getInsideFlag());

    m.updateOutersections();
    emit("num_intersections", m.getNumIntersections());
    emit("intersections", m.getIntersections());
    emit("outersections", m.getOutersections());
    emit("tu", m.getTU());
    emit("ut", m.getUT());
    emit("shape_counts", m.getShapeCounts());

    if (flags & 1) {
        m.updateForceEnergy();
        emit("energy", m.getEnergy());
        emit("forces", m.getForces());
        if (flags & 2) {
            m.projectForce();
            emit("forces_projected", m.getForces());
            emit("max_unbalanced_force", m.getMaxUnbalancedForce());
        }
    }
    if (flags & 4) {
        m.updateOverlapArea(point_density);
        emit("overlap_area", m.getOverlapArea());
        emit("intersections_counter", m.getIntersectionsCounter());
    }
    if (flags & (8 | 16)) {
        m.setStiffness(scal[1]);
        m.setCompressibility(scal[2]);
    }
    if (flags & 8) {
        m.setModelEnum(simControlStruct::modelEnum::softBody);
        m.updateForceEnergy();
        emit("soft_energy", m.getEnergy());
        emit("soft_forces", m.getForces());
    }
    if (flags & 16) {
        m.setModelEnum(simControlStruct::modelEnum::hybrid);
        m.updateForceEnergy();
        emit("hybrid_energy", m.getEnergy());
        emit("hybrid_forces", m.getForces());
    }
    std::fclose(g_out);
    return 0;
}
