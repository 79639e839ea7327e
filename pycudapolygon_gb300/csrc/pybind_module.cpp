// pybind_module.cpp -- the `libpyCudaPolygon` extension module.
//
// Same module name, enums and `Model` method table as the reference's
// binding (camdennis/pyCudaPolygon src/pybindWrapper.cpp:12-108), so the
// reference's Python layer (pyCudaPolygon.py, enums.py, the mixins) runs on
// it unchanged.  Every method forwards to the pcp_model_* C ABI
// (include/pcp_gb300.h).  Differences a caller can see:
//   * array getters return numpy arrays instead of lists (the reference's
//     Python layer wraps every getter in np.array already);
//   * a CUDA or capacity error raises RuntimeError instead of exit();
//   * a few extra methods (xpbdProject, getVelocities, getPairCount, ...).
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "pcp_gb300.h"

namespace py = pybind11;

enum class minimizerEnum { GD = 0, FIRE = 1 };
struct simControlStruct {
    enum class modelEnum { normal = 0, edgeOnly = 1, areaOnly = 2, softBody = 3, abnormal = 4,
                           hybrid = 5 };
};

static void check(int rc) {
    if (rc != PCP_OK) throw std::runtime_error(std::string("pcp_gb300: ") + pcp_last_error());
}

using darr = py::array_t<double, py::array::c_style | py::array::forcecast>;
using iarr = py::array_t<int, py::array::c_style | py::array::forcecast>;

class Model {
public:
    explicit Model(int size) { check(pcp_model_create(size, &m_)); }
    ~Model() { pcp_model_destroy(m_); }
    Model(const Model&) = delete;
    Model& operator=(const Model&) = delete;

    pcp_model* handle() { return m_; }

    // initialisers / helpers
    void initializeNeighborCells() { check(pcp_model_initialize_neighbor_cells(m_)); }
    void sortKeys(int endBit) { check(pcp_model_sort_keys(m_, endBit)); }

    // setters
    void setNumVertices(int n) { check(pcp_model_set_num_vertices(m_, n)); }
    void setPositions(darr a) {
        // the reference prints and ignores a wrong length (model.cpp:522-528)
        pcp_model_set_positions(m_, a.data(), (int)a.size());
    }
    void setForces(darr a) { check(pcp_model_set_forces(m_, a.data(), (int)a.size())); }
    void setModelEnum(simControlStruct::modelEnum e) { check(pcp_model_set_model_enum(m_, (int)e)); }
    void setStartIndices(iarr a) { check(pcp_model_set_start_indices(m_, a.data(), (int)a.size())); }
    void setMaxEdgeLength(double l) { check(pcp_model_set_max_edge_length(m_, l)); }
    void setTargetEdgeLengths(darr a) { check(pcp_model_set_target_edge_lengths(m_, a.data(), (int)a.size())); }
    void setTargetAreas(darr a) { check(pcp_model_set_target_areas(m_, a.data(), (int)a.size())); }
    void setStiffness(double k) { check(pcp_model_set_stiffness(m_, k)); }
    void setCompressibility(double c) { check(pcp_model_set_compressibility(m_, c)); }
    double getStiffness() { double v; check(pcp_model_get_stiffness(m_, &v)); return v; }
    double getCompressibility() { double v; check(pcp_model_get_compressibility(m_, &v)); return v; }

    // updaters
    void updatePolygonGeometry() { check(pcp_model_update_polygon_geometry(m_)); }
    void projectForce() { check(pcp_model_project_force(m_)); }
    int shakeProject(int nIter, double tol) { int it = 0; check(pcp_model_shake_project(m_, nIter, tol, &it)); return it; }
    int xpbdProject(int nIter, double tol) { int it = 0; check(pcp_model_xpbd_project(m_, nIter, tol, &it)); return it; }
    int getLastShakeIters() { int v; check(pcp_model_get_last_shake_iters(m_, &v)); return v; }
    void saveTentativePositions() { check(pcp_model_save_tentative_positions(m_)); }
    double getMaxEffectiveForce(double dt, minimizerEnum t) {
        double v; check(pcp_model_get_max_effective_force(m_, dt, (int)t, &v)); return v;
    }
    void updateNeighborCells() { check(pcp_model_update_neighbor_cells(m_)); }
    void updateNeighbors() { check(pcp_model_update_neighbors(m_)); }
    void updateValidAndCounts() { check(pcp_model_update_valid_and_counts(m_)); }
    void updateCompactedIntersections() { check(pcp_model_update_compacted_intersections(m_)); }
    void updateOutersections() { check(pcp_model_update_outersections(m_)); }
    void updateOverlapArea(int d) { check(pcp_model_update_overlap_area(m_, d)); }
    void updateForceEnergy() { check(pcp_model_update_force_energy(m_)); }
    void updatePositions(double dt) { check(pcp_model_update_positions(m_, dt)); }
    void resetAreas() { check(pcp_model_reset_areas(m_)); }
    void resetVelocities() { check(pcp_model_reset_velocities(m_)); }

    std::tuple<double, double, double, int> minimizeFIREStep(double dt, double alpha, int nPos,
                                                             double dtMax, double alphaStart,
                                                             double fAlpha, double fInc,
                                                             double fDec, int nMin, int shakeIter) {
        double out[4];
        {
            py::gil_scoped_release nogil;
            check(pcp_model_fire_step(m_, dt, alpha, nPos, dtMax, alphaStart, fAlpha, fInc, fDec,
                                      nMin, shakeIter, out));
        }
        return {out[0], out[1], out[2], (int)out[3]};
    }
    std::tuple<double, double, int> minimizeFIRE(double thr, double dtInit, int maxSteps,
                                                 double dtMax, double alphaStart, double fAlpha,
                                                 double fInc, double fDec, int nMin, int shakeIter) {
        double out[3];
        {
            py::gil_scoped_release nogil;
            check(pcp_model_minimize_fire(m_, thr, dtInit, maxSteps, dtMax, alphaStart, fAlpha,
                                          fInc, fDec, nMin, shakeIter, out));
        }
        return {out[0], out[1], (int)out[2]};
    }

    py::tuple minimizeFIREDevice(double thr, double dt, int maxSteps, double dtMax,
                                 double alphaStart, double fAlpha, double fInc, double fDec,
                                 int nMin, int shakeIter) {
        double out[6];
        {
            py::gil_scoped_release nogil;
            check(pcp_model_minimize_fire_driver(m_, thr, dt, maxSteps, dtMax, alphaStart, fAlpha,
                                                 fInc, fDec, nMin, shakeIter, out));
        }
        if (maxSteps <= 0) return py::make_tuple(out[0], out[1], 0);
        py::list stats;
        stats.append(out[3]); stats.append(out[4]); stats.append(out[5]);
        return py::make_tuple(out[0], out[1], (int)out[2], stats);
    }
    void setPositionsDevice(std::uintptr_t ptr, int len) {
        check(pcp_model_set_positions_device(m_, reinterpret_cast<const double*>(ptr), len));
    }
    double overlapEnergyGradient(int mode, bool search, std::uintptr_t outPtr) {
        double e = 0.0;
        {
            py::gil_scoped_release nogil;
            check(pcp_model_overlap_energy_gradient(m_, mode, search ? 1 : 0, &e,
                                                    reinterpret_cast<double*>(outPtr)));
        }
        return e;
    }
    void fireSetStopRule(double tol, int stagnantLimit) {
        check(pcp_model_fire_set_stop_rule(m_, tol, stagnantLimit));
    }
    py::tuple fireRunStats() {
        double out[4];
        check(pcp_model_fire_run_stats(m_, out));
        return py::make_tuple((int)out[0], out[1], out[2], out[3]);
    }
    void fireSetup(double thr, double dt, int maxSteps, double dtMax, double alphaStart,
                   double fAlpha, double fInc, double fDec, int nMin, int shakeIter) {
        py::gil_scoped_release nogil;
        check(pcp_model_fire_setup(m_, thr, dt, maxSteps, dtMax, alphaStart, fAlpha, fInc, fDec,
                                   nMin, shakeIter));
    }
    void fireContinue(int n) { check(pcp_model_fire_continue(m_, n)); }
    py::tuple fireStatus() {
        double out[8];
        int redo = 0;
        {
            py::gil_scoped_release nogil;
            check(pcp_model_fire_status(m_, out, &redo));
        }
        return py::make_tuple(out[0], out[1], out[2], (int)out[3], out[4], (long long)out[5],
                              out[6] != 0.0, (int)out[7], redo != 0);
    }
    void contactsStage(int s) { check(pcp_model_contacts_stage(m_, s)); }

    // scalar getters
    int getNumVertices() { int v; check(pcp_model_get_num_vertices(m_, &v)); return v; }
    int getNumPolygons() { int v; check(pcp_model_get_num_polygons(m_, &v)); return v; }
    int getNumIntersections() { int v; check(pcp_model_get_num_intersections(m_, &v)); return v; }
    int getMaxNeighbors() { int v; check(pcp_model_get_max_neighbors(m_, &v)); return v; }
    int getBoxSize() { int v; check(pcp_model_get_box_size(m_, &v)); return v; }
    double getEnergy() { double v; check(pcp_model_get_energy(m_, &v)); return v; }
    double getMaxUnbalancedForce() { double v; check(pcp_model_get_max_unbalanced_force(m_, &v)); return v; }
    double getMaxEdgeLength() { double v; check(pcp_model_get_max_edge_length(m_, &v)); return v; }
    double getOverlapArea() { double v; check(pcp_model_get_overlap_area(m_, &v)); return v; }
    long long getPairCount() { long long v; check(pcp_model_get_pair_count(m_, &v)); return v; }
    long long getNarrowPairTotal() {
        long long v;
        check(pcp_model_get_narrow_pair_total(m_, &v));
        return v;
    }
    long long getLaunchCount() { long long v; check(pcp_model_get_launch_count(m_, &v)); return v; }
    std::tuple<int, int> getNarrowPairCount() {
        int a = 0, b = 0;
        check(pcp_model_get_narrow_pair_count(m_, &a, &b));
        return std::make_tuple(a, b);
    }
    std::string getModelEnum() {
        int e; check(pcp_model_get_model_enum(m_, &e));
        static const char* names[] = {"normal", "edgeOnly", "areaOnly", "softBody", "abnormal", "hybrid"};
        return (e >= 0 && e < 6) ? names[e] : std::to_string(e);
    }

    template <typename T, typename F>
    py::array_t<T> arr(F getter) {
        int n = 0;
        check(getter(m_, nullptr, 0, &n));
        py::array_t<T> out(n);
        if (n > 0) {
            int n2 = 0;
            check(getter(m_, out.mutable_data(), n, &n2));
        }
        return out;
    }
    py::array_t<double> getPositions() { return arr<double>(pcp_model_get_positions); }
    py::array_t<double> getForces() { return arr<double>(pcp_model_get_forces); }
    py::array_t<double> getVelocities() { return arr<double>(pcp_model_get_velocities); }
    py::array_t<double> getAreas() { return arr<double>(pcp_model_get_areas); }
    py::array_t<double> getCOM() { return arr<double>(pcp_model_get_com); }
    py::array_t<double> getPerimeters() { return arr<double>(pcp_model_get_perimeters); }
    py::array_t<double> getEdgeLengths() { return arr<double>(pcp_model_get_edge_lengths); }
    py::array_t<double> getConstraints() { return arr<double>(pcp_model_get_constraints); }
    py::array_t<double> getTargetAreas() { return arr<double>(pcp_model_get_target_areas); }
    py::array_t<double> getTargetEdgeLengths() { return arr<double>(pcp_model_get_target_edge_lengths); }
    py::array_t<double> getTU() { return arr<double>(pcp_model_get_tu); }
    py::array_t<double> getUT() { return arr<double>(pcp_model_get_ut); }
    py::array_t<int> getShapeId() { return arr<int>(pcp_model_get_shape_id); }
    py::array_t<int> getNeighborCells() { return arr<int>(pcp_model_get_neighbor_cells); }
    py::array_t<int> getNeighborIndices() { return arr<int>(pcp_model_get_neighbor_indices); }
    py::array_t<int> getBoxCounts() { return arr<int>(pcp_model_get_box_counts); }
    py::array_t<int> getNeighbors() { return arr<int>(pcp_model_get_neighbors); }
    py::array_t<int> getNumNeighbors() { return arr<int>(pcp_model_get_num_neighbors); }
    py::array_t<int> getShapeCounts() { return arr<int>(pcp_model_get_shape_counts); }
    py::array_t<int> getIntersectionsCounter() { return arr<int>(pcp_model_get_intersections_counter); }
    py::array_t<uint64_t> getIntersections() { return arr<uint64_t>(pcp_model_get_intersections); }
    py::array_t<uint64_t> getOutersections() { return arr<uint64_t>(pcp_model_get_outersections); }
    py::array_t<uint32_t> getKeys() { return arr<uint32_t>(pcp_model_get_keys); }
    py::array_t<bool> getInsideFlag() {
        int n = 0;
        check(pcp_model_get_inside_flag(m_, nullptr, 0, &n));
        std::vector<uint8_t> tmp(n);
        if (n > 0) check(pcp_model_get_inside_flag(m_, tmp.data(), n, &n));
        py::array_t<bool> out(n);
        bool* d = out.mutable_data();
        for (int i = 0; i < n; ++i) d[i] = tmp[i] != 0;
        return out;
    }
    std::vector<int> getStartIndices() {
        int n = 0;
        check(pcp_model_get_start_indices(m_, nullptr, 0, &n));
        std::vector<int> v(n);
        if (n > 0) check(pcp_model_get_start_indices(m_, v.data(), n, &n));
        return v;
    }
    uintptr_t devicePositions() { double* p; check(pcp_model_device_positions(m_, &p)); return (uintptr_t)p; }
    uintptr_t deviceForces() { double* p; check(pcp_model_device_forces(m_, &p)); return (uintptr_t)p; }
    uintptr_t handlePtr() { return (uintptr_t)m_; }
    void setStream(uintptr_t s) { check(pcp_model_set_stream(m_, (void*)s)); }

    void setLaunchShape(int narrowBlocks, int forceBlocks) {
        check(pcp_model_set_launch_shape(m_, narrowBlocks, forceBlocks));
    }
    std::tuple<int, int> getLaunchShape() {
        int out[2];
        check(pcp_model_get_launch_shape(m_, out));
        return {out[0], out[1]};
    }
    pcp_model* raw() const { return m_; }

private:
    pcp_model* m_ = nullptr;
};

// Many independent systems minimised together (an addition: the reference
// has one system per Model).  Holds references to the Model objects so that
// they outlive the batch's use of them.
class Batch {
public:
    Batch() { check(pcp_batch_create(&b_)); }
    ~Batch() { pcp_batch_destroy(b_); }
    Batch(const Batch&) = delete;
    Batch& operator=(const Batch&) = delete;
    void add(py::object model) {
        Model& mm = model.cast<Model&>();
        check(pcp_batch_add(b_, mm.raw()));
        keep_.push_back(model);
    }
    int size() const { return (int)keep_.size(); }
    void setStreams(int n, int chunk) { check(pcp_batch_set_streams(b_, n, chunk)); }
    py::array_t<double> minimizeFIRE(int rule, double thr, double dt, int maxSteps, double dtMax,
                                     double alphaStart, double fAlpha, double fInc, double fDec,
                                     int nMin, int shakeIter) {
        std::vector<double> out(4 * keep_.size());
        {
            py::gil_scoped_release nogil;
            check(pcp_batch_minimize_fire(b_, rule, thr, dt, maxSteps, dtMax, alphaStart, fAlpha,
                                          fInc, fDec, nMin, shakeIter, out.data()));
        }
        py::array_t<double> a({(py::ssize_t)keep_.size(), (py::ssize_t)4});
        std::memcpy(a.mutable_data(), out.data(), out.size() * sizeof(double));
        return a;
    }
    py::array_t<int> autotune(int steps) {
        std::vector<int> out(2 * keep_.size());
        {
            py::gil_scoped_release nogil;
            check(pcp_batch_autotune(b_, steps, out.data()));
        }
        py::array_t<int> a({(py::ssize_t)keep_.size(), (py::ssize_t)2});
        std::memcpy(a.mutable_data(), out.data(), out.size() * sizeof(int));
        return a;
    }
    std::string report() {
        int len = 0;
        check(pcp_batch_autotune_report(b_, nullptr, 0, &len));
        std::string s(len + 1, '\0');
        check(pcp_batch_autotune_report(b_, &s[0], len + 1, &len));
        s.resize(len);
        return s;
    }

private:
    pcp_batch* b_ = nullptr;
    std::vector<py::object> keep_;
};

PYBIND11_MODULE(libpyCudaPolygon, m) {
    py::enum_<minimizerEnum>(m, "minimizerEnum")
        .value("GD", minimizerEnum::GD)
        .value("FIRE", minimizerEnum::FIRE);
    py::enum_<simControlStruct::modelEnum>(m, "modelEnum")
        .value("normal", simControlStruct::modelEnum::normal)
        .value("edgeOnly", simControlStruct::modelEnum::edgeOnly)
        .value("areaOnly", simControlStruct::modelEnum::areaOnly)
        .value("softBody", simControlStruct::modelEnum::softBody)
        .value("hybrid", simControlStruct::modelEnum::hybrid)
        .value("abnormal", simControlStruct::modelEnum::abnormal);

    py::class_<Model>(m, "Model")
        .def(py::init<int>())
        .def("initializeNeighborCells", &Model::initializeNeighborCells)
        .def("sortKeys", &Model::sortKeys)
        .def("getKeys", &Model::getKeys)
        .def("setNumVertices", &Model::setNumVertices)
        .def("setPositions", &Model::setPositions)
        .def("setForces", &Model::setForces)
        .def("setModelEnum", &Model::setModelEnum)
        .def("setStartIndices", &Model::setStartIndices)
        .def("setMaxEdgeLength", &Model::setMaxEdgeLength)
        .def("setTargetEdgeLengths", &Model::setTargetEdgeLengths)
        .def("setTargetAreas", &Model::setTargetAreas)
        .def("setStiffness", &Model::setStiffness)
        .def("setCompressibility", &Model::setCompressibility)
        .def("getStiffness", &Model::getStiffness)
        .def("getCompressibility", &Model::getCompressibility)
        .def("updatePolygonGeometry", &Model::updatePolygonGeometry)
        .def("projectForce", &Model::projectForce)
        .def("shakeProject", &Model::shakeProject, py::arg("nIter"), py::arg("tol") = 1e-15)
        .def("getLastShakeIters", &Model::getLastShakeIters)
        .def("saveTentativePositions", &Model::saveTentativePositions)
        .def("getMaxEffectiveForce", &Model::getMaxEffectiveForce)
        .def("updateNeighborCells", &Model::updateNeighborCells)
        .def("updateNeighbors", &Model::updateNeighbors)
        .def("updateValidAndCounts", &Model::updateValidAndCounts)
        .def("updateCompactedIntersections", &Model::updateCompactedIntersections)
        .def("updateOutersections", &Model::updateOutersections)
        .def("updateOverlapArea", &Model::updateOverlapArea)
        .def("updateForceEnergy", &Model::updateForceEnergy)
        .def("updatePositions", &Model::updatePositions)
        .def("resetAreas", &Model::resetAreas)
        .def("getNumVertices", &Model::getNumVertices)
        .def("getNumPolygons", &Model::getNumPolygons)
        .def("getShapeId", &Model::getShapeId)
        .def("getPositions", &Model::getPositions)
        .def("getIntersectionsCounter", &Model::getIntersectionsCounter)
        .def("getModelEnum", &Model::getModelEnum)
        .def("getStartIndices", &Model::getStartIndices)
        .def("getMaxEdgeLength", &Model::getMaxEdgeLength)
        .def("getAreas", &Model::getAreas)
        .def("getNeighborCells", &Model::getNeighborCells)
        .def("getNeighborIndices", &Model::getNeighborIndices)
        .def("getIntersections", &Model::getIntersections)
        .def("getNumIntersections", &Model::getNumIntersections)
        .def("getOutersections", &Model::getOutersections)
        .def("getNeighbors", &Model::getNeighbors)
        .def("getNumNeighbors", &Model::getNumNeighbors)
        .def("getBoxCounts", &Model::getBoxCounts)
        .def("getInsideFlag", &Model::getInsideFlag)
        .def("getPerimeters", &Model::getPerimeters)
        .def("getForces", &Model::getForces)
        .def("getTU", &Model::getTU)
        .def("getUT", &Model::getUT)
        .def("getShapeCounts", &Model::getShapeCounts)
        .def("getEnergy", &Model::getEnergy)
        .def("getConstraints", &Model::getConstraints)
        .def("getTargetEdgeLengths", &Model::getTargetEdgeLengths)
        .def("getTargetAreas", &Model::getTargetAreas)
        .def("getEdgeLengths", &Model::getEdgeLengths)
        .def("getMaxUnbalancedForce", &Model::getMaxUnbalancedForce)
        .def("getCOM", &Model::getCOM)
        .def("getOverlapArea", &Model::getOverlapArea)
        .def("resetVelocities", &Model::resetVelocities)
        .def("minimizeFIREStep", &Model::minimizeFIREStep, py::arg("dt"), py::arg("alpha"),
             py::arg("nPos"), py::arg("dtMax") = 0.1, py::arg("alphaStart") = 0.1,
             py::arg("fAlpha") = 0.99, py::arg("fInc") = 1.1, py::arg("fDec") = 0.5,
             py::arg("nMin") = 5, py::arg("shakeIter") = 5)
        .def("minimizeFIRE", &Model::minimizeFIRE, py::arg("maxForceThreshold"),
             py::arg("dtInit"), py::arg("maxSteps"), py::arg("dtMax") = 0.1,
             py::arg("alphaStart") = 0.1, py::arg("fAlpha") = 0.99, py::arg("fInc") = 1.1,
             py::arg("fDec") = 0.5, py::arg("nMin") = 5, py::arg("shakeIter") = 5)
        // additions (not in the reference's table)
        .def("xpbdProject", &Model::xpbdProject, py::arg("nIter"), py::arg("tol") = 0.0)
        .def("getVelocities", &Model::getVelocities)
        .def("getMaxNeighbors", &Model::getMaxNeighbors)
        .def("getBoxSize", &Model::getBoxSize)
        .def("getPairCount", &Model::getPairCount)
        .def("getNarrowPairTotal", &Model::getNarrowPairTotal)
        .def("getLaunchCount", &Model::getLaunchCount)
        .def("getNarrowPairCount", &Model::getNarrowPairCount)
        .def("devicePositions", &Model::devicePositions)
        .def("deviceForces", &Model::deviceForces)
        .def("handle", &Model::handlePtr)
        .def("setStream", &Model::setStream)
        .def("fireSetup", &Model::fireSetup, py::arg("maxForceThreshold"), py::arg("dtInit"),
             py::arg("maxSteps"), py::arg("dtMax") = 0.1, py::arg("alphaStart") = 0.1,
             py::arg("fAlpha") = 0.99, py::arg("fInc") = 1.1, py::arg("fDec") = 0.5,
             py::arg("nMin") = 5, py::arg("shakeIter") = 5)
        .def("minimizeFIREDevice", &Model::minimizeFIREDevice,
             py::arg("maxForceThreshold") = 1e-14, py::arg("dt") = 1e-3,
             py::arg("maxSteps") = 100000000, py::arg("dtMax") = 0.1,
             py::arg("alphaStart") = 0.1, py::arg("fAlpha") = 0.99, py::arg("fInc") = 1.1,
             py::arg("fDec") = 0.5, py::arg("nMin") = 5, py::arg("shakeIter") = 5)
        .def("fireSetStopRule", &Model::fireSetStopRule, py::arg("energyTol"),
             py::arg("stagnantLimit"))
        .def("fireRunStats", &Model::fireRunStats)
        .def("setPositionsDevice", &Model::setPositionsDevice, py::arg("ptr"), py::arg("len"))
        .def("overlapEnergyGradient", &Model::overlapEnergyGradient, py::arg("mode"),
             py::arg("search"), py::arg("outPtr"))
        .def("fireContinue", &Model::fireContinue)
        .def("fireStatus", &Model::fireStatus)
        .def("contactsStage", &Model::contactsStage)
        .def("setLaunchShape", &Model::setLaunchShape, py::arg("narrowBlocks"),
             py::arg("forceBlocks"))
        .def("getLaunchShape", &Model::getLaunchShape);

    py::class_<Batch>(m, "Batch")
        .def(py::init<>())
        .def("add", &Batch::add)
        .def("size", &Batch::size)
        .def("setStreams", &Batch::setStreams, py::arg("streams"), py::arg("chunkSteps"))
        .def("minimizeFIRE", &Batch::minimizeFIRE, py::arg("rule") = 1,
             py::arg("maxForceThreshold") = 1e-14, py::arg("dt") = 1e-3,
             py::arg("maxSteps") = 100000000, py::arg("dtMax") = 0.1,
             py::arg("alphaStart") = 0.1, py::arg("fAlpha") = 0.99, py::arg("fInc") = 1.1,
             py::arg("fDec") = 0.5, py::arg("nMin") = 5, py::arg("shakeIter") = 5)
        .def("autotune", &Batch::autotune, py::arg("steps") = 8)
        .def("report", &Batch::report);
}
