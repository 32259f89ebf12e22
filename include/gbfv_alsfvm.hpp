// gbfv_alsfvm.hpp: C++ host adapters that present the gbfv C ABI through the
// interfaces alsfvm's hot path is written against, for the "gb300" platform.
//
// Each class mirrors one reference interface (names, argument meaning, error
// behaviour: failures throw std::runtime_error with the library's message, as
// the reference's THROW does, alsutils/include/alsutils/error/Exception.hpp:27):
//
//   Memory          memory::Memory<real>        alsfvm/include/alsfvm/memory/Memory.hpp:27-343
//   Volume          volume::Volume              alsfvm/include/alsfvm/volume/Volume.hpp:30-343
//   Grid            grid::Grid                  alsfvm/include/alsfvm/grid/Grid.hpp:40-80
//   NumericalFlux   numflux::NumericalFlux      alsfvm/include/alsfvm/numflux/NumericalFlux.hpp:44-52
//   Reconstruction  reconstruction::Reconstruction
//                                               alsfvm/include/alsfvm/reconstruction/Reconstruction.hpp:46-58
//   Boundary        boundary::Boundary          alsfvm/include/alsfvm/boundary/Boundary.hpp:30-31
//   CellComputer    equation::CellComputer      alsfvm/include/alsfvm/equation/CellComputer.hpp:35-70
//   Simulator       simulator::Simulator        alsfvm/src/simulator/Simulator.cpp:26-214
//   MeanVariance    alsuq::stats::MeanVariance  alsuq/src/stats/MeanVariance.cpp:30-67
//
// Volumes of this platform live in device memory as one block of nvar padded
// arrays (the layout include/gbfv.h documents). Link with libgbfv.so and the
// CUDA runtime.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbfv.h"

namespace gbfv_alsfvm {

using real = double;
struct ivec3 {
    int x = 0, y = 0, z = 0;
    ivec3() = default;
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    int operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
struct rvec3 {
    real x = 0, y = 0, z = 0;
    rvec3() = default;
    rvec3(real a, real b, real c) : x(a), y(b), z(c) {}
    real operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

inline void check(int rc) {
    if (rc != GBFV_OK) throw std::runtime_error(std::string("gbfv: ") + gbfv_last_error());
}
inline void check_cuda(cudaError_t e) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA: ") + cudaGetErrorString(e));
}

// The names of one configuration as in the reference's XML (<fvm> nodes).
struct Scheme {
    std::string equation = "euler2", flux = "hll3", reconstruction = "weno2", integrator = "rungekutta3",
                boundary = "periodic";
    real gamma = 1.4, cfl = 0.4;
    int precision = GBFV_FP64;
};

class Grid {
public:
    // origin (lower corner), top (upper corner), cells per dimension
    Grid(rvec3 origin, rvec3 top, ivec3 dimensions) : origin(origin), top(top), dims(dimensions) {}
    const ivec3& getDimensions() const { return dims; }
    rvec3 getOrigin() const { return origin; }
    rvec3 getTop() const { return top; }
    // inactive dimensions get length 1 (alsfvm/src/grid/Grid.cpp:24-42)
    rvec3 getCellLengths() const {
        return rvec3((top.x - origin.x) / dims.x, dims.y == 1 ? 1.0 : (top.y - origin.y) / dims.y,
                     dims.z == 1 ? 1.0 : (top.z - origin.z) / dims.z);
    }
    int getActiveDimension() const { return dims.z > 1 ? 3 : (dims.y > 1 ? 2 : 1); }

private:
    rvec3 origin, top;
    ivec3 dims;
};

// One conserved variable's padded array inside a Volume's device block, with
// Memory<real>'s arithmetic on the device (the operations the reference's
// integrators and MeanVariance use, alsfvm/include/alsfvm/memory/
// Memory.hpp:166-302), each synchronous on return.
class Memory {
public:
    Memory(real* dev, size_t size) : dev(dev), size(size) {}
    real* getPointer() { return dev; }
    const real* getPointer() const { return dev; }
    size_t getSize() const { return size; }
    bool isOnHost() const { return false; }
    void copyToHost(real* host, size_t count) const {
        check_cuda(cudaMemcpy(host, dev, count * sizeof(real), cudaMemcpyDeviceToHost));
    }
    void copyFromHost(const real* host, size_t count) {
        check_cuda(cudaMemcpy(dev, host, count * sizeof(real), cudaMemcpyHostToDevice));
    }
    void operator+=(const Memory& o) { binary(GBFV_MEMORY_ADD, o); }
    void operator-=(const Memory& o) { binary(GBFV_MEMORY_SUBTRACT, o); }
    void operator*=(const Memory& o) { binary(GBFV_MEMORY_MULTIPLY, o); }
    void operator/=(const Memory& o) { binary(GBFV_MEMORY_DIVIDE, o); }
    void operator+=(real x) { sync(gbfv_memory_op_scalar(GBFV_MEMORY_ADD, dev, x, n(), GBFV_FP64, nullptr)); }
    void operator-=(real x) { sync(gbfv_memory_op_scalar(GBFV_MEMORY_SUBTRACT, dev, x, n(), GBFV_FP64, nullptr)); }
    void operator*=(real x) { sync(gbfv_memory_op_scalar(GBFV_MEMORY_MULTIPLY, dev, x, n(), GBFV_FP64, nullptr)); }
    void operator/=(real x) { sync(gbfv_memory_op_scalar(GBFV_MEMORY_DIVIDE, dev, x, n(), GBFV_FP64, nullptr)); }
    void makeZero() { sync(gbfv_memory_make_zero(dev, n(), GBFV_FP64, nullptr)); }
    void addLinearCombination(real a1, real a2, const Memory& v2, real a3, const Memory& v3, real a4,
                              const Memory& v4, real a5, const Memory& v5) {
        sync(gbfv_memory_add_linear_combination(dev, a1, a2, v2.dev, a3, v3.dev, a4, v4.dev, a5, v5.dev, n(),
                                                GBFV_FP64, nullptr));
    }
    void addPower(const Memory& o, double power, double factor = 1.0) {
        same_size(o);
        sync(gbfv_memory_add_power(dev, o.dev, power, factor, n(), GBFV_FP64, nullptr));
    }
    void subtractPower(const Memory& o, double power) {
        same_size(o);
        sync(gbfv_memory_subtract_power(dev, o.dev, power, n(), GBFV_FP64, nullptr));
    }

private:
    real* dev;
    size_t size;
    long long n() const { return (long long)size; }
    void same_size(const Memory& o) const {
        if (o.size != size) throw std::runtime_error("Memory size not the same");
    }
    static void sync(int rc) {
        check(rc);
        check_cuda(cudaStreamSynchronize(nullptr));
    }
    void binary(int op, const Memory& o) {
        same_size(o);
        sync(gbfv_memory_op(op, dev, o.dev, n(), GBFV_FP64, nullptr));
    }
};

class Volume {
public:
    Volume(const std::string& equation, ivec3 n, int ghosts) : n(n), ghosts(ghosts) {
        nvar = gbfv_num_variables(equation.c_str());
        if (nvar < 0) check(nvar);
        const int dim = n.z > 1 ? 3 : (n.y > 1 ? 2 : 1);
        t = ivec3(n.x + 2 * ghosts, dim > 1 ? n.y + 2 * ghosts : n.y, dim > 2 ? n.z + 2 * ghosts : n.z);
        total = (size_t)t.x * t.y * t.z;
        real* p = nullptr;
        check_cuda(cudaMalloc(&p, nvar * total * sizeof(real)));
        block.reset(p, [](real* q) { cudaFree(q); });
        check_cuda(cudaMemset(p, 0, nvar * total * sizeof(real)));
        for (int k = 0; k < nvar; ++k) areas.emplace_back(p + k * total, total);
    }
    size_t getNumberOfVariables() const { return (size_t)nvar; }
    Memory& getScalarMemoryArea(size_t i) { return areas.at(i); }
    const Memory& getScalarMemoryArea(size_t i) const { return areas.at(i); }
    size_t getTotalNumberOfXCells() const { return (size_t)t.x; }
    size_t getTotalNumberOfYCells() const { return (size_t)t.y; }
    size_t getTotalNumberOfZCells() const { return (size_t)t.z; }
    size_t getNumberOfXCells() const { return (size_t)n.x; }
    size_t getNumberOfYCells() const { return (size_t)n.y; }
    size_t getNumberOfZCells() const { return (size_t)n.z; }
    int getNumberOfGhostCells() const { return ghosts; }
    size_t getTotalSize() const { return total; }
    void* data() { return block.get(); }
    const void* data() const { return block.get(); }
    void makeZero() { check_cuda(cudaMemset(block.get(), 0, nvar * total * sizeof(real))); }
    // padded host copy, nvar * total values
    std::vector<real> toHost() const {
        std::vector<real> h(nvar * total);
        check_cuda(cudaMemcpy(h.data(), block.get(), h.size() * sizeof(real), cudaMemcpyDeviceToHost));
        return h;
    }
    void fromHost(const std::vector<real>& h) {
        if (h.size() != nvar * total) throw std::runtime_error("Volume::fromHost: size mismatch");
        check_cuda(cudaMemcpy(block.get(), h.data(), h.size() * sizeof(real), cudaMemcpyHostToDevice));
    }

private:
    ivec3 n, t;
    int ghosts, nvar;
    size_t total;
    std::shared_ptr<real> block;
    std::vector<Memory> areas;
};

namespace detail {
inline gbfv_desc describe(const Scheme& s, const Grid& g) {
    gbfv_desc d{};
    d.equation = s.equation.c_str();
    d.flux = s.flux.c_str();
    d.reconstruction = s.reconstruction.c_str();
    d.integrator = s.integrator.c_str();
    d.boundary = s.boundary.c_str();
    d.n[0] = g.getDimensions().x;
    d.n[1] = g.getDimensions().y;
    d.n[2] = g.getDimensions().z;
    const rvec3 o = g.getOrigin(), t = g.getTop();
    d.lower[0] = o.x; d.lower[1] = o.y; d.lower[2] = o.z;
    d.upper[0] = t.x; d.upper[1] = t.y; d.upper[2] = t.z;
    d.gamma = s.gamma;
    d.cfl = s.cfl;
    d.precision = s.precision;
    return d;
}
struct SolverHandle {
    gbfv_solver* h = nullptr;
    SolverHandle(const Scheme& s, const Grid& g) {
        gbfv_desc d = describe(s, g);
        check(gbfv_create(&d, &h));
    }
    ~SolverHandle() { gbfv_destroy(h); }
    SolverHandle(const SolverHandle&) = delete;
    SolverHandle& operator=(const SolverHandle&) = delete;
};
}  // namespace detail

// NumericalFlux::computeFlux: out = sum_d (F_{i-1/2} - F_{i+1/2}) on the cells
// of the region [start, n + end) (the whole interior by default), unscaled,
// the other cells of out unchanged; waveSpeed = per-direction maximum speed
// of the region's faces. A stream (cudaStream_t) may be given; the call is
// synchronous on return.
class NumericalFlux {
public:
    NumericalFlux(const Scheme& s, const Grid& g) : scheme(s), solver(s, g) {}
    void computeFlux(const Volume& conservedVariables, rvec3& waveSpeed, bool /*computeWaveSpeed*/, Volume& output,
                     const ivec3& start = ivec3(), const ivec3& end = ivec3(), void* stream = nullptr) {
        const size_t nv = conservedVariables.getNumberOfVariables();
        std::vector<const void*> in(nv);
        std::vector<void*> out(nv);
        for (size_t k = 0; k < nv; ++k) {
            in[k] = conservedVariables.getScalarMemoryArea(k).getPointer();
            out[k] = output.getScalarMemoryArea(k).getPointer();
        }
        const int s[3] = {start.x, start.y, start.z}, e[3] = {end.x, end.y, end.z};
        double ws[3];
        check(gbfv_compute_flux_region(solver.h, in.data(), out.data(), ws, s, e, stream));
        waveSpeed = rvec3(ws[0], ws[1], ws[2]);
    }
    size_t getNumberOfGhostCells() const { return (size_t)gbfv_ghost_cells(scheme.reconstruction.c_str()); }

private:
    Scheme scheme;
    detail::SolverHandle solver;
};

class Reconstruction {
public:
    Reconstruction(const Scheme& s, const Grid& g) : scheme(s), solver(s, g) {}
    // indicatorVariable: the reference always passes 0 (rho / u)
    void performReconstruction(const Volume& inputVariables, size_t direction, size_t indicatorVariable,
                               Volume& leftOut, Volume& rightOut, const ivec3& = ivec3(), const ivec3& = ivec3()) {
        if (indicatorVariable != 0) throw std::runtime_error("Only indicator variable 0 is supported");
        check(gbfv_reconstruct(solver.h, (int)direction, inputVariables.data(), leftOut.data(), rightOut.data()));
    }
    size_t getNumberOfGhostCells() const { return (size_t)gbfv_ghost_cells(scheme.reconstruction.c_str()); }

private:
    Scheme scheme;
    detail::SolverHandle solver;
};

class Boundary {
public:
    Boundary(const Scheme& s, const Grid& g) : solver(s, g) {}
    void applyBoundaryConditions(Volume& volume, const Grid&) { check(gbfv_apply_boundary(solver.h, volume.data())); }

private:
    detail::SolverHandle solver;
};

class CellComputer {
public:
    CellComputer(const Scheme& s, const Grid& g) : solver(s, g) {}
    bool obeysConstraints(const Volume& conservedVariables) {
        int ok = 0;
        check(gbfv_obeys_constraints(solver.h, conservedVariables.data(), &ok));
        return ok != 0;
    }

private:
    detail::SolverHandle solver;
};

// Simulator: the step loop with the state on the device. setInitialValue
// takes interior primitive values (rho, u..., p) or (u), x fastest.
class Simulator {
public:
    Simulator(const Scheme& s, const Grid& g, real endTime, int numberOfSaves = 0)
        : scheme(s), grid(g), endTime(endTime), numberOfSaves(numberOfSaves), solver(s, g) {}
    void setInitialValue(const std::vector<real>& primitiveInterior) {
        check(gbfv_set_primitive(solver.h, primitiveInterior.data()));
    }
    void setSimulationState(const std::vector<real>& conservedPadded) {
        check(gbfv_set_state(solver.h, conservedPadded.data()));
    }
    bool atEnd() { return getCurrentTime() >= endTime; }
    // incrementSolution + checkConstraints: throws when the state breaks them
    void performStep() { check(gbfv_advance(solver.h, endTime, numberOfSaves, 1)); }
    // the alsvinncli loop in one call (dt stays on the device)
    void run() { check(gbfv_advance(solver.h, endTime, numberOfSaves, 0)); }
    real getCurrentTime() {
        double t = 0;
        check(gbfv_time(solver.h, &t, nullptr, nullptr));
        return t;
    }
    long long getNumberOfStepsPerformed() {
        long long s = 0;
        check(gbfv_time(solver.h, nullptr, &s, nullptr));
        return s;
    }
    real getEndTime() const { return endTime; }
    std::vector<real> getConservedState() {
        long long total = 0;
        check(gbfv_extents(solver.h, nullptr, &total));
        std::vector<real> h((size_t)gbfv_num_variables(scheme.equation.c_str()) * (size_t)total);
        check(gbfv_get_state(solver.h, h.data()));
        return h;
    }
    const Grid& getGrid() const { return grid; }

private:
    Scheme scheme;
    Grid grid;
    real endTime;
    int numberOfSaves;
    detail::SolverHandle solver;
};

// MeanVariance over the samples handed to computeStatistics (FP64 Welford on
// the device); finalizeStatistics gives mean and (population) variance as in
// the reference after combineStatistics on one rank.
class MeanVariance {
public:
    explicit MeanVariance(size_t count) {
        check(gbfv_stats_create((long long)count, &st));
        this->count = count;
    }
    ~MeanVariance() { gbfv_stats_destroy(st); }
    MeanVariance(const MeanVariance&) = delete;
    MeanVariance& operator=(const MeanVariance&) = delete;
    void computeStatistics(const Volume& conservedVariables) {
        check(gbfv_stats_add_device(st, conservedVariables.data(), GBFV_FP64));
    }
    // combine with another rank's accumulator (Chan et al. merge)
    void combineStatistics(const MeanVariance& other) { check(gbfv_stats_merge(st, other.st)); }
    void finalizeStatistics(std::vector<real>& mean, std::vector<real>& variance) {
        mean.resize(count);
        variance.resize(count);
        long long n = 0;
        check(gbfv_stats_result(st, mean.data(), variance.data(), &n));
    }

private:
    gbfv_stats* st = nullptr;
    size_t count = 0;
};

}  // namespace gbfv_alsfvm
