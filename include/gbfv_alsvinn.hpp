// gbfv_alsvinn.hpp: the "gb300" platform for alsvinn itself.
//
// Classes derived from alsvinn's own abstract interfaces, compiled inside
// alsvinn's build (its include paths alsfvm/include, alsutils/include,
// alsuq/include, plus this directory and the CUDA runtime's headers) and
// linked with libgbfv.so. With them registered in alsvinn's factories as
// platform "gb300", the reference's unchanged Simulator, ConservedSystem,
// Runge-Kutta integrators and alsuq statistics run on GB300 device state:
//
//   GB300Memory<real>      memory::Memory<real>             alsfvm/include/alsfvm/memory/Memory.hpp:27-343
//   GB300NumericalFlux     numflux::NumericalFlux           alsfvm/include/alsfvm/numflux/NumericalFlux.hpp:44-52
//   GB300Reconstruction    reconstruction::Reconstruction   alsfvm/include/alsfvm/reconstruction/Reconstruction.hpp:46-58
//   GB300Boundary          boundary::Boundary               alsfvm/include/alsfvm/boundary/Boundary.hpp:30-31
//   GB300CellComputer      equation::CellComputer           alsfvm/include/alsfvm/equation/CellComputer.hpp:35-70
//
// alsuq's MeanVariance needs no class of its own: it works through Memory's
// operator+=, addPower and subtractPower, which GB300Memory runs on the
// device, so REGISTER_STATISTICS(gb300, meanvar, MeanVariance) registers the
// reference's own class for this platform.
//
// Volumes keep one device array per variable (one GB300Memory each, as the
// reference's Volume holds them); the operator calls pass those arrays to the
// gbfv_*_vars / gbfv_compute_flux_region entry points. Every call is
// synchronous on return, as the reference's CUDA path is. Failures throw
// std::runtime_error through the reference's THROW
// (alsutils/include/alsutils/error/Exception.hpp:27).
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "alsfvm/boundary/Boundary.hpp"
#include "alsfvm/equation/CellComputer.hpp"
#include "alsfvm/grid/Grid.hpp"
#include "alsfvm/memory/HostMemory.hpp"
#include "alsfvm/memory/Memory.hpp"
#include "alsfvm/numflux/NumericalFlux.hpp"
#include "alsfvm/reconstruction/Reconstruction.hpp"
#include "alsfvm/volume/Volume.hpp"
#include "alsutils/error/Exception.hpp"
#include "gbfv.h"

namespace alsfvm {
namespace gb300 {

inline void check(int rc) {
    if (rc != GBFV_OK) THROW("gbfv: " << gbfv_last_error());
}
inline void check_cuda(cudaError_t e) {
    if (e != cudaSuccess) THROW("CUDA: " << cudaGetErrorString(e));
}

template <class T> struct precision_of;
template <> struct precision_of<double> { static constexpr int value = GBFV_FP64; };
template <> struct precision_of<float> { static constexpr int value = GBFV_FP32; };

// Device memory of one variable: nx * ny * nz values (padded extents).
template <class T>
class GB300Memory : public memory::Memory<T> {
public:
    GB300Memory(size_t nx, size_t ny, size_t nz) : memory::Memory<T>(nx, ny, nz) {
        check_cuda(cudaMalloc(&dev, bytes()));
        check_cuda(cudaMemset(dev, 0, bytes()));
    }
    ~GB300Memory() override { cudaFree(dev); }
    GB300Memory(const GB300Memory&) = delete;
    GB300Memory& operator=(const GB300Memory&) = delete;

    std::shared_ptr<memory::Memory<T> > makeInstance() const override {
        return std::make_shared<GB300Memory<T> >(this->nx, this->ny, this->nz);
    }
    void copyFrom(const memory::Memory<T>& other) override {
        if (other.getSize() != this->getSize()) THROW("GB300Memory::copyFrom: size mismatch");
        check_cuda(cudaMemcpy(dev, other.getPointer(), bytes(),
                              other.isOnHost() ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice));
    }
    bool isOnHost() const override { return false; }
    T* getPointer() override { return dev; }
    const T* getPointer() const override { return dev; }
    void copyToHost(T* buffer, size_t length) const override {
        if (length < this->getSize()) THROW("GB300Memory::copyToHost: buffer too small");
        check_cuda(cudaMemcpy(buffer, dev, bytes(), cudaMemcpyDeviceToHost));
    }
    void copyFromHost(const T* buffer, size_t length) override {
        const size_t n = length < this->getSize() ? length : this->getSize();
        check_cuda(cudaMemcpy(dev, buffer, n * sizeof(T), cudaMemcpyHostToDevice));
    }

    void operator+=(const memory::Memory<T>& o) override { binary(GBFV_MEMORY_ADD, o); }
    void operator*=(const memory::Memory<T>& o) override { binary(GBFV_MEMORY_MULTIPLY, o); }
    void operator-=(const memory::Memory<T>& o) override { binary(GBFV_MEMORY_SUBTRACT, o); }
    void operator/=(const memory::Memory<T>& o) override { binary(GBFV_MEMORY_DIVIDE, o); }
    void operator+=(real s) override { scalar(GBFV_MEMORY_ADD, s); }
    void operator*=(real s) override { scalar(GBFV_MEMORY_MULTIPLY, s); }
    void operator-=(real s) override { scalar(GBFV_MEMORY_SUBTRACT, s); }
    void operator/=(real s) override { scalar(GBFV_MEMORY_DIVIDE, s); }
    void makeZero() override { sync(gbfv_memory_make_zero(dev, count(), precision_of<T>::value, nullptr)); }

    // the region copied out through a host copy of the whole array, as the
    // reference's CudaMemory does (alsfvm/src/cuda/CudaMemory.cpp)
    void copyInternalCells(size_t startX, size_t endX, size_t startY, size_t endY, size_t startZ, size_t endZ,
                           T* output, size_t outputSize) override {
        std::vector<T> host(this->getSize());
        copyToHost(host.data(), host.size());
        const size_t cx = endX - startX, cy = endY - startY, cz = endZ - startZ;
        if (cx * cy * cz > outputSize) THROW("GB300Memory::copyInternalCells: output too small");
        for (size_t z = 0; z < cz; ++z)
            for (size_t y = 0; y < cy; ++y)
                for (size_t x = 0; x < cx; ++x)
                    output[(z * cy + y) * cx + x] =
                        host[((startZ + z) * this->ny + (startY + y)) * this->nx + (startX + x)];
    }

    void addLinearCombination(T a1, T a2, const memory::Memory<T>& v2, T a3, const memory::Memory<T>& v3, T a4,
                              const memory::Memory<T>& v4, T a5, const memory::Memory<T>& v5) override {
        on_device(v2);
        on_device(v3);
        on_device(v4);
        on_device(v5);
        sync(gbfv_memory_add_linear_combination(dev, a1, a2, v2.getPointer(), a3, v3.getPointer(), a4,
                                                v4.getPointer(), a5, v5.getPointer(), count(),
                                                precision_of<T>::value, nullptr));
    }
    void addPower(const memory::Memory<T>& o, double power) override { addPower(o, power, 1.0); }
    void addPower(const memory::Memory<T>& o, double power, double factor) override {
        on_device(o);
        sync(gbfv_memory_add_power(dev, o.getPointer(), power, factor, count(), precision_of<T>::value, nullptr));
    }
    void subtractPower(const memory::Memory<T>& o, double power) override {
        on_device(o);
        sync(gbfv_memory_subtract_power(dev, o.getPointer(), power, count(), precision_of<T>::value, nullptr));
    }

    std::shared_ptr<memory::Memory<T> > getHostMemory() override {
        auto h = std::make_shared<memory::HostMemory<T> >(this->nx, this->ny, this->nz);
        copyToHost(h->getPointer(), h->getSize());
        return h;
    }
    const std::shared_ptr<const memory::Memory<T> > getHostMemory() const override {
        auto h = std::make_shared<memory::HostMemory<T> >(this->nx, this->ny, this->nz);
        copyToHost(h->getPointer(), h->getSize());
        return h;
    }

    real getTotalVariation(int p, const ivec3& start, const ivec3& end) const override {
        return total_variation(-1, p, start, end);
    }
    real getTotalVariation(int direction, int p, const ivec3& start, const ivec3& end) const override {
        return total_variation(direction, p, start, end);
    }

private:
    T* dev = nullptr;
    size_t bytes() const { return this->nx * this->ny * this->nz * sizeof(T); }
    long long count() const { return (long long)(this->nx * this->ny * this->nz); }
    void on_device(const memory::Memory<T>& o) const {
        if (o.isOnHost()) THROW("GB300Memory: the other memory area is on the host");
        if (o.getSize() != this->getSize()) THROW("GB300Memory: memory size not the same");
    }
    static void sync(int rc) {
        check(rc);
        check_cuda(cudaStreamSynchronize(nullptr));
    }
    void binary(int op, const memory::Memory<T>& o) {
        on_device(o);
        sync(gbfv_memory_op(op, dev, o.getPointer(), count(), precision_of<T>::value, nullptr));
    }
    void scalar(int op, real s) { sync(gbfv_memory_op_scalar(op, dev, s, count(), precision_of<T>::value, nullptr)); }
    real total_variation(int direction, int p, const ivec3& start, const ivec3& end) const {
        const int ext[3] = {(int)this->nx, (int)this->ny, (int)this->nz};
        const int s[3] = {start.x, start.y, start.z}, e[3] = {end.x, end.y, end.z};
        double r = 0;
        check(gbfv_memory_total_variation(dev, ext, p, direction, s, e, precision_of<T>::value, &r, nullptr));
        return (real)r;
    }
};

// The device arrays of a volume's variables (every one must be device memory).
inline std::vector<const void*> arrays_of(const volume::Volume& v) {
    std::vector<const void*> a(v.getNumberOfVariables());
    for (size_t k = 0; k < a.size(); ++k) {
        auto m = v.getScalarMemoryArea(k);
        if (m->isOnHost()) THROW("gb300: volume variable " << k << " is not in device memory");
        a[k] = m->getPointer();
    }
    return a;
}
inline std::vector<void*> arrays_of(volume::Volume& v) {
    std::vector<void*> a(v.getNumberOfVariables());
    for (size_t k = 0; k < a.size(); ++k) {
        auto m = v.getScalarMemoryArea(k);
        if (m->isOnHost()) THROW("gb300: volume variable " << k << " is not in device memory");
        a[k] = m->getPointer();
    }
    return a;
}

// The names of one configuration as in alsvinn's XML (<fvm> nodes).
struct Scheme {
    std::string equation, flux, reconstruction, boundary;
    real gamma = 1.4;
};

// A gbfv solver for one grid and scheme: the handle the operator calls use.
class Solver {
public:
    Solver(const Scheme& s, const grid::Grid& g) : names(s) {
        gbfv_desc d{};
        d.equation = names.equation.c_str();
        d.flux = names.flux.c_str();
        d.reconstruction = names.reconstruction.c_str();
        d.integrator = "rungekutta3";  // operator calls do not step
        d.boundary = names.boundary.c_str();
        const ivec3 n = g.getDimensions();
        const rvec3 lo = g.getOrigin(), hi = g.getTop();
        for (int k = 0; k < 3; ++k) {
            d.n[k] = n[k];
            d.lower[k] = lo[k];
            d.upper[k] = hi[k];
        }
        d.gamma = names.gamma;
        d.cfl = 0.5;
        d.precision = precision_of<real>::value;
        check(gbfv_create(&d, &h));
    }
    ~Solver() { gbfv_destroy(h); }
    Solver(const Solver&) = delete;
    Solver& operator=(const Solver&) = delete;
    gbfv_solver* get() const { return h; }
    const Scheme& scheme() const { return names; }

private:
    Scheme names;
    gbfv_solver* h = nullptr;
};

class GB300NumericalFlux : public numflux::NumericalFlux {
public:
    GB300NumericalFlux(const Scheme& s, const grid::Grid& g) : solver(s, g) {}
    // out gets sum_d (F_{i-1/2} - F_{i+1/2}) on the cells of the region only;
    // waveSpeed the maximum face speed per direction over the region's faces
    void computeFlux(const volume::Volume& conservedVariables, rvec3& waveSpeed, bool /*computeWaveSpeed*/,
                     volume::Volume& output, const ivec3& start = {0, 0, 0},
                     const ivec3& end = {0, 0, 0}) override {
        auto in = arrays_of(conservedVariables);
        auto out = arrays_of(output);
        const int s[3] = {start.x, start.y, start.z}, e[3] = {end.x, end.y, end.z};
        double ws[3];
        check(gbfv_compute_flux_region(solver.get(), in.data(), out.data(), ws, s, e, nullptr));
        waveSpeed = rvec3(ws[0], ws[1], ws[2]);
    }
    size_t getNumberOfGhostCells() override {
        return (size_t)gbfv_ghost_cells(solver.scheme().reconstruction.c_str());
    }

private:
    Solver solver;
};

class GB300Reconstruction : public reconstruction::Reconstruction {
public:
    GB300Reconstruction(const Scheme& s, const grid::Grid& g) : solver(s, g) {}
    // the indicator variable is variable 0 (rho or u), as every reference
    // caller passes it
    void performReconstruction(const volume::Volume& inputVariables, size_t direction, size_t indicatorVariable,
                               volume::Volume& leftOut, volume::Volume& rightOut, const ivec3& start = {0, 0, 0},
                               const ivec3& end = {0, 0, 0}) override {
        if (indicatorVariable != 0) THROW("gb300: the indicator variable must be 0");
        auto in = arrays_of(inputVariables);
        auto l = arrays_of(leftOut);
        auto r = arrays_of(rightOut);
        const int s[3] = {start.x, start.y, start.z}, e[3] = {end.x, end.y, end.z};
        check(gbfv_reconstruct_vars(solver.get(), (int)direction, in.data(), l.data(), r.data(), s, e, nullptr));
    }
    size_t getNumberOfGhostCells() override {
        return (size_t)gbfv_ghost_cells(solver.scheme().reconstruction.c_str());
    }

private:
    Solver solver;
};

class GB300Boundary : public boundary::Boundary {
public:
    GB300Boundary(const Scheme& s, const grid::Grid& g) : solver(s, g) {}
    void applyBoundaryConditions(volume::Volume& volume, const grid::Grid&) override {
        auto v = arrays_of(volume);
        check(gbfv_apply_boundary_vars(solver.get(), v.data(), nullptr));
    }

private:
    Solver solver;
};

class GB300CellComputer : public equation::CellComputer {
public:
    GB300CellComputer(const Scheme& s, const grid::Grid& g) : solver(s, g) {}
    void computeExtraVariables(const volume::Volume& conservedVariables, volume::Volume& extraVariables) override {
        auto in = arrays_of(conservedVariables);
        auto out = arrays_of(extraVariables);
        check(gbfv_extra_variables_vars(solver.get(), in.data(), out.data(), nullptr));
    }
    real computeMaxWaveSpeed(const volume::Volume& conservedVariables, size_t direction) override {
        auto in = arrays_of(conservedVariables);
        double w = 0;
        check(gbfv_max_wave_speed_vars(solver.get(), in.data(), (int)direction, &w, nullptr));
        return (real)w;
    }
    bool obeysConstraints(const volume::Volume& conservedVariables) override {
        auto in = arrays_of(conservedVariables);
        int ok = 0;
        check(gbfv_obeys_constraints_vars(solver.get(), in.data(), &ok, nullptr));
        return ok != 0;
    }
    void computeFromPrimitive(const volume::Volume& primitiveVariables, volume::Volume& conservedVariables) override {
        auto in = arrays_of(primitiveVariables);
        auto out = arrays_of(conservedVariables);
        check(gbfv_prim_to_cons_vars(solver.get(), in.data(), out.data(), nullptr));
    }

private:
    Solver solver;
};

}  // namespace gb300
}  // namespace alsfvm
