// C driver over the reference's own CPU implementation (oracle build only).
//
// Test infrastructure: this file is compiled together with the unmodified
// reference sources by the Makefile beside it into oracle/_ref/libalsref.so.
// It is used to generate golden fixtures and to validate the C restatement in
// oracle/fvoracle.c. It is never part of the product.
//
// Every entry point builds the reference objects through the reference's own
// factories, the same way alsvinncli does (alsfvm/src/config/SimulatorSetup.cpp:
// 171-229), and exchanges state as plain padded, x-fastest double arrays, one per
// conserved variable (alsfvm/include/alsfvm/memory/View.hpp:116-118).

#include "alsfvm/DeviceConfiguration.hpp"
#include "alsfvm/boundary/BoundaryFactory.hpp"
#include "alsfvm/diffusion/NoDiffusion.hpp"
#include "alsfvm/equation/CellComputerFactory.hpp"
#include "alsfvm/equation/euler/EulerParameters.hpp"
#include "alsfvm/functional/FunctionalFactory.hpp"
#include "alsfvm/functional/structure_common.hpp"
#include "alsfvm/grid/Grid.hpp"
#include "alsfvm/init/InitialData.hpp"
#include "alsfvm/integrator/IntegratorFactory.hpp"
#include "alsfvm/io/FixedIntervalWriter.hpp"
#include "alsfvm/memory/MemoryFactory.hpp"
#include "alsfvm/numflux/NumericalFluxFactory.hpp"
#include "alsfvm/reconstruction/ReconstructionFactory.hpp"
#include "alsfvm/simulator/ConservedSystem.hpp"
#include "alsfvm/simulator/Simulator.hpp"
#include "alsfvm/simulator/SimulatorParameters.hpp"
#include "alsfvm/volume/VolumeFactory.hpp"
#include "alsfvm/mpi/RequestContainer.hpp"
#include "alsuq/distribution/Uniform.hpp"
#include "alsuq/generator/STLMersenne.hpp"
#include "alsuq/mpi/Configuration.hpp"
#include "alsuq/stats/MeanVariance.hpp"
#include "alsuq/stats/StructureBasic.hpp"
#include "alsuq/stats/StatisticsParameters.hpp"
#include "alsutils/debug/stacktrace.hpp"

#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <omp.h>
#include <string>
#include <vector>

// Two definitions the linked subset of the reference needs but whose sources
// sit in translation units outside it (stack traces, MPI request waits).
namespace alsutils {
namespace debug {
std::string getLongStacktrace() { return ""; }
}
}
namespace alsfvm {
namespace mpi {
void RequestContainer::waitForAll() {}
}
}

using namespace alsfvm;

namespace {

thread_local std::string g_error;

int nvar_of(const std::string& eq) {
    if (eq == "euler1") return 3;
    if (eq == "euler2") return 4;
    if (eq == "euler3") return 5;
    if (eq == "burgers") return 1;
    return -1;
}

struct Setup {
    std::string equation, flux, recon, boundary, integrator;
    int n[3];
    rvec3 lower, upper;
    double gamma, cfl;
    std::shared_ptr<DeviceConfiguration> device;
    std::shared_ptr<memory::MemoryFactory> memory;
    std::shared_ptr<simulator::SimulatorParameters> params;
    std::shared_ptr<grid::Grid> grid;

    Setup(const char* eq, const char* fl, const char* rc, const char* bc, const char* integ,
        const int dims[3], const double lo[3], const double hi[3], double gamma_, double cfl_)
        : equation(eq), flux(fl), recon(rc), boundary(bc), integrator(integ ? integ : ""),
          gamma(gamma_), cfl(cfl_) {
        for (int d = 0; d < 3; ++d) n[d] = dims[d];
        lower = rvec3(lo[0], lo[1], lo[2]);
        upper = rvec3(hi[0], hi[1], hi[2]);
        device = std::make_shared<DeviceConfiguration>("cpu");
        memory = std::make_shared<memory::MemoryFactory>(device);
        params = std::make_shared<simulator::SimulatorParameters>(equation, "cpu");
        params->setCFLNumber(cfl);
        if (equation.rfind("euler", 0) == 0) {
            static_cast<equation::euler::EulerParameters&>(params->getEquationParameters())
                .setGamma(gamma);
        }
        auto bcs = boundary == "periodic" ? boundary::allPeriodic() : boundary::allNeumann();
        grid = std::make_shared<grid::Grid>(lower, upper, ivec3(n[0], n[1], n[2]), bcs);
    }
};

// Copies interior primitive values given by the caller into the primitive
// volume and converts them with the reference's CellComputer, the path the
// reference's Python initial data takes (alsfvm/src/init/PythonInitialData.cpp).
class ArrayInitialData : public init::InitialData {
public:
    ArrayInitialData(const double* prim, int nvar, const int n[3]) : prim(prim), nvar(nvar) {
        for (int d = 0; d < 3; ++d) this->n[d] = n[d];
    }
    void setInitialData(volume::Volume& conserved, volume::Volume& primitive,
        equation::CellComputer& cellComputer, grid::Grid&) override {
        const size_t tx = primitive.getTotalNumberOfXCells();
        const size_t ty = primitive.getTotalNumberOfYCells();
        const size_t gx = primitive.getNumberOfXGhostCells();
        const size_t gy = primitive.getNumberOfYGhostCells();
        const size_t gz = primitive.getNumberOfZGhostCells();
        const size_t cells = (size_t)n[0] * n[1] * n[2];
        for (int v = 0; v < nvar; ++v) {
            double* p = primitive.getScalarMemoryArea(v)->getPointer();
            for (int z = 0; z < n[2]; ++z)
                for (int y = 0; y < n[1]; ++y)
                    for (int x = 0; x < n[0]; ++x)
                        p[(z + gz) * tx * ty + (y + gy) * tx + (x + gx)] =
                            prim[v * cells + ((size_t)z * n[1] + y) * n[0] + x];
        }
        cellComputer.computeFromPrimitive(primitive, conserved);
    }
    void setParameters(const init::Parameters&) override {}
    boost::property_tree::ptree getDescription() const override { return {}; }

private:
    const double* prim;
    int nvar;
    int n[3];
};

// Records the conserved state handed to the writers after every step.
class CaptureWriter : public io::Writer {
public:
    CaptureWriter(double* out, int nvar) : out(out), nvar(nvar) {}
    void write(const volume::Volume& v, const grid::Grid&,
        const simulator::TimestepInformation& info) override {
        const size_t total = v.getScalarMemoryArea(0)->getSize();
        for (int k = 0; k < nvar; ++k)
            std::memcpy(out + k * total, v.getScalarMemoryArea(k)->getPointer(), total * sizeof(double));
        time = info.getCurrentTime();
        ++writes;
    }
    void finalize(const grid::Grid&, const simulator::TimestepInformation&) override {}
    double* out;
    int nvar;
    double time = 0;
    int writes = 0;
};

void copy_in(volume::Volume& v, const double* src, int nvar) {
    const size_t total = v.getScalarMemoryArea(0)->getSize();
    for (int k = 0; k < nvar; ++k)
        std::memcpy(v.getScalarMemoryArea(k)->getPointer(), src + k * total, total * sizeof(double));
}

void copy_out(const volume::Volume& v, double* dst, int nvar) {
    const size_t total = v.getScalarMemoryArea(0)->getSize();
    for (int k = 0; k < nvar; ++k)
        std::memcpy(dst + k * total, v.getScalarMemoryArea(k)->getPointer(), total * sizeof(double));
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_error.c_str(); }

void ref_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }

// Number of ghost cells the reference allocates for a flux/reconstruction pair
// (alsfvm/src/numflux/NumericalFluxCPU.cpp:226-231).
int ref_ghost_cells(const char* equation, const char* flux, const char* recon, int dim) {
    try {
        int dims[3] = {16, dim > 1 ? 16 : 1, dim > 2 ? 16 : 1};
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, flux, recon, "periodic", "forwardeuler", dims, lo, hi, 1.4, 0.5);
        numflux::NumericalFluxFactory f(equation, flux, recon, s.params, s.device);
        return (int)f.createNumericalFlux(*s.grid)->getNumberOfGhostCells();
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// One evaluation of the spatial operator through ConservedSystem (the call the
// integrators make, alsfvm/src/simulator/ConservedSystem.cpp:31-103): out gets
// the unscaled flux difference on interior cells, ws the per-direction maximum
// wave speed. U and out are padded arrays of nvar * total cells.
int ref_compute_flux(const char* equation, const char* flux, const char* recon,
    const int dims[3], double gamma, const double* U, double* out, double ws[3]) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, flux, recon, "periodic", "forwardeuler", dims, lo, hi, gamma, 0.5);
        numflux::NumericalFluxFactory f(equation, flux, recon, s.params, s.device);
        auto nf = f.createNumericalFlux(*s.grid);
        std::shared_ptr<integrator::System> system(new simulator::ConservedSystem(nf,
            std::make_shared<diffusion::NoDiffusion>()));
        volume::VolumeFactory vf(equation, s.memory);
        const size_t g = nf->getNumberOfGhostCells();
        auto vin = vf.createConservedVolume(dims[0], dims[1], dims[2], g);
        auto vout = vf.createConservedVolume(dims[0], dims[1], dims[2], g);
        const int nvar = nvar_of(equation);
        copy_in(*vin, U, nvar);
        vout->makeZero();
        rvec3 w(0, 0, 0);
        (*system)(*vin, w, true, *vout);
        copy_out(*vout, out, nvar);
        ws[0] = w.x; ws[1] = w.y; ws[2] = w.z;
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// One region call of the reference's NumericalFlux (NumericalFluxCPU::
// computeFlux with start / end, alsfvm/src/numflux/NumericalFluxCPU.cpp:
// 167-221): out (padded, nvar * total) is read first and only the region's
// cells change; ws gets the wave speeds the call returns.
int ref_compute_flux_region(const char* equation, const char* flux, const char* recon,
    const int dims[3], double gamma, const double* U, double* out, double ws[3], const int start[3],
    const int end[3]) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, flux, recon, "periodic", "forwardeuler", dims, lo, hi, gamma, 0.5);
        numflux::NumericalFluxFactory f(equation, flux, recon, s.params, s.device);
        auto nf = f.createNumericalFlux(*s.grid);
        volume::VolumeFactory vf(equation, s.memory);
        const size_t g = nf->getNumberOfGhostCells();
        auto vin = vf.createConservedVolume(dims[0], dims[1], dims[2], g);
        auto vout = vf.createConservedVolume(dims[0], dims[1], dims[2], g);
        const int nvar = nvar_of(equation);
        copy_in(*vin, U, nvar);
        copy_in(*vout, out, nvar);
        rvec3 w(0, 0, 0);
        nf->computeFlux(*vin, w, true, *vout, ivec3(start[0], start[1], start[2]), ivec3(end[0], end[1], end[2]));
        copy_out(*vout, out, nvar);
        ws[0] = w.x; ws[1] = w.y; ws[2] = w.z;
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// Reconstruction of every variable in one direction (indicator variable 0),
// over the reference's own cell range; left/right are padded arrays that the
// caller pre-fills (cells outside the range keep their contents).
int ref_reconstruct(const char* equation, const char* recon, const int dims[3], double gamma,
    int direction, const double* U, double* left, double* right) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, "godunov", recon, "periodic", "forwardeuler", dims, lo, hi, gamma, 0.5);
        reconstruction::ReconstructionFactory rf;
        auto r = rf.createReconstruction(recon, equation, *s.params, s.memory, *s.grid, s.device);
        volume::VolumeFactory vf(equation, s.memory);
        const size_t g = r->getNumberOfGhostCells();
        auto vin = vf.createConservedVolume(dims[0], dims[1], dims[2], g);
        auto vl = vf.createConservedVolume(dims[0], dims[1], dims[2], g);
        auto vr = vf.createConservedVolume(dims[0], dims[1], dims[2], g);
        const int nvar = nvar_of(equation);
        copy_in(*vin, U, nvar);
        copy_in(*vl, left, nvar);
        copy_in(*vr, right, nvar);
        r->performReconstruction(*vin, direction, 0, *vl, *vr);
        copy_out(*vl, left, nvar);
        copy_out(*vr, right, nvar);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// Ghost-cell fill of nvar padded arrays in place (BoundaryCPU).
int ref_boundary(const char* boundary, const int dims[3], int ghosts, int nvar, double* U) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        const char* eq = nvar == 1 ? "burgers" : nvar == 3 ? "euler1" : nvar == 4 ? "euler2" : "euler3";
        Setup s(eq, "godunov", "none", boundary, "forwardeuler", dims, lo, hi, 1.4, 0.5);
        boundary::BoundaryFactory bf(boundary, s.device);
        auto b = bf.createBoundary(ghosts);
        volume::VolumeFactory vf(eq, s.memory);
        auto v = vf.createConservedVolume(dims[0], dims[1], dims[2], ghosts);
        copy_in(*v, U, nvar);
        b->applyBoundaryConditions(*v, *s.grid);
        copy_out(*v, U, nvar);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// Full simulation through Simulator::performStep (the alsvinncli loop,
// alsvinncli/src/main.cpp:217-232). prim holds the interior primitive
// variables at the cell midpoints (nvar * nx*ny*nz, x fastest). When
// number_of_saves > 0 a FixedIntervalWriter with interval end_time /
// number_of_saves is attached as writer and dt adjuster exactly as
// SimulatorSetup::createWriter wires it. The loop stops at atEnd() or after
// max_steps steps (max_steps <= 0: no limit). out receives the padded
// conserved state at the end; dts (optional, capacity max_dts) the dt of each
// step.
int ref_run(const char* equation, const char* flux, const char* recon, const char* integrator,
    const char* boundary, const int dims[3], const double lower[3], const double upper[3],
    double gamma, double cfl, double end_time, int number_of_saves, int max_steps,
    const double* prim, double* out, double* t_out, int* steps_out, double* dts, int max_dts) {
    try {
        Setup s(equation, flux, recon, boundary, integrator, dims, lower, upper, gamma, cfl);
        volume::VolumeFactory vf(equation, s.memory);
        integrator::IntegratorFactory intf(integrator);
        boundary::BoundaryFactory bf(boundary, s.device);
        numflux::NumericalFluxFactory nff(equation, flux, recon, s.params, s.device);
        equation::CellComputerFactory ccf(s.params, s.device);
        std::string eqname = equation;
        auto diffusion = std::shared_ptr<diffusion::DiffusionOperator>(new diffusion::NoDiffusion());
        simulator::Simulator sim(*s.params, s.grid, vf, intf, bf, nff, ccf, s.memory, end_time,
            s.device, eqname, diffusion, "oracle");
        const int nvar = nvar_of(equation);
        std::shared_ptr<init::InitialData> init(new ArrayInitialData(prim, nvar, s.n));
        sim.setInitialValue(init);
        auto capture = std::make_shared<CaptureWriter>(out, nvar);
        std::shared_ptr<io::Writer> every(capture);
        sim.addWriter(every);
        if (number_of_saves > 0) {
            std::shared_ptr<io::Writer> nullw(new CaptureWriter(out, nvar));
            std::shared_ptr<io::Writer> fixed(new io::FixedIntervalWriter(nullw,
                end_time / number_of_saves, end_time, false));
            sim.addWriter(fixed);
            auto adj = std::dynamic_pointer_cast<integrator::TimestepAdjuster>(fixed);
            sim.addTimestepAdjuster(adj);
        }
        sim.callWriters();  // state at t = 0 into out
        int steps = 0;
        double tprev = sim.getCurrentTime();
        while (!sim.atEnd() && (max_steps <= 0 || steps < max_steps)) {
            sim.performStep();
            if (dts && steps < max_dts) dts[steps] = sim.getCurrentTime() - tprev;
            tprev = sim.getCurrentTime();
            ++steps;
        }
        *t_out = sim.getCurrentTime();
        *steps_out = steps;
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// Primitive -> conserved on padded arrays through the reference CellComputer.
int ref_prim_to_cons(const char* equation, const int dims[3], int ghosts, double gamma,
    const double* prim, double* cons) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, "godunov", "none", "periodic", "forwardeuler", dims, lo, hi, gamma, 0.5);
        equation::CellComputerFactory ccf(s.params, s.device);
        auto cc = ccf.createComputer();
        volume::VolumeFactory vf(equation, s.memory);
        auto vp = vf.createPrimitiveVolume(dims[0], dims[1], dims[2], ghosts);
        auto vc = vf.createConservedVolume(dims[0], dims[1], dims[2], ghosts);
        const int nvar = nvar_of(equation);
        copy_in(*vp, prim, nvar);
        cc->computeFromPrimitive(*vp, *vc);
        copy_out(*vc, cons, nvar);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// CPUCellComputer::obeysConstraints over a padded state: 1 obeys, 0 not, -1 error.
int ref_obeys_constraints(const char* equation, const int dims[3], int ghosts, double gamma,
    const double* U) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, "godunov", "none", "periodic", "forwardeuler", dims, lo, hi, gamma, 0.5);
        equation::CellComputerFactory ccf(s.params, s.device);
        auto cc = ccf.createComputer();
        volume::VolumeFactory vf(equation, s.memory);
        auto v = vf.createConservedVolume(dims[0], dims[1], dims[2], ghosts);
        copy_in(*v, U, nvar_of(equation));
        return cc->obeysConstraints(*v) ? 1 : 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// Draws through the reference generator and Uniform distribution: the process-
// wide mt19937_64 shared by every STLMersenne (alsuq/src/generator/
// STLMersenne.cpp:22-85). Samples must be requested in increasing order within
// one process, as the reference Runner does.
int ref_uniform(int dimension, int sample, double lower, double upper, double* out) {
    try {
        alsuq::generator::STLMersenne gen(dimension);
        char lo[64], hi[64];
        std::snprintf(lo, sizeof lo, "%.17g", lower);
        std::snprintf(hi, sizeof hi, "%.17g", upper);
        std::map<std::string, std::string> values{{"lower", lo}, {"upper", hi}};
        alsutils::parameters::Parameters p(values);
        alsuq::distribution::Uniform dist(p);
        for (int c = 0; c < dimension; ++c) out[c] = dist.generate(gen, c, sample);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// The Runner's parameter draws for samples sample_start .. sample_start +
// nsamples - 1 (alsuq/src/run/Runner.cpp:39-52): per sample, each parameter
// in the order given (the caller passes them in name order, as std::map
// iterates), components ascending, through one STLMersenne per parameter on
// the process-wide engine and Uniform(lower, upper). Valid once per process:
// the engine is static.
int ref_generate_sequence(int nparams, const int* dims, const double* lowers, const double* uppers,
    long long sample_start, long long nsamples, double* out) {
    try {
        std::vector<std::unique_ptr<alsuq::generator::STLMersenne>> gens;
        std::vector<std::unique_ptr<alsuq::distribution::Uniform>> dists;
        for (int p = 0; p < nparams; ++p) {
            gens.emplace_back(new alsuq::generator::STLMersenne(dims[p]));
            char lo[64], hi[64];
            std::snprintf(lo, sizeof lo, "%.17g", lowers[p]);
            std::snprintf(hi, sizeof hi, "%.17g", uppers[p]);
            std::map<std::string, std::string> values{{"lower", lo}, {"upper", hi}};
            alsutils::parameters::Parameters pp(values);
            dists.emplace_back(new alsuq::distribution::Uniform(pp));
        }
        long long k = 0;
        for (long long s = sample_start; s < sample_start + nsamples; ++s)
            for (int p = 0; p < nparams; ++p)
                for (int c = 0; c < dims[p]; ++c) out[k++] = dists[p]->generate(*gens[p], c, (size_t)s);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// MeanVariance over nsamples padded states all taken at the same time
// (alsuq/src/stats/MeanVariance.cpp:30-67 with StatisticsHelper::
// combineStatistics on one rank). mean/var receive padded arrays.
int ref_meanvar(const char* equation, const int dims[3], int ghosts, int nsamples,
    const double* const* samples, double* mean, double* var) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, "godunov", "none", "periodic", "forwardeuler", dims, lo, hi, 1.4, 0.5);
        boost::property_tree::ptree tree;
        auto& sp = *new alsuq::stats::StatisticsParameters(tree);
        sp.setNumberOfSamples(nsamples);
        sp.setPlatform("cpu");
        sp.setMpiConfiguration(std::make_shared<alsutils::mpi::Configuration>(MPI_COMM_WORLD, "cpu"));
        // Held for the life of the process: tearing the statistics object down
        // against the single-rank MPI stand-in is not needed for the result.
        auto& mv = *new alsuq::stats::MeanVariance(sp);
        const int nvar = nvar_of(equation);
        auto wm = std::make_shared<CaptureWriter>(mean, nvar);
        auto wv = std::make_shared<CaptureWriter>(var, nvar);
        std::shared_ptr<io::Writer> wmw(wm), wvw(wv);
        mv.addWriter("mean", wmw);
        mv.addWriter("variance", wvw);
        volume::VolumeFactory vf(equation, s.memory);
        auto v = vf.createConservedVolume(dims[0], dims[1], dims[2], ghosts);
        simulator::TimestepInformation info(0.5, 1);
        for (int k = 0; k < nsamples; ++k) {
            copy_in(*v, samples[k], nvar);
            mv.computeStatistics(*v, *s.grid, info);
        }
        mv.combineStatistics();
        mv.finalizeStatistics();
        mv.writeStatistics(*s.grid);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// One sample's cube structure function (StructureCube::computeStatistics,
// alsuq/src/stats/StructureCube.cpp:36-76, through the reference's own
// alsfvm/include/alsfvm/functional/structure_common.hpp): out receives nvar
// arrays of number_of_h values, entry h the sum over cells and over the
// cube surface at distance h of |u - u_h|^p / (nx ny nz).
int ref_structure_cube(const char* equation, const char* boundary, const int dims[3], int ghosts, int number_of_h,
    double p, const double* U, double* out) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, "godunov", "none", boundary, "forwardeuler", dims, lo, hi, 1.4, 0.5);
        const int nvar = nvar_of(equation);
        volume::VolumeFactory vf(equation, s.memory);
        auto in = vf.createConservedVolume(dims[0], dims[1], dims[2], ghosts);
        copy_in(*in, U, nvar);
        auto o = vf.createConservedVolume(number_of_h, 1, 1, 0);
        o->makeZero();
        if (std::string(boundary) == "periodic")
            functional::dispatchComputeStructureCubeCPU<boundary::PERIODIC>(*o, *in, number_of_h, p);
        else
            functional::dispatchComputeStructureCubeCPU<boundary::NEUMANN>(*o, *in, number_of_h, p);
        copy_out(*o, out, nvar);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// One functional of the reference's CPU factory applied to one padded state
// (alsfvm/src/functional/FunctionalFactory.cpp, the functional classes under
// alsfvm/src/functional/): the output volume is created as
// IntervalFunctionalWriter::makeVolumes does (functional size, the
// functional's ghost cells), zeroed, the functional applied with `weight`;
// out receives the interior of every variable, size_out its extents.
int ref_functional(const char* name, const char* equation, const char* boundary, const int dims[3], int ghosts,
    const double lower[3], const double upper[3], int degree, double min_value, double max_value,
    const char* variables, double gamma, double p, int number_of_h, double weight, const double* U, double* out,
    int size_out[3]) {
    try {
        Setup s(equation, "godunov", "none", boundary, "forwardeuler", dims, lower, upper, gamma, 0.5);
        const int nvar = nvar_of(equation);
        volume::VolumeFactory vf(equation, s.memory);
        auto in = vf.createConservedVolume(dims[0], dims[1], dims[2], ghosts);
        copy_in(*in, U, nvar);
        char buf[5][64];
        std::snprintf(buf[0], sizeof buf[0], "%d", degree);
        std::snprintf(buf[1], sizeof buf[1], "%.17g", min_value);
        std::snprintf(buf[2], sizeof buf[2], "%.17g", max_value);
        std::snprintf(buf[3], sizeof buf[3], "%.17g", gamma);
        std::snprintf(buf[4], sizeof buf[4], "%.17g", p);
        std::map<std::string, std::string> values{{"degree", buf[0]}, {"minValue", buf[1]}, {"maxValue", buf[2]},
                                                  {"gamma", buf[3]}, {"p", buf[4]},
                                                  {"numberOfH", std::to_string(number_of_h)}};
        if (variables && *variables) values["variables"] = variables;
        alsutils::parameters::Parameters params(values);
        functional::FunctionalFactory factory;
        auto f = factory.makeFunctional("cpu", name, params);
        const ivec3 fs = f->getFunctionalSize(*s.grid);
        const ivec3 gh = f->getGhostCellSizes(*s.grid, *in);
        auto o = vf.createConservedVolume(fs.x, fs.y, fs.z, gh.x);
        o->makeZero();
        (*f)(*o, *in, weight, *s.grid);
        const size_t tx = o->getTotalNumberOfXCells(), ty = o->getTotalNumberOfYCells();
        const size_t gx = o->getNumberOfXGhostCells(), gy = o->getNumberOfYGhostCells(),
                     gz = o->getNumberOfZGhostCells();
        const size_t cells = (size_t)fs.x * fs.y * fs.z;
        for (int v = 0; v < nvar; ++v) {
            const double* src = o->getScalarMemoryArea(v)->getPointer();
            for (int z = 0; z < fs.z; ++z)
                for (int y = 0; y < fs.y; ++y)
                    for (int x = 0; x < fs.x; ++x)
                        out[v * cells + ((size_t)z * fs.y + y) * fs.x + x] =
                            src[(z + gz) * tx * ty + (y + gy) * tx + (x + gx)];
        }
        size_out[0] = fs.x;
        size_out[1] = fs.y;
        size_out[2] = fs.z;
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// One sample's StructureBasic statistic (alsuq/src/stats/StructureBasic.cpp)
// through the reference's StatisticsHelper on one rank: out receives nvar
// arrays of number_of_h values.
int ref_structure_basic(const char* equation, const char* boundary, const int dims[3], int ghosts, int number_of_h,
    double p, int direction, const double* U, double* out) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, "godunov", "none", boundary, "forwardeuler", dims, lo, hi, 1.4, 0.5);
        boost::property_tree::ptree tree;
        tree.put("direction", direction);
        tree.put("p", p);
        tree.put("numberOfH", number_of_h);
        auto& sp = *new alsuq::stats::StatisticsParameters(tree);
        sp.setNumberOfSamples(1);
        sp.setPlatform("cpu");
        sp.setMpiConfiguration(std::make_shared<alsutils::mpi::Configuration>(MPI_COMM_WORLD, "cpu"));
        auto& sb = *new alsuq::stats::StructureBasic(sp);
        const int nvar = nvar_of(equation);
        auto w = std::make_shared<CaptureWriter>(out, nvar);
        std::shared_ptr<io::Writer> ww(w);
        sb.addWriter(sb.getStatisticsNames()[0], ww);
        volume::VolumeFactory vf(equation, s.memory);
        auto v = vf.createConservedVolume(dims[0], dims[1], dims[2], ghosts);
        copy_in(*v, U, nvar);
        simulator::TimestepInformation info(0.5, 1);
        sb.computeStatistics(*v, *s.grid, info);
        sb.combineStatistics();
        sb.finalizeStatistics();
        sb.writeStatistics(*s.grid);
        return w->writes == 1 ? 0 : -1;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

// HostMemory::getTotalVariation(direction, p, start, end) of each variable of
// one padded state between the ghost layers (the per-sample quantity of
// alsuq's bv_direction statistic, alsuq/src/stats/BoundedVariationDirection.cpp).
int ref_total_variation_direction(const char* equation, const int dims[3], int ghosts, int direction, int p,
    const double* U, double* out) {
    try {
        double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
        Setup s(equation, "godunov", "none", "periodic", "forwardeuler", dims, lo, hi, 1.4, 0.5);
        const int nvar = nvar_of(equation);
        volume::VolumeFactory vf(equation, s.memory);
        auto in = vf.createConservedVolume(dims[0], dims[1], dims[2], ghosts);
        copy_in(*in, U, nvar);
        const ivec3 start = in->getNumberOfGhostCells();
        const ivec3 end = in->getSize() - in->getNumberOfGhostCells();
        for (int v = 0; v < nvar; ++v)
            out[v] = in->getScalarMemoryArea(v)->getTotalVariation(direction, p, start, end);
        return 0;
    } catch (std::exception& e) {
        g_error = e.what();
        return -1;
    }
}

}  // extern "C"
