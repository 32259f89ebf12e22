// Compiles the "gb300" platform classes (include/gbfv_alsvinn.hpp) as
// subclasses of alsvinn's own abstract interfaces, against alsvinn's headers,
// and links them with alsvinn's CPU library and libgbfv.so: every pure
// virtual of Memory<real>, NumericalFlux, Reconstruction, Boundary and
// CellComputer is implemented with the reference's signature, and the
// reference's own MeanVariance registers for the platform. The objects are
// built only when a CUDA device is present (argument "run").
#include <cstdio>
#include <cstring>
#include <memory>

#include "alsuq/stats/MeanVariance.hpp"
#include "alsuq/stats/stats_util.hpp"
#include "gbfv_alsvinn.hpp"

namespace alsuq {
namespace stats {
REGISTER_STATISTICS(gb300, meanvar, MeanVariance)
}  // namespace stats
}  // namespace alsuq

using namespace alsfvm;

// Each interface pointer is taken from the platform class, so the classes
// must be complete (no pure virtual left) for this unit to compile.
static int build_all(const grid::Grid& grid) {
    gb300::Scheme s{"euler2", "hll3", "weno2", "periodic", 1.4};
    std::shared_ptr<memory::Memory<real> > m = std::make_shared<gb300::GB300Memory<real> >(36, 36, 1);
    std::shared_ptr<numflux::NumericalFlux> f = std::make_shared<gb300::GB300NumericalFlux>(s, grid);
    std::shared_ptr<reconstruction::Reconstruction> r = std::make_shared<gb300::GB300Reconstruction>(s, grid);
    std::shared_ptr<boundary::Boundary> b = std::make_shared<gb300::GB300Boundary>(s, grid);
    std::shared_ptr<equation::CellComputer> c = std::make_shared<gb300::GB300CellComputer>(s, grid);
    *m += 1.0;
    *m *= 2.0;
    std::vector<real> h(m->getSize());
    m->copyToHost(h.data(), h.size());
    return (h[0] == 2.0 && f->getNumberOfGhostCells() == 2 && r->getNumberOfGhostCells() == 2 && b && c) ? 0 : 1;
}

int main(int argc, char** argv) {
    if (argc > 1 && std::strcmp(argv[1], "run") == 0) {
        grid::Grid grid(rvec3(0, 0, 0), rvec3(1, 1, 0), ivec3(32, 32, 1));
        const int rc = build_all(grid);
        std::printf(rc == 0 ? "ALL PASSED\n" : "FAILED\n");
        return rc;
    }
    std::printf("linked\n");
    return 0;
}
