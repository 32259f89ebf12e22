// Tests of the C++ adapters (include/gbfv_alsfvm.hpp) in the style of the
// reference's own library tests: consistency of the numerical flux on a
// constant state (test/library_tests/src/fvm/flux/numericalfluxtest.cpp),
// WENO2 known answers (test/library_tests/src/fvm/reconstruction/WenoTest.cpp),
// the boundary index maps (test/library_tests/src/fvm/boundary/BoundaryTest.cpp),
// the constraint check, the simulator loop and mean / variance.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "gbfv_alsfvm.hpp"

using namespace gbfv_alsfvm;

static int g_failures = 0, g_checks = 0;
#define EXPECT_TRUE(c)                                                              \
    do {                                                                            \
        ++g_checks;                                                                 \
        if (!(c)) {                                                                 \
            ++g_failures;                                                           \
            std::printf("  FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);            \
        }                                                                           \
    } while (0)
#define EXPECT_NEAR(a, b, tol) EXPECT_TRUE(std::fabs((a) - (b)) <= (tol))

static void run(const char* name, const std::function<void()>& f) {
    const int before = g_failures;
    try {
        f();
    } catch (std::exception& e) {
        ++g_failures;
        std::printf("  EXCEPTION %s\n", e.what());
    }
    std::printf("[%s] %s\n", g_failures == before ? "PASS" : "FAIL", name);
}

static size_t idx(const Volume& v, int x, int y, int z) {
    return ((size_t)z * v.getTotalNumberOfYCells() + y) * v.getTotalNumberOfXCells() + x;
}

int main() {
    run("NumericalFlux.ConstantStateHasZeroDivergence", [] {
        for (const char* eq : {"euler1", "euler2", "euler3"}) {
            for (const char* fl : {"hll", "hll3"}) {
                Scheme s;
                s.equation = eq;
                s.flux = fl;
                const int dim = eq[5] - '0';
                ivec3 n(12, dim > 1 ? 10 : 1, dim > 2 ? 9 : 1);
                Grid g(rvec3(0, 0, 0), rvec3(1, 1, 1), n);
                NumericalFlux flux(s, g);
                Volume U(eq, n, (int)flux.getNumberOfGhostCells()), out(eq, n, (int)flux.getNumberOfGhostCells());
                const size_t nv = U.getNumberOfVariables(), total = U.getTotalSize();
                std::vector<real> h(nv * total);
                for (size_t i = 0; i < total; ++i) {
                    h[i] = 1.2;                                            // rho
                    for (int k = 0; k < dim; ++k) h[(1 + k) * total + i] = 0.3 * (k + 1);  // momentum
                    h[(nv - 1) * total + i] = 3.0;                         // energy
                }
                U.fromHost(h);
                rvec3 ws;
                flux.computeFlux(U, ws, true, out);
                for (real v : out.toHost()) EXPECT_NEAR(v, 0.0, 1e-13);
                EXPECT_TRUE(ws.x > 0);
            }
        }
    });

    run("Weno.ConstantInConstantOut", [] {
        Scheme s;
        s.equation = "burgers";
        s.flux = "godunov";
        ivec3 n(16, 1, 1);
        Grid g(rvec3(0, 0, 0), rvec3(1, 1, 1), n);
        Reconstruction rec(s, g);
        Volume in("burgers", n, 2), left("burgers", n, 2), right("burgers", n, 2);
        in.fromHost(std::vector<real>(in.getTotalSize(), 0.7));
        rec.performReconstruction(in, 0, 0, left, right);
        const auto l = left.toHost(), r = right.toHost();
        for (size_t x = 1; x + 1 < in.getTotalSize(); ++x) {
            EXPECT_NEAR(l[x], 0.7, 1e-15);
            EXPECT_NEAR(r[x], 0.7, 1e-15);
        }
    });

    run("Weno.ReconstructionSimple", [] {
        // u = x^2 on the cells; the WENO2 weights follow from the smoothness
        // indicators b0 = (u[i+1]-u[i])^2, b1 = (u[i]-u[i-1])^2 with
        // eps = 1e-8: left face alpha = (1, 2)/(3 (eps+b)^2), right face (2, 1)
        Scheme s;
        s.equation = "burgers";
        s.flux = "godunov";
        ivec3 n(10, 1, 1);
        Grid g(rvec3(0, 0, 0), rvec3(1, 1, 1), n);
        Reconstruction rec(s, g);
        Volume in("burgers", n, 2), left("burgers", n, 2), right("burgers", n, 2);
        std::vector<real> u(in.getTotalSize());
        for (size_t i = 0; i < u.size(); ++i) u[i] = 0.1 * i * i;
        in.fromHost(u);
        rec.performReconstruction(in, 0, 0, left, right);
        const auto l = left.toHost(), r = right.toHost();
        const real eps = 1e-8;
        for (size_t i = 1; i + 1 < u.size(); ++i) {
            const real b0 = (u[i + 1] - u[i]) * (u[i + 1] - u[i]);
            const real b1 = (u[i] - u[i - 1]) * (u[i] - u[i - 1]);
            const real a0l = 1 / (3 * (eps + b0) * (eps + b0)), a1l = 2 / (3 * (eps + b1) * (eps + b1));
            const real a0r = 2 / (3 * (eps + b0) * (eps + b0)), a1r = 1 / (3 * (eps + b1) * (eps + b1));
            const real w0l = a0l / (a0l + a1l), w1l = a1l / (a0l + a1l);
            const real w0r = a0r / (a0r + a1r), w1r = a1r / (a0r + a1r);
            const real el = 0.5 * (w1l * u[i - 1] + (3 * w0l + w1l) * u[i] - w0l * u[i + 1]);
            const real er = 0.5 * (w0r * u[i + 1] + (3 * w1r + w0r) * u[i] - w1r * u[i - 1]);
            EXPECT_NEAR(l[i], el, 1e-13 * (1 + std::fabs(el)));
            EXPECT_NEAR(r[i], er, 1e-13 * (1 + std::fabs(er)));
        }
    });

    run("Boundary.NeumannAndPeriodicIndexMaps", [] {
        for (const char* bc : {"neumann", "periodic"}) {
            Scheme s;
            s.equation = "burgers";
            s.flux = "godunov";
            s.boundary = bc;
            ivec3 n(6, 5, 1);
            Grid g(rvec3(0, 0, 0), rvec3(1, 1, 1), n);
            Boundary b(s, g);
            Volume v("burgers", n, 2);
            std::vector<real> h(v.getTotalSize());
            for (size_t i = 0; i < h.size(); ++i) h[i] = (real)i;
            v.fromHost(h);
            b.applyBoundaryConditions(v, g);
            const auto o = v.toHost();
            const bool per = std::string(bc) == "periodic";
            // x ghosts of an interior row: Neumann mirrors (ghost 1 <- 2, ghost
            // 0 <- 3), periodic wraps (ghost 1 <- 7, ghost 0 <- 6)
            for (int y = 2; y < 7; ++y) {
                EXPECT_TRUE(o[idx(v, 1, y, 0)] == h[idx(v, per ? 7 : 2, y, 0)]);
                EXPECT_TRUE(o[idx(v, 0, y, 0)] == h[idx(v, per ? 6 : 3, y, 0)]);
                EXPECT_TRUE(o[idx(v, 8, y, 0)] == h[idx(v, per ? 2 : 7, y, 0)]);
                EXPECT_TRUE(o[idx(v, 9, y, 0)] == h[idx(v, per ? 3 : 6, y, 0)]);
            }
            // a corner takes both maps
            EXPECT_TRUE(o[idx(v, 0, 0, 0)] == h[idx(v, per ? 6 : 3, per ? 5 : 3, 0)]);
        }
    });

    run("CellComputer.ObeysConstraints", [] {
        Scheme s;
        ivec3 n(8, 8, 1);
        Grid g(rvec3(0, 0, 0), rvec3(1, 1, 1), n);
        CellComputer cc(s, g);
        Volume v("euler2", n, 2);
        const size_t total = v.getTotalSize();
        std::vector<real> h(4 * total);
        for (size_t i = 0; i < total; ++i) {
            h[i] = 1.0;
            h[3 * total + i] = 2.5;
        }
        v.fromHost(h);
        EXPECT_TRUE(cc.obeysConstraints(v));
        h[3 * total + 7] = -1.0;  // negative energy -> negative pressure (a ghost cell)
        v.fromHost(h);
        EXPECT_TRUE(!cc.obeysConstraints(v));
        h[3 * total + 7] = std::nan("");
        v.fromHost(h);
        EXPECT_TRUE(!cc.obeysConstraints(v));
    });

    run("Simulator.SodShockTubeReachesEndTime", [] {
        Scheme s;
        s.equation = "euler1";
        s.boundary = "neumann";
        s.cfl = 0.475;
        const int N = 256;
        Grid g(rvec3(-5, 0, 0), rvec3(5, 1, 1), ivec3(N, 1, 1));
        std::vector<real> prim(3 * N);
        const real dx = 10.0 / N;
        for (int i = 0; i < N; ++i) {
            const bool left = -5 + dx * i + dx / 2.0 < 0;
            prim[i] = left ? 1.0 : 0.125;
            prim[2 * N + i] = left ? 1.0 : 0.1;
        }
        Simulator a(s, g, 1.3, 1), b(s, g, 1.3, 1);
        a.setInitialValue(prim);
        b.setInitialValue(prim);
        while (!a.atEnd()) a.performStep();
        b.run();
        EXPECT_TRUE(a.getCurrentTime() == 1.3);
        EXPECT_TRUE(a.getNumberOfStepsPerformed() == b.getNumberOfStepsPerformed());
        EXPECT_TRUE(a.getConservedState() == b.getConservedState());
        const auto U = a.getConservedState();
        for (int i = 2; i < N + 2; ++i) EXPECT_TRUE(U[i] > 0.1 && U[i] < 1.01);
    });

    run("Simulator.ConstraintViolationThrows", [] {
        Scheme s;
        s.equation = "euler1";
        s.boundary = "neumann";
        Grid g(rvec3(-5, 0, 0), rvec3(5, 1, 1), ivec3(32, 1, 1));
        std::vector<real> prim(3 * 32, 1.0);
        for (int i = 0; i < 32; ++i) prim[32 + i] = 0.0;
        prim[2 * 32 + 10] = -2.0;
        Simulator sim(s, g, 1.0);
        sim.setInitialValue(prim);
        bool threw = false;
        try {
            sim.performStep();
        } catch (std::runtime_error&) {
            threw = true;
        }
        EXPECT_TRUE(threw);
    });

    run("MeanVariance.KnownSamples", [] {
        ivec3 n(4, 1, 1);
        Volume v("burgers", n, 2);
        MeanVariance mv(v.getTotalSize());
        for (real a : {1.0, 2.0, 4.0}) {
            v.fromHost(std::vector<real>(v.getTotalSize(), a));
            mv.computeStatistics(v);
        }
        std::vector<real> m, var;
        mv.finalizeStatistics(m, var);
        for (size_t i = 0; i < m.size(); ++i) {
            EXPECT_NEAR(m[i], 7.0 / 3.0, 1e-15);
            EXPECT_NEAR(var[i], (1 + 4 + 16) / 3.0 - 49.0 / 9.0, 1e-14);
        }
    });

    run("NumericalFlux.ConservedSystemRegionsEqualWholeDomain", [] {
        // ConservedSystem::operator() (alsfvm/src/simulator/ConservedSystem.cpp:
        // 59-96): the interior region, then the bottom and top strip of every
        // dimension; together they give the whole-domain operator
        Scheme s;
        ivec3 n(40, 28, 1);
        Grid g(rvec3(0, 0, 0), rvec3(1, 1, 1), n);
        NumericalFlux flux(s, g);
        const int gc = (int)flux.getNumberOfGhostCells();
        Volume U("euler2", n, gc), whole("euler2", n, gc), split("euler2", n, gc);
        const size_t total = U.getTotalSize();
        std::vector<real> h(4 * total);
        for (size_t i = 0; i < total; ++i) {
            const double x = 0.37 * (double)(i % 44), y = 0.21 * (double)(i / 44);
            h[i] = 1.5 + 0.2 * std::sin(x + y);
            h[total + i] = 0.3 * std::cos(x);
            h[2 * total + i] = -0.2 * std::sin(y);
            h[3 * total + i] = 4.0 + 0.1 * std::cos(x - y);
        }
        U.fromHost(h);
        rvec3 wsWhole, ws(0, 0, 0);
        flux.computeFlux(U, wsWhole, true, whole);
        const int size[2] = {n.x + 2 * gc, n.y + 2 * gc};
        rvec3 w;
        flux.computeFlux(U, w, true, split, ivec3(gc, gc, 0), ivec3(-gc, -gc, 0));
        ws = w;
        for (int d = 0; d < 2; ++d) {
            ivec3 endBottom(d == 0 ? -size[0] + 3 * gc : 0, d == 1 ? -size[1] + 3 * gc : 0, 0);
            flux.computeFlux(U, w, true, split, ivec3(), endBottom);
            ws = rvec3(std::max(ws.x, w.x), std::max(ws.y, w.y), 0);
            ivec3 startTop(d == 0 ? size[0] - 3 * gc : 0, d == 1 ? size[1] - 3 * gc : 0, 0);
            flux.computeFlux(U, w, true, split, startTop, ivec3());
            ws = rvec3(std::max(ws.x, w.x), std::max(ws.y, w.y), 0);
        }
        const auto a = whole.toHost(), b = split.toHost();
        bool same = true;
        for (int k = 0; k < 4; ++k)
            for (int y = gc; y < n.y + gc; ++y)
                for (int x = gc; x < n.x + gc; ++x) {
                    const size_t i = k * total + idx(U, x, y, 0);
                    same = same && a[i] == b[i];
                }
        EXPECT_TRUE(same);
        EXPECT_TRUE(ws.x == wsWhole.x && ws.y == wsWhole.y);
    });

    run("Memory.RungeKuttaStageAlgebra", [] {
        // RungeKutta3::performSubstep's second stage (alsfvm/src/integrator/
        // RungeKutta3.cpp:69-77): out *= dt/dx; out += U1; out *= 1/3;
        // out += U0; out *= 3/4, on the device, against the same on the host
        ivec3 n(50, 1, 1);
        Volume out("burgers", n, 2), U1("burgers", n, 2), U0("burgers", n, 2);
        const size_t total = out.getTotalSize();
        std::vector<real> o(total), u1(total), u0(total);
        for (size_t i = 0; i < total; ++i) {
            o[i] = std::sin(0.3 * i);
            u1[i] = 1.0 + 0.01 * i;
            u0[i] = 2.0 - 0.02 * i;
        }
        out.fromHost(o);
        U1.fromHost(u1);
        U0.fromHost(u0);
        const real c = 0.0123;
        Memory& m = out.getScalarMemoryArea(0);
        m *= c;
        m += U1.getScalarMemoryArea(0);
        m *= 1. / 3.;
        m += U0.getScalarMemoryArea(0);
        m *= 3. / 4.;
        const auto got = out.toHost();
        bool same = true;
        for (size_t i = 0; i < total; ++i) {
            real v = o[i];
            v *= c;
            v += u1[i];
            v *= 1. / 3.;
            v += u0[i];
            v *= 3. / 4.;
            same = same && got[i] == v;
        }
        EXPECT_TRUE(same);
        // MeanVariance's second moment: addPower(u, 2), then subtractPower(mean, 2)
        Volume sq("burgers", n, 2);
        sq.getScalarMemoryArea(0).addPower(U1.getScalarMemoryArea(0), 2);
        sq.getScalarMemoryArea(0).subtractPower(U0.getScalarMemoryArea(0), 2);
        const auto q = sq.toHost();
        bool ok = true;
        for (size_t i = 0; i < total; ++i) ok = ok && q[i] == (0.0 + u1[i] * u1[i]) - u0[i] * u0[i];
        EXPECT_TRUE(ok);
    });

    std::printf("%d checks, %d failures\n", g_checks, g_failures);
    if (g_failures == 0) std::printf("ALL PASSED\n");
    return g_failures == 0 ? 0 : 1;
}
