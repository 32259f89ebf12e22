"""The reference's own CUDA path on the GPU: its kernels (NumericalFluxCUDA,
ReconstructionCUDA, BoundaryCUDA, vector_operations, CUDACellComputer),
compiled unmodified for sm_103a, driven by oracle/refcuda the way the
reference's Simulator drives them on the cuda platform.

- Against the oracle (the CPU restatement pinned to the reference's CPU
  build): Sod, Kelvin-Helmholtz and Taylor-Green runs agree within 1e-10
  relative L1 per conserved variable (the CUDA build contracts multiply-adds
  and uses --use_fast_math, so it is not bit-identical to the CPU build),
  with the same step count and end time. This shows the launch sequence
  restated in oracle/refcuda is the reference's step.
- The product's FP64 solver against the reference's CUDA path: within the
  same 1e-10.
- The reference's launch count per step: what the fused step replaces.

The cubins build from the reference's sources (oracle/refbuild, target
cuda); where they are absent the tests skip and say so.
"""
import math

import numpy as np
import pytest

import workloads
from alsvinn_gb300 import lib
from conftest import interior, rel_l1
from oracle import fvoracle
from oracle import refcuda

pytestmark = pytest.mark.gpu

G = 2


@pytest.fixture(scope="module")
def refcuda_ready(cuda_device):
    why = refcuda.missing()
    if why:
        pytest.skip(why)
    return True


def padded_conserved(eq, n, prim):
    """The oracle's primitive -> conserved map over the padded volume, the
    way Simulator::setInitialValue prepares the reference's cuda volumes
    (computed on the CPU, then copied)."""
    dim = workloads.dimension(n)
    t = workloads.padded_shape(n, G)
    nv = prim.shape[0]
    P = np.zeros((nv, t[2], t[1], t[0]))
    gz, gy = (G if dim > 2 else 0), (G if dim > 1 else 0)
    P[:, gz:gz + n[2], gy:gy + n[1], G:G + n[0]] = prim.reshape(nv, n[2], n[1], n[0])
    return fvoracle.prim_to_cons(eq, n, G, 1.4, P.reshape(nv, -1))


CASES = {
    "sod2048": dict(eq="euler1", n=(2048, 1, 1), lower=(-5, 0, 0), upper=(5, 1, 1), bc="neumann", cfl=0.475,
                    end=1.3, steps=60, prim=lambda: workloads.sod_prim(2048)),
    "kh128": dict(eq="euler2", n=(128, 128, 1), lower=(0, 0, 0), upper=(1, 1, 0), bc="periodic", cfl=0.4,
                  end=1e9, steps=20, prim=lambda: workloads.kh_prim(128, fvoracle.uniform(40, 3))),
    "tg24": dict(eq="euler3", n=(24, 24, 24), lower=(0, 0, 0), upper=(2 * math.pi,) * 3, bc="periodic", cfl=0.4,
                 end=1e9, steps=10, prim=lambda: workloads.tg_prim(24)),
}


def _case(name):
    c = CASES[name]
    return c, c["prim"]()


@pytest.mark.parametrize("name", list(CASES))
def test_reference_cuda_path_matches_the_oracle(refcuda_ready, name):
    c, prim = _case(name)
    nv = prim.shape[0]
    rc, ref, ref_t, ref_steps = fvoracle.run(c["eq"], "hll3", "weno2", "rungekutta3", c["bc"], c["n"], c["lower"],
                                             c["upper"], 1.4, c["cfl"], c["end"], 0, c["steps"], prim, G, nv)
    assert rc == 0 and ref_steps == c["steps"]
    with refcuda.Solver(c["eq"], "hll3", "weno2", "rungekutta3", c["bc"], c["n"], c["lower"], c["upper"], 1.4,
                        c["cfl"]) as s:
        s.set_state(padded_conserved(c["eq"], c["n"], prim))
        t, steps = s.run(c["end"], 0, c["steps"])
        U = s.get_state()
    assert steps == ref_steps
    assert abs(t - ref_t) <= 1e-12 * ref_t
    err = rel_l1(interior(U, c["n"], G), interior(ref, c["n"], G))
    assert (err <= 1e-10).all(), err


def test_reference_cuda_path_runs_sod_to_its_end_time(refcuda_ready):
    """The Sod configuration to t = 1.3 with the writer's dt clamp (one save):
    the reference's CUDA path and the oracle take the same steps to the same
    end time."""
    c, prim = _case("sod2048")
    rc, ref, ref_t, ref_steps = fvoracle.run("euler1", "hll3", "weno2", "rungekutta3", "neumann", c["n"], c["lower"],
                                             c["upper"], 1.4, c["cfl"], 1.3, 1, 0, prim, G, 3)
    assert rc == 0
    with refcuda.Solver("euler1", "hll3", "weno2", "rungekutta3", "neumann", c["n"], c["lower"], c["upper"], 1.4,
                        c["cfl"]) as s:
        s.set_state(padded_conserved("euler1", c["n"], prim))
        t, steps = s.run(1.3, 1, 0)
        U = s.get_state()
    assert steps == ref_steps and abs(t - 1.3) <= 1e-12 and abs(ref_t - 1.3) <= 1e-12
    err = rel_l1(interior(U, c["n"], G), interior(ref, c["n"], G))
    assert (err <= 1e-10).all(), err


@pytest.mark.parametrize("flux,integrator,bc", [("hll", "rungekutta2", "neumann"), ("hll3", "forwardeuler", "periodic")])
def test_reference_cuda_path_other_schemes(refcuda_ready, flux, integrator, bc):
    n = (96, 80, 1)
    prim = workloads.kh_prim(96, fvoracle.uniform(40, 1))[:, :96 * 80]
    rc, ref, ref_t, ref_steps = fvoracle.run("euler2", flux, "weno2", integrator, bc, n, (0, 0, 0), (1, 1, 0), 1.4,
                                             0.4, 1e9, 0, 12, prim, G, 4)
    assert rc == 0
    with refcuda.Solver("euler2", flux, "weno2", integrator, bc, n, (0, 0, 0), (1, 1, 0), 1.4, 0.4) as s:
        s.set_state(padded_conserved("euler2", n, prim))
        t, steps = s.run(1e9, 0, 12)
        U = s.get_state()
    assert steps == 12 and abs(t - ref_t) <= 1e-12 * ref_t
    err = rel_l1(interior(U, n, G), interior(ref, n, G))
    assert (err <= 1e-10).all(), err


@pytest.mark.parametrize("name", ["kh128", "tg24"])
def test_product_fp64_matches_the_reference_cuda_path(refcuda_ready, name):
    c, prim = _case(name)
    with refcuda.Solver(c["eq"], "hll3", "weno2", "rungekutta3", c["bc"], c["n"], c["lower"], c["upper"], 1.4,
                        c["cfl"]) as r:
        r.set_state(padded_conserved(c["eq"], c["n"], prim))
        rt, rsteps = r.run(c["end"], 0, c["steps"])
        R = r.get_state()
    with lib.Solver(c["eq"], "hll3", "weno2", "rungekutta3", c["bc"], c["n"], c["lower"], c["upper"], cfl=c["cfl"],
                    precision=lib.FP64) as s:
        s.set_primitive(prim)
        s.advance(c["end"], 0, c["steps"])
        t, steps, _ = s.time()
        U = s.get_state()
    assert steps == rsteps and abs(t - rt) <= 1e-12 * rt
    err = rel_l1(interior(U, c["n"], G), interior(R, c["n"], G))
    assert (err <= 1e-10).all(), err


def test_product_fp64_matches_the_reference_cuda_path_at_full_size(refcuda_ready):
    """Kelvin-Helmholtz 1024 x 1024, the benchmark workload: three SSP-RK3
    steps of the reference's CUDA path and of the product's FP64 solver from
    the same initial data agree within 1e-10 relative L1 per variable, with
    the same end time."""
    n = (1024, 1024, 1)
    prim = workloads.kh_prim(1024, fvoracle.uniform(40, 0))
    with refcuda.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", n, (0, 0, 0), (1, 1, 0)) as r:
        r.set_state(padded_conserved("euler2", n, prim))
        rt, rsteps = r.run(1e9, 0, 3)
        R = r.get_state()
    with lib.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", n, (0, 0, 0), (1, 1, 0), cfl=0.4,
                    precision=lib.FP64) as s:
        s.set_primitive(prim)
        s.advance(1e9, 0, 3)
        t, steps, _ = s.time()
        U = s.get_state()
    assert steps == rsteps == 3 and abs(t - rt) <= 1e-12 * rt
    err = rel_l1(interior(U, n, G), interior(R, n, G))
    assert (err <= 1e-10).all(), err


def test_reference_cuda_launches_per_step(refcuda_ready):
    """2D RK3: per stage five computeFlux calls (the interior and four side
    strips), each a makeZero plus, per direction, a reconstruction, a face
    flux, cub's two-pass max and a combine; then the Volume arithmetic per
    variable and the boundary per variable and side; one constraint check per
    step. Counted here: the reference kernels this driver launches (cub's and
    thrust's own launches not included)."""
    n = (64, 64, 1)
    prim = workloads.kh_prim(64, fvoracle.uniform(40, 0))
    with refcuda.Solver("euler2", "hll3", "weno2", "rungekutta3", "periodic", n, (0, 0, 0), (1, 1, 0)) as s:
        s.set_state(padded_conserved("euler2", n, prim))
        before = s.launches()
        s.run(1e9, 0, 2)
        per_step = (s.launches() - before) / 2
    flux_calls = 3 * 5 * (1 + 2 * 3)      # stages x calls x (makeZero + dirs x (recon, flux, combine))
    algebra = 4 * (2 + 5 + 5)              # variables x (stage 1, 2, 3 operations)
    boundary = 3 * 4 * 4                   # stages x variables x sides
    assert per_step == flux_calls + algebra + boundary + 1
