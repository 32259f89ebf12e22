"""The axis structure function (alsuq's structure_basic) on the device
against the oracle (pinned to the reference's StructureBasic by
tests/golden/structure_basic.npz), and as an alsuqcli statistic."""
import os
import shutil

import numpy as np
import pytest

import workloads
from alsvinn_gb300 import config, initdata, lib, runner
from oracle import fvoracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(workloads.STRUCTURE_BASIC_CASES))
@pytest.mark.parametrize("precision", [lib.FP64, lib.FP32])
def test_structure_basic_matches_the_oracle(cuda_device, name, precision):
    import torch
    eq, bc, n, g, H, p, d = workloads.STRUCTURE_BASIC_CASES[name]
    U = workloads.smooth_random_state(eq, workloads.padded_shape(n, g), np.random.default_rng(11))
    if precision == lib.FP32:
        U = U.astype(np.float32).astype(np.float64)
    want = fvoracle.structure_basic(eq, bc, n, g, H, p, d, U)
    s = lib.Structure(bc, n, g, workloads.NVAR[eq], H, p, direction=d)
    try:
        dt = torch.float32 if precision == lib.FP32 else torch.float64
        x = torch.tensor(U, dtype=dt, device="cuda")
        s.add_device(x.data_ptr(), precision)
        s.add_device(x.data_ptr(), precision)
        got, count = s.result()
        assert count == 2
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15)
    finally:
        s.close()


def test_alsuq_structure_basic_statistic(cuda_device, tmp_path):
    inputs = os.path.join(os.path.dirname(os.path.abspath(__file__)), "inputs")
    for f in ("kh_uq.xml", "kh_global.py"):
        shutil.copy(os.path.join(inputs, f), str(tmp_path / f))
    xml = str(tmp_path / "kh_uq.xml")
    text = open(xml).read().replace(
        "<stats>", "<stats><stat><name>structure_basic</name><direction>1</direction><p>2</p><numberOfH>4</numberOfH>"
        "<numberOfSaves>1</numberOfSaves><writer><type>netcdf</type><basename>kh_sb</basename></writer></stat>")
    open(xml, "w").write(text)
    cfg = config.read_config(xml)
    assert cfg.uq.stats[0].output_names() == ["structure_basic_2.000000"]
    r = runner.Runner(cfg, lib.FP64_EXACT, output_dir=str(tmp_path))
    r.run()
    f, u = cfg.fvm, cfg.uq
    g = lib.ghost_cells(f.reconstruction)
    draws = runner.sample_parameters(u, range(u.samples))
    want = 0
    for s in range(u.samples):
        prm = dict(f.init_parameters)
        prm.update(draws[s])
        prim = initdata.evaluate(f.python_program, f.equation, f.lower, f.upper, f.dimension, prm)
        rc, U, t, steps = fvoracle.run(f.equation, f.flux, f.reconstruction, f.integrator, f.boundary, f.dimension,
                                       f.lower, f.upper, f.gamma, f.cfl, f.end_time, 1, 0,
                                       prim.reshape(prim.shape[0], -1), g, workloads.NVAR[f.equation])
        assert rc == 0
        want = want + fvoracle.structure_basic(f.equation, f.boundary, f.dimension, g, 4, 2.0, 1, U)
    n, got = r.statistics[0][0]
    assert n == u.samples
    np.testing.assert_allclose(got, want / u.samples, rtol=1e-12, atol=1e-15)
    assert (tmp_path / "kh_sb_structure_basic_2.000000").exists()
