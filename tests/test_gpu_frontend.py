"""The XML front end end to end on the GPU: alsvinncli and alsuqcli inputs run
through config -> initial data -> Simulator / Runner -> writers, compared
with the oracle run on the same initial data (bit for bit with the exact
arithmetic variant; the statistics within the Welford-versus-sums rounding)."""
import os
import shutil

import numpy as np
import pytest

import workloads
from alsvinn_gb300 import alsuqcli, alsvinncli, config, initdata, lib, runner
from alsvinn_gb300.simulator import interior
from oracle import fvoracle

pytestmark = pytest.mark.gpu

INPUTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "inputs")


def _copy_inputs(tmp_path, names):
    for n in names:
        shutil.copy(os.path.join(INPUTS, n), str(tmp_path / n))


def _oracle_run(f, prim, end_time, saves):
    g = lib.ghost_cells(f.reconstruction)
    rc, U, t, steps = fvoracle.run(f.equation, f.flux, f.reconstruction, f.integrator, f.boundary, f.dimension,
                                   f.lower, f.upper, f.gamma, f.cfl, end_time, saves, 0,
                                   prim.reshape(prim.shape[0], -1), g, workloads.NVAR[f.equation])
    assert rc == 0
    return U, t, steps


def test_alsvinncli_sod_matches_the_oracle_at_every_save(cuda_device, tmp_path):
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    _copy_inputs(tmp_path, ["sod.xml", "sod.py"])
    xml = str(tmp_path / "sod.xml")
    assert alsvinncli.main([xml, "--precision", "fp64-exact"]) == 0
    f = config.read_config(xml).fvm
    prim = initdata.evaluate(f.python_program, f.equation, f.lower, f.upper, f.dimension, f.init_parameters)
    g = lib.ghost_cells(f.reconstruction)
    interval = f.end_time / f.writer.number_of_saves
    with netcdf(str(tmp_path / "sod_out.nc"), "r", mmap=False) as nc:
        rho, mx, E = (np.array(nc.variables[v][0]) for v in ("rho", "mx", "E"))
    for k in range(1, f.writer.number_of_saves + 1):
        # the writer's trajectory up to save k is the oracle's with k saves to k * interval
        end = f.end_time if k == f.writer.number_of_saves else k * interval
        U, t, steps = _oracle_run(f, prim, end, k)
        want = interior(U, f.dimension, g)
        got = np.stack([rho[k - 1], mx[k - 1], E[k - 1]]).reshape(want.shape)
        assert np.array_equal(got, want), k


def test_simulator_steps_like_the_reference_loop(cuda_device, tmp_path):
    """perform_step one step at a time and run() give the same state."""
    from alsvinn_gb300.simulator import Simulator
    _copy_inputs(tmp_path, ["sod.xml", "sod.py"])
    f = config.read_config(str(tmp_path / "sod.xml")).fvm
    f.writer = None
    prim = initdata.evaluate(f.python_program, f.equation, f.lower, f.upper, f.dimension)
    a = Simulator(f, lib.FP64_EXACT)
    b = Simulator(f, lib.FP64_EXACT)
    a.set_initial_value(prim)
    b.set_initial_value(prim)
    n = 0
    while not a.at_end():
        a.perform_step()
        n += 1
    b.run()
    assert n == a.get_number_of_timesteps() == b.get_number_of_timesteps()
    assert a.get_current_time() == b.get_current_time() >= f.end_time
    assert np.array_equal(a.solver.get_state(), b.solver.get_state())
    a.close()
    b.close()


def _uq_expected(cfg, end_time, saves):
    f, u = cfg.fvm, cfg.uq
    draws = runner.sample_parameters(u, range(u.sample_start, u.sample_start + u.samples))
    states = []
    for s in sorted(draws):
        p = dict(f.init_parameters)
        p.update(draws[s])
        prim = initdata.evaluate(f.python_program, f.equation, f.lower, f.upper, f.dimension, p)
        states.append(_oracle_run(f, prim, end_time, saves)[0])
    return fvoracle.meanvar(states)


def _check_stats(res, m_ref, v_ref, count):
    n, mean, var = res
    assert n == count
    mean = mean.reshape(m_ref.shape)
    var = var.reshape(v_ref.shape)
    np.testing.assert_allclose(mean, m_ref, rtol=1e-13, atol=1e-15)
    # Welford M2 / n against the reference's sum(u^2)/n - mean^2
    scale = np.abs(m_ref).max(axis=1, keepdims=True) ** 2
    assert (np.abs(var - v_ref) / scale).max() < 1e-12


@pytest.mark.parametrize("engine", ["serial", "batch"])
def test_alsuq_statistics_match_the_oracle(cuda_device, tmp_path, engine):
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    _copy_inputs(tmp_path, ["kh_uq.xml", "kh_global.py"])
    xml = str(tmp_path / "kh_uq.xml")
    cfg = config.read_config(xml)
    r = runner.Runner(cfg, lib.FP64_EXACT, output_dir=str(tmp_path), engine=engine)
    results = r.run()
    assert r.engine == engine and len(results) == 1
    m_ref, v_ref = _uq_expected(cfg, cfg.fvm.end_time, 1)
    _check_stats(results[0], m_ref, v_ref, cfg.uq.samples)
    with netcdf(str(tmp_path / "kh_uq_stats_mean"), "r", mmap=False) as nc:
        g = lib.ghost_cells(cfg.fvm.reconstruction)
        want = interior(m_ref, cfg.fvm.dimension, g)
        got = np.stack([np.array(nc.variables[v][0, 0]) for v in ("rho", "mx", "my", "E")]).reshape(want.shape)
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("engine", ["serial", "batch"])
def test_alsuq_statistics_at_several_save_times(cuda_device, tmp_path, engine):
    """Mean / variance at two save times: the serial engine's statistics
    clamp, and the ensemble folding each member at its save clamp."""
    _copy_inputs(tmp_path, ["kh_uq.xml", "kh_global.py"])
    xml = str(tmp_path / "kh_uq.xml")
    text = open(xml).read().replace("<numberOfSaves>1</numberOfSaves>", "<numberOfSaves>2</numberOfSaves>")
    open(xml, "w").write(text)
    cfg = config.read_config(xml)
    r = runner.Runner(cfg, lib.FP64_EXACT, output_dir=str(tmp_path), engine=engine)
    assert r.engine == engine
    results = r.run()
    assert len(results) == 2
    T = cfg.fvm.end_time
    for k, (end, saves) in enumerate(((T / 2, 1), (T, 2))):
        m_ref, v_ref = _uq_expected(cfg, end, saves)
        _check_stats(results[k], m_ref, v_ref, cfg.uq.samples)


def test_alsuqcli_runs_the_input(cuda_device, tmp_path, capsys):
    _copy_inputs(tmp_path, ["kh_uq.xml", "kh_global.py"])
    assert alsuqcli.main([str(tmp_path / "kh_uq.xml"), "--precision", "fp32"]) == 0
    out = capsys.readouterr().out
    assert '"engine": "batch"' in out
    assert os.path.exists(str(tmp_path / "kh_uq_stats_variance"))


def test_alsuq_structure_functions_match_the_oracle(cuda_device, tmp_path):
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    _copy_inputs(tmp_path, ["kh_uq.xml", "kh_global.py"])
    xml = str(tmp_path / "kh_uq.xml")
    text = open(xml).read().replace(
        "<stats>",
        "<stats><stat><name>structure_cube</name><p>2</p><numberOfH>5</numberOfH><numberOfSaves>1</numberOfSaves>"
        "<writer><type>netcdf</type><basename>kh_uq_sf</basename></writer></stat>")
    open(xml, "w").write(text)
    cfg = config.read_config(xml)
    r = runner.Runner(cfg, lib.FP64_EXACT, output_dir=str(tmp_path))
    assert r.engine == "serial"
    r.run()
    f, u = cfg.fvm, cfg.uq
    draws = runner.sample_parameters(u, range(u.samples))
    g = lib.ghost_cells(f.reconstruction)
    want = 0
    for s in range(u.samples):
        p = dict(f.init_parameters)
        p.update(draws[s])
        prim = initdata.evaluate(f.python_program, f.equation, f.lower, f.upper, f.dimension, p)
        U = _oracle_run(f, prim, f.end_time, 1)[0]
        want = want + fvoracle.structure_cube(f.equation, f.boundary, f.dimension, g, 5, 2.0, U)
    want = want / u.samples
    n, got = r.statistics[0][0]
    assert n == u.samples
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15)
    with netcdf(str(tmp_path / "kh_uq_sf_structure_cube_2.000000"), "r", mmap=False) as nc:
        assert nc.dimensions["x"] == 5
        np.testing.assert_allclose(np.array(nc.variables["rho"][0, 0]).reshape(-1), want[0], rtol=1e-12)


FUNCTIONAL_STATS = (
    "<stat><name>onepointmoment</name><p>2</p><numberOfSaves>1</numberOfSaves>"
    "<writer><type>netcdf</type><basename>kh_m</basename></writer></stat>"
    "<stat><name>bv</name><p>1</p><numberOfSaves>1</numberOfSaves>"
    "<writer><type>netcdf</type><basename>kh_bv</basename></writer></stat>"
    "<stat><name>bv_direction</name><p>2</p><numberOfSaves>1</numberOfSaves>"
    "<writer><type>netcdf</type><basename>kh_bvd</basename></writer></stat>"
    "<stat><name>functional</name><functionalName>log_entropy</functionalName><gamma>1.4</gamma>"
    "<numberOfSaves>1</numberOfSaves><writer><type>netcdf</type><basename>kh_le</basename></writer></stat>"
    "<stat><name>functional</name><functionalName>legendre_pointwise</functionalName><degree>3</degree>"
    "<minValue>-4</minValue><maxValue>8</maxValue><variables>rho E</variables>"
    "<numberOfSaves>1</numberOfSaves><writer><type>netcdf</type><basename>kh_lp</basename></writer></stat>")


def test_alsuq_functional_statistics_match_the_oracle(cuda_device, tmp_path):
    """onepointmoment, bv, bv_direction and functional statistics (log
    entropy, Legendre) of the serial engine against the oracle's functionals
    of the oracle's runs, averaged over the samples."""
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    _copy_inputs(tmp_path, ["kh_uq.xml", "kh_global.py"])
    xml = str(tmp_path / "kh_uq.xml")
    text = open(xml).read().replace("<stats>", "<stats>" + FUNCTIONAL_STATS)
    open(xml, "w").write(text)
    cfg = config.read_config(xml)
    r = runner.Runner(cfg, lib.FP64_EXACT, output_dir=str(tmp_path))
    assert r.engine == "serial"
    r.run()
    f, u = cfg.fvm, cfg.uq
    g = lib.ghost_cells(f.reconstruction)
    draws = runner.sample_parameters(u, range(u.samples))
    states = []
    for s in range(u.samples):
        p = dict(f.init_parameters)
        p.update(draws[s])
        prim = initdata.evaluate(f.python_program, f.equation, f.lower, f.upper, f.dimension, p)
        states.append(_oracle_run(f, prim, f.end_time, 1)[0])

    def mean_of(name, **kw):
        return sum(fvoracle.functional(name, f.equation, f.boundary, f.dimension, g, f.lower, f.upper, U, **kw)[0]
                   for U in states) / u.samples

    by_name = {st.name + (st.functional.name if st.functional else ""): k for k, st in enumerate(u.stats)}
    n, got = r.statistics[by_name["onepointmoment"]][0]
    assert n == u.samples
    np.testing.assert_allclose(got[0], mean_of("moment", degree=2), rtol=1e-13)
    np.testing.assert_allclose(r.statistics[by_name["bv"]][0][1][0], mean_of("bv", degree=1), rtol=1e-12)
    # bv_direction keeps the last sample of the rank (the reference assigns its snapshot), divided by the count
    last = states[-1]
    for d in range(2):
        want = fvoracle.functional("bv_direction", f.equation, f.boundary, f.dimension, g, f.lower, f.upper, last,
                                   degree=2, direction=d)[0] / u.samples
        np.testing.assert_allclose(r.statistics[by_name["bv_direction"]][0][1][d], want, rtol=1e-12)
    np.testing.assert_allclose(r.statistics[by_name["functionallog_entropy"]][0][1][0],
                               mean_of("log_entropy", gamma=1.4), rtol=1e-12)
    lp = mean_of("legendre_pointwise", degree=3, min_value=-4.0, max_value=8.0, variables="rho E")
    np.testing.assert_allclose(r.statistics[by_name["functionallegendre_pointwise"]][0][1][0], lp, rtol=1e-14,
                               atol=1e-16)
    # the files carry the reference's statistic names
    for base, names in (("kh_m", ["m2"]), ("kh_bv", ["bv_1"]), ("kh_bvd", ["bv_x_2", "bv_y_2", "bv_z_2"]),
                        ("kh_le", ["mean_log_entropy"]), ("kh_lp", ["mean_legendre_pointwise"])):
        for nm in names:
            path = tmp_path / ("%s_%s" % (base, nm))
            assert path.exists(), path
            with netcdf(str(path), "r", mmap=False) as nc:
                assert "rho" in nc.variables


def _padded(interior_values, n, g):
    """A padded array (nvar, total) holding the interior values, zero ghosts."""
    dim = 3 if n[2] > 1 else (2 if n[1] > 1 else 1)
    t = [n[d] + 2 * g if d < dim else n[d] for d in range(3)]
    V = np.zeros((interior_values.shape[0], t[2], t[1], t[0]))
    gz, gy = (g if dim > 2 else 0), (g if dim > 1 else 0)
    V[:, gz:gz + n[2], gy:gy + n[1], g:g + n[0]] = interior_values.reshape(interior_values.shape[0], n[2], n[1], n[0])
    return V.reshape(V.shape[0], -1)


def test_alsvinncli_functionals_write_at_their_save_times(cuda_device, tmp_path):
    """<functionals>: identity every endTime / 2 (a second save clamp beside
    the writer's endTime / 3) and log entropy every endTime / 3 (sharing the
    writer's clamp), both written at t = 0 and at each of their save times."""
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    _copy_inputs(tmp_path, ["sod.xml", "sod.py"])
    xml = str(tmp_path / "sod.xml")
    text = open(xml).read().replace("<writer>", (
        "<functionals>"
        "<functional><name>identity</name><numberOfSaves>2</numberOfSaves>"
        "<writer><type>netcdf</type><basename>sod_id</basename><numberOfSaves>2</numberOfSaves></writer>"
        "</functional>"
        "<functional><name>log_entropy</name><numberOfSaves>3</numberOfSaves>"
        "<writer><type>netcdf</type><basename>sod_le</basename><numberOfSaves>3</numberOfSaves></writer>"
        "</functional></functionals><writer>"), 1)
    open(xml, "w").write(text)
    assert alsvinncli.main([xml, "--precision", "fp64-exact"]) == 0
    f = config.read_config(xml).fvm
    g = lib.ghost_cells(f.reconstruction)
    n = f.dimension
    prim = initdata.evaluate(f.python_program, f.equation, f.lower, f.upper, f.dimension, f.init_parameters)
    U0 = fvoracle.prim_to_cons(f.equation, n, g, f.gamma, _padded(prim.reshape(prim.shape[0], -1), n, g))
    with netcdf(str(tmp_path / "sod_out.nc"), "r", mmap=False) as nc:
        states = [np.stack([np.array(nc.variables[v][0, k]) for v in ("rho", "mx", "E")]) for k in range(3)]
    with netcdf(str(tmp_path / "sod_id"), "r", mmap=False) as nc:
        ident = [np.stack([np.array(nc.variables[v][0, k]) for v in ("rho", "mx", "E")]) for k in range(3)]
    with netcdf(str(tmp_path / "sod_le"), "r", mmap=False) as nc:
        le = np.array(nc.variables["E"][0]).reshape(4)
    # the identity at t = 0 is the initial state; at the end it equals the writer's last save
    assert np.array_equal(ident[0].reshape(3, -1), interior(U0, n, g).reshape(3, -1))
    assert np.array_equal(ident[2], states[2])
    # log entropy at t = 0 and at the writer's three save times (the same clamp)
    want = [fvoracle.functional("log_entropy", f.equation, f.boundary, n, g, f.lower, f.upper, U0, gamma=f.gamma)[0]]
    for k in range(3):
        Uk = _padded(states[k].reshape(3, -1), n, g)
        want.append(fvoracle.functional("log_entropy", f.equation, f.boundary, n, g, f.lower, f.upper, Uk,
                                        gamma=f.gamma)[0])
    np.testing.assert_allclose(le, [w[-1, 0] for w in want], rtol=1e-12)


def test_batch_engine_writes_the_fvm_writer_like_the_serial_engine(cuda_device, tmp_path):
    """An alsuqcli input with an fvm writer runs on the ensemble engine: the
    writer is each member's second save clamp, the wave stops at every
    writer save and the host writes the members' states. The file equals
    the serial engine's bit for bit (exact variant); the statistics, taken
    at two save times that differ from the writer's three, match the
    serial engine's to the Welford fold order's rounding."""
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    out = {}
    for engine in ("serial", "batch"):
        d = tmp_path / engine
        d.mkdir()
        _copy_inputs(d, ["kh_uq.xml", "kh_global.py"])
        xml = str(d / "kh_uq.xml")
        text = open(xml).read().replace("<numberOfSaves>1</numberOfSaves>", "<numberOfSaves>2</numberOfSaves>")
        text = text.replace("</integrator>", "</integrator>\n  <writer><type>netcdf</type><basename>kh_uq_fvm</basename>"
                            "<numberOfSaves>3</numberOfSaves><writeInitialTimestep>1</writeInitialTimestep>"
                            "</writer>")
        open(xml, "w").write(text)
        cfg = config.read_config(xml)
        r = runner.Runner(cfg, lib.FP64_EXACT, output_dir=str(d), engine=engine)
        assert r.engine == engine
        stats = r.run()
        with netcdf(str(d / "kh_uq_fvm"), "r", mmap=False) as nc:
            arrays = {v: np.array(nc.variables[v][:]) for v in ("rho", "mx", "my", "E")}
        out[engine] = (stats, arrays, r.timesteps)
    (s_stats, s_arr, s_steps), (b_stats, b_arr, b_steps) = out["serial"], out["batch"]
    assert s_steps == b_steps
    for v in s_arr:
        assert s_arr[v].shape[:2] == (4, 4)  # members x (initial + 3 saves)
        assert np.array_equal(s_arr[v], b_arr[v]), v
    assert len(s_stats) == len(b_stats) == 2
    for (n1, m1, v1), (n2, m2, v2) in zip(s_stats, b_stats):
        assert n1 == n2 == 4
        np.testing.assert_allclose(m2, m1, rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(v2, v1, rtol=1e-9, atol=1e-13)
