"""NetCDF output, hot start and model error from file on the GPU: the
reference's regression (T/schemes/NetCDF_test.py) and a continued run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _double_jet(gpu_ctx, **kw):
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils import BenchmarkCases, Common
    c = BenchmarkCases.double_jet_case(nx=96, ny=64, dx=5000.0, dy=5000.0, seed=11)
    return CDKLM16.CDKLM16(gpu_ctx, c["eta0"], c["hu0"], c["hv0"], c["H"], 96, 64, c["dx"], c["dy"], 0.0, c["g"],
                           c["f"], c["r"], coriolis_beta=c["coriolis_beta"],
                           boundary_conditions=Common.BoundaryConditions(*c["boundary"]), **kw)


# attributes that name device resources or are set by the file's own run
_SKIP = {"stream_handle", "t"}


def test_simulator_and_model_error_from_file(gpu_ctx, tmp_path):
    """A simulator written at construction, with a SOAR model error set and
    the file closed, comes back from the file with the same scalar
    attributes, and so does its model error (the reference's test)."""
    from gpuocean_gb300.SWEsimulators import CDKLM16
    fn = str(tmp_path / "netcdf_test" / "netcdf_test.nc")
    sim = _double_jet(gpu_ctx, write_netcdf=True, netcdf_filename=fn, model_time_step=60.0)
    sim.setSOARModelError(small_scale_perturbation_amplitude=3e-3, small_scale_perturbation_interpolation_factor=3)
    sim.closeNetCDF()
    file_sim = CDKLM16.CDKLM16.fromfilename(gpu_ctx, fn, cont_write_netcdf=False)
    file_sim.setModelErrorFromFile(fn)
    try:
        compared = 0
        for attr in dir(sim):
            if attr.startswith("__") or attr in _SKIP:
                continue
            a = getattr(sim, attr)
            if np.isscalar(a):
                assert a == getattr(file_sim, attr), attr
                compared += 1
        assert round(sim.t) == round(file_sim.t)
        assert compared > 20
        compared = 0
        for attr in dir(sim.model_error):
            if attr.startswith("__"):
                continue
            a = getattr(sim.model_error, attr)
            if np.isscalar(a):
                assert a == getattr(file_sim.model_error, attr), "model_error." + attr
                compared += 1
        assert compared > 5
    finally:
        file_sim.cleanUp()
        sim.cleanUp()


def test_hot_start_continues_the_run(gpu_ctx, tmp_path):
    """The state written after 20 minutes, read back into a new simulator,
    continues as the original run does (bit for bit)."""
    from gpuocean_gb300.SWEsimulators import CDKLM16
    from gpuocean_gb300.utils.SimReader import SimNetCDFReader
    fn = str(tmp_path / "hot_start")
    a = _double_jet(gpu_ctx, write_netcdf=True, netcdf_filename=fn)
    for _ in range(2):
        a.step(600.0)
    a.closeNetCDF()
    r = SimNetCDFReader(fn + ".nc", ignore_ghostcells=False)
    assert r.getNumTimeSteps() == 3  # construction + two calls of step
    eta, hu, hv, t = r.getLastTimeStep()
    assert t == np.float32(a.t)
    for x, y in zip((eta, hu, hv), a.download()):
        np.testing.assert_array_equal(x, np.asarray(y))
    r.close()
    b = CDKLM16.CDKLM16.fromfilename(gpu_ctx, fn + ".nc", cont_write_netcdf=False)
    try:
        assert b.dt == a.dt and b.nx == a.nx and str(b.boundary_conditions) == str(a.boundary_conditions)
        na, nb = a.num_iterations, b.num_iterations
        a.step(900.0)
        b.step(900.0)
        assert a.num_iterations - na == b.num_iterations - nb > 0
        for x, y in zip(a.download(), b.download()):
            np.testing.assert_array_equal(np.asarray(x)[2:-2, 2:-2], np.asarray(y)[2:-2, 2:-2])
    finally:
        b.cleanUp()
        a.cleanUp()
