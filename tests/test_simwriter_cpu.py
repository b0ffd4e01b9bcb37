"""NetCDF writer and reader on the host (no GPU): a stand-in simulator with the
attributes the writer reads, written over a few time steps and read back
(the layout of the reference's U/SimWriter.py and U/SimReader.py)."""
import numpy as np

from gpuocean_gb300.utils import Common
from gpuocean_gb300.utils.SimReader import SimNetCDFReader
from gpuocean_gb300.utils.SimWriter import SimNetCDFWriter


class _Bathymetry:
    def __init__(self, Hi, Hm):
        self.Hi, self.Hm = Hi, Hm

    def download(self, stream):
        return self.Hi, self.Hm


class _Wind:
    source_filename = None


class _Noise:
    def __init__(self):
        self.soar_q0 = np.float32(2.5e-3)
        self.interpolation_factor = np.int32(3)


class OceanStateNoise(_Noise):
    pass


class CDKLM16:
    """Host stand-in with the attributes SimNetCDFWriter reads."""

    def __init__(self, nx, ny, rng):
        self.nx, self.ny, self.dx, self.dy = nx, ny, np.float32(2000.0), np.float32(3000.0)
        self.ghost_cells_x = self.ghost_cells_y = 2
        self.gpu_stream = None
        self.boundary_conditions = Common.BoundaryConditions(1, 2, 1, 2)
        self.rk_order, self.theta, self.f, self.coriolis_beta = 2, np.float32(1.3), np.float32(1.2e-4), np.float32(2e-11)
        self.y_zero_reference_cell = np.float32(2.0)
        self.A, self.g, self.r = "NA", np.float32(9.81), np.float32(0.0)
        self.dt, self.t, self.model_time_step = np.float32(15.5), 0.0, np.float32(60.0)
        self.wind_stress = _Wind()
        self.model_error = None
        self.bathymetry = _Bathymetry(rng.uniform(50, 60, (ny + 5, nx + 5)).astype(np.float32),
                                      rng.uniform(50, 60, (ny + 4, nx + 4)).astype(np.float32))
        self.rng = rng
        self.state = None
        self.advance(0.0)

    def advance(self, dt):
        self.t += dt
        self.state = tuple(self.rng.standard_normal((self.ny + 4, self.nx + 4)).astype(np.float32) for _ in range(3))

    def download(self):
        return self.state


def test_write_read_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    sim = CDKLM16(20, 14, rng)
    fn = str(tmp_path / "out" / "run")
    states = []
    with SimNetCDFWriter(sim, filename=fn) as w:
        states.append((sim.t, sim.state))
        for _ in range(3):
            sim.advance(60.0)
            w.writeTimestep(sim)
            states.append((sim.t, sim.state))
        sim.model_error = OceanStateNoise()
        w.writeModelError(sim)
        name = w.output_file_name
    assert name == fn + ".nc"

    r = SimNetCDFReader(name, ignore_ghostcells=False)
    assert r.get("simulator_short") == "CDKLM16"
    assert r.get("nx") == 20 and r.get("ny") == 14
    assert r.get("dx") == np.float32(2000.0) and r.get("dt") == np.float32(15.5)
    assert r.get("time_integrator") == 2 and r.get("minmod_theta") == np.float32(1.3)
    assert r.get("coriolis_force") == np.float32(1.2e-4) and r.get("coriolis_beta") == np.float32(2e-11)
    assert r.get("has_model_error") == "True" and r.get("model_error_name") == "OceanStateNoise"
    assert r.get("small_scale_perturbation_amplitude") == np.float32(2.5e-3)
    assert r.get("small_scale_perturbation_interpolation_factor") == 3
    assert r.get("missing") == "not found" and not r.has("missing") and r.has("eta") and r.has("nx")
    assert str(r.getBC()) == str(sim.boundary_conditions)
    assert r.getNumTimeSteps() == 4
    np.testing.assert_array_equal(r.getTimes(), np.float32([t for t, _ in states]))
    np.testing.assert_array_equal(r.getH(), sim.bathymetry.Hi)
    np.testing.assert_array_equal(r.getHm(), sim.bathymetry.Hm)
    for k, (t, st) in enumerate(states):
        eta, hu, hv, tt = r.getTimeStep(k)
        assert tt == np.float32(t)
        for a, b in zip((eta, hu, hv), st):
            np.testing.assert_array_equal(a, b)
    eta, hu, hv, tt = r.getLastTimeStep()
    np.testing.assert_array_equal(eta, states[-1][1][0])
    eta, hu, hv, tt = r.getStateAtTime(120.0)
    np.testing.assert_array_equal(hv, states[2][1][2])
    r.close()

    # interior only
    r = SimNetCDFReader(name, ignore_ghostcells=True)
    eta, hu, hv, tt = r.getTimeStep(1)
    np.testing.assert_array_equal(eta, states[1][1][0][2:-2, 2:-2])
    x, y = r.getAxis()
    assert x.shape == (20,) and y.shape == (14,)
    assert x[0] == np.float32(1000.0)
    r.close()


def test_boundary_conditions_text_round_trip():
    for bc in (Common.BoundaryConditions(), Common.BoundaryConditions(2, 2, 2, 2),
               Common.BoundaryConditions(3, 4, 3, 4, spongeCells={"north": 10, "south": 10, "east": 5, "west": 5})):
        back = Common.BoundaryConditions.fromstring(str(bc))
        assert (back.north, back.east, back.south, back.west) == (bc.north, bc.east, bc.south, bc.west)
        assert {k: int(v) for k, v in back.spongeCells.items()} == {k: int(v) for k, v in bc.spongeCells.items()}


def test_reader_returns_native_byte_order(tmp_path):
    """Arrays handed to the simulators are uploaded as raw bytes: the reader
    returns them in the machine's byte order (the file holds big-endian)."""
    rng = np.random.default_rng(5)
    sim = CDKLM16(8, 6, rng)
    with SimNetCDFWriter(sim, filename=str(tmp_path / "n")) as w:
        name = w.output_file_name
    r = SimNetCDFReader(name, ignore_ghostcells=False)
    eta, hu, hv, t = r.getLastTimeStep()
    for a in (eta, hu, hv, r.getH(), r.getHm(), r.getTimes()):
        assert a.dtype.isnative
    np.testing.assert_array_equal(np.frombuffer(eta.tobytes(), np.float32).reshape(eta.shape), sim.state[0])
    r.close()
