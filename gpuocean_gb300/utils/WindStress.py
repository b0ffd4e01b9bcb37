"""Wind stress forcing (counterpart of the reference's ``utils/WindStress.py:39-121``).

Holds time stamps and 2D fields of wind (m/s) and/or wind stress.  When only
wind is given, the stress follows the drag law of the reference
(U/WindStress.py:86-121): C_d = 1.2e-3 below 11 m/s, else 4.9e-4 + 6.5e-5 |W|,
tau = rho_air/rho_water * C_d |W| W.
"""
import numpy as np


class WindStress:
    def __init__(self, source_filename=None, t=None, wind_u=None, wind_v=None, stress_u=None, stress_v=None):
        self.source_filename = source_filename
        self.t = [0]
        self.wind_u = [np.zeros((1, 1), dtype=np.float32)]
        self.wind_v = [np.zeros((1, 1), dtype=np.float32)]
        self.stress_u = None
        self.stress_v = None
        self.numWindSteps = 1
        if t is not None:
            assert wind_u is not None or stress_u is not None, "any information in x direction missing"
            assert wind_v is not None or stress_v is not None, "any information in y direction missing"
            n = len(t)
            for arr in (wind_u, wind_v, stress_u, stress_v):
                if arr is not None:
                    assert len(arr) == n, str(n) + " vs " + str(len(arr))
                    for a in arr:
                        assert a.dtype == np.float32, "Wind data needs to be of type np.float32"
            self.numWindSteps = n
            self.t = t
            if wind_u is not None:
                self.wind_u, self.wind_v = wind_u, wind_v
            self.stress_u, self.stress_v = stress_u, stress_v

    def compute_wind_stress_from_wind(self, wind_u=None, wind_v=None):
        wind_u = self.wind_u if wind_u is None else wind_u
        wind_v = self.wind_v if wind_v is None else wind_v
        self.stress_u, self.stress_v = [], []
        rho_a, rho_w = 1.225, 1025
        for i in range(self.numWindSteps):
            speed = np.sqrt(np.power(wind_u[i], 2) + np.power(wind_v[i], 2))
            c_drag = np.where(speed < 11, 0.0012, 0.00049 + 0.000065 * speed)
            stress = c_drag * speed * rho_a / rho_w
            self.stress_u.append((stress * wind_u[i]).astype(np.float32))
            self.stress_v.append((stress * wind_v[i]).astype(np.float32))
