"""Atmospheric pressure forcing (counterpart of ``utils/AtmosphericPressure.py:26-82``).

Pressure fields are stored relative to ``shiftValue`` (1000 hPa by default)
and as float32.
"""
import numpy as np


class AtmosphericPressure:
    def __init__(self, t=None, P=None, shiftValue=100000):
        self.t = [0]
        self.P = [np.zeros((1, 1), dtype=np.float32)]
        self.numAtmPressures = 1
        if P is not None:
            if len(P) > 1:
                assert t is not None, "Missing timestamps t"
                assert len(t) == len(P), str(len(t)) + " vs " + str(len(P))
            else:
                t = self.t
            self.numAtmPressures = len(t)
            self.t = t
            self.P = [np.array(p, dtype=np.float64) for p in P]
        self.shiftValue = shiftValue if P is not None else 0
        self.P = [(p - self.shiftValue).astype(np.float32) for p in self.P]

    def getOriginalP(self):
        return [p + self.shiftValue for p in self.P]
