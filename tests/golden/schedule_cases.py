"""Cases and a recording stand-in simulator for the observation-schedule
traces (shared by ``make_schedule_golden.py`` and the CPU test)."""
import numpy as np

# (observation time, block length, start time, blocks taken before, coarse
# partner, model error after the final block)
_RAW = [
    (180.0, 60.0, 0.0, 0, False, True),      # whole number of blocks: first block merged
    (60.0, 60.0, 0.0, 0, False, True),       # exactly one block
    (200.0, 60.0, 0.0, 0, False, True),      # leftover of a third of a block
    (183.0, 60.0, 0.0, 0, False, True),      # short leftover merged into a longer first block
    (63.0, 60.0, 0.0, 0, False, True),       # short leftover, nothing to merge with
    (60.2, 60.0, 0.0, 0, False, True),       # tiny leftover, above the drop threshold
    (60.0005, 60.0, 0.0, 0, False, True),    # leftover below the drop threshold
    (179.6, 60.0, 0.0, 0, False, True),      # time left rounds up: negative leftover merged
    (59.9995, 60.0, 0.0, 0, False, True),    # time left rounds up to one block
    (30.0, 60.0, 0.0, 0, False, True),       # less than a block: assertion
    (600.0, 60.0, 0.0, 0, False, True),      # ten blocks: dt refreshed after blocks 5 and 10
    (400.0, 60.0, 0.0, 3, False, True),      # counter carried over: refresh after the 2nd and 7th block
    (3600.0, 60.0, 3000.0, 0, True, True),   # coarse partner, start time not zero
    (250.0, 60.0, 0.0, 0, True, False),      # partner, no model error after the final block
    (900.0, 100.0, 0.0, 4, True, False),     # another block length
    (1000.0, 60.0, 700.0, 0, False, False),  # leftover with the final block deterministic
]

CASES = [dict(observation_time=o, model_time_step=m, t0=t0, total_time_steps=n, partner=p, final=f)
         for o, m, t0, n, p, f in _RAW]


class Recorder:
    """Stands in for a simulator: records the calls dataAssimilationStep
    makes and advances t by the length of every step."""

    def __init__(self, name, t, model_time_step, total_time_steps, log):
        self.name = name
        self.t = float(t)
        self.model_time_step = model_time_step
        self.total_time_steps = total_time_steps
        self.write_netcdf = False
        self.log = log

    def step(self, t_end, apply_stochastic_term=True, write_now=True, update_dt=False):
        self.log.append([self.name, "step", float(t_end), bool(apply_stochastic_term)])
        self.t += float(t_end)
        return self.t

    def perturbState(self, perturbation_scale=1.0, update_random_field=True, q0_scale=1):
        self.log.append([self.name, "perturbState", float(perturbation_scale)])

    def perturbSimilarAs(self, otherSim, perturbation_scale=1.0):
        self.log.append([self.name, "perturbSimilarAs", otherSim.name, float(np.float64(perturbation_scale))])

    def updateDt(self, courant_number=None):
        self.log.append([self.name, "updateDt", courant_number])
