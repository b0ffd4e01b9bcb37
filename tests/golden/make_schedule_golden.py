"""Golden call traces of the reference's ``CDKLM16.dataAssimilationStep``.

``dataAssimilationStep`` (src/gpuocean/SWEsimulators/CDKLM16.py:742-806) is
pure host logic: it decides, from the time left to an observation, which
``step`` / ``perturbState`` / ``perturbSimilarAs`` / ``updateDt`` calls a
simulator (and its coarse partner) makes.  This script imports the method
from a reference checkout (PyCUDA, matplotlib and netCDF4 replaced by inert
stubs) and runs it unchanged on recording stand-ins for the simulators, for
a set of observation times, block lengths, start times and flags, and writes
the recorded call sequences to ``assimilation_schedule_reference.json`` next
to this file.  ``tests/test_observation_schedule_cpu.py`` replays the same
cases through this package's ``dataAssimilationStep`` and compares.

Usage:  python tests/golden/make_schedule_golden.py REFERENCE_ROOT (or $GPUOCEAN_REFERENCE)
"""
import json
import os
import sys
from unittest import mock

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from schedule_cases import CASES, Recorder  # noqa: E402


def import_reference(root):
    sys.dont_write_bytecode = True   # the checkout is read-only: no __pycache__ inside it
    for name in ["pycuda", "pycuda.driver", "pycuda.gpuarray", "pycuda.compiler", "pycuda.curandom",
                 "pycuda.autoinit", "matplotlib", "matplotlib.pyplot", "matplotlib.gridspec",
                 "matplotlib.animation", "matplotlib.colors", "netCDF4", "mpi4py"]:
        sys.modules.setdefault(name, mock.MagicMock())
    sys.path.insert(0, os.path.join(root, "src"))
    from gpuocean.SWEsimulators import CDKLM16
    return CDKLM16.CDKLM16


def run_case(method, case):
    log = []
    sim = Recorder("self", case["t0"], case["model_time_step"], case["total_time_steps"], log)
    other = Recorder("other", case["t0"], case["model_time_step"], 0, log) if case["partner"] else None
    try:
        method(sim, case["observation_time"], otherSim=other, model_error_final_step=case["final"],
               write_now=False)
        outcome = "ok"
    except AssertionError:
        outcome = "assertion"
    return {"calls": log, "outcome": outcome, "blocks_after": sim.total_time_steps}


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GPUOCEAN_REFERENCE")
    if not root:
        sys.exit("usage: %s REFERENCE_ROOT (or set GPUOCEAN_REFERENCE)" % sys.argv[0])
    cls = import_reference(root)
    out = [dict(case, **run_case(cls.dataAssimilationStep, case)) for case in CASES]
    with open(os.path.join(HERE, "assimilation_schedule_reference.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", len(out), "traces")


if __name__ == "__main__":
    main()
