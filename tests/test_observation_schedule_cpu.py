"""The run-to-observation plan (``CDKLM16.dataAssimilationStep``) against
call traces recorded from the reference's own method
(``tests/golden/make_schedule_golden.py``): the same steps, model errors
(with their scales), partner perturbations and dt refreshes, in the same
order, for leftover, merged, dropped and whole-block cases; and the block
plan itself for a few cases written out by hand."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from schedule_cases import CASES, Recorder  # noqa: E402

from gpuocean_gb300.SWEsimulators import CDKLM16  # noqa: E402
from gpuocean_gb300.SWEsimulators.ObservationSchedule import Block, blocks_to_observation  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "assimilation_schedule_reference.json")


def _run(case):
    log = []
    sim = Recorder("self", case["t0"], case["model_time_step"], case["total_time_steps"], log)
    other = Recorder("other", case["t0"], case["model_time_step"], 0, log) if case["partner"] else None
    try:
        CDKLM16.CDKLM16.dataAssimilationStep(sim, case["observation_time"], otherSim=other,
                                             model_error_final_step=case["final"], write_now=False)
        outcome = "ok"
    except AssertionError:
        outcome = "assertion"
    return log, outcome, sim.total_time_steps


def _same(a, b):
    if len(a) != len(b):
        return False
    for x, y in zip(a, b):
        if isinstance(x, float) or isinstance(y, float):
            if not (isinstance(x, (int, float)) and isinstance(y, (int, float))):
                return False
            if not np.isclose(x, y, rtol=1e-15, atol=0.0):
                return False
        elif x != y:
            return False
    return True


def test_golden_covers_the_cases():
    with open(GOLDEN) as f:
        golden = json.load(f)
    assert [{k: g[k] for k in CASES[0]} for g in golden] == CASES


@pytest.mark.parametrize("idx", range(len(CASES)))
def test_trace_matches_reference(idx):
    with open(GOLDEN) as f:
        golden = json.load(f)[idx]
    log, outcome, n = _run(CASES[idx])
    assert outcome == golden["outcome"]
    if outcome == "ok":
        assert n == golden["blocks_after"]
        assert len(log) == len(golden["calls"])
        for got, want in zip(log, golden["calls"]):
            assert _same(got, want), (got, want)


def test_plan_by_hand():
    r = np.sqrt
    assert blocks_to_observation(180.0, 60.0) == [Block(60.0, 1.0)] * 3
    assert blocks_to_observation(200.0, 60.0) == [Block(20.0, float(r(20 / 60)))] + [Block(60.0, 1.0)] * 3
    assert blocks_to_observation(183.0, 60.0) == [Block(63.0, float(r(63 / 60))), Block(60.0, 1.0), Block(60.0, 1.0)]
    assert blocks_to_observation(63.0, 60.0) == [Block(3.0, float(r(3 / 60))), Block(60.0, 1.0)]
    assert blocks_to_observation(60.0005, 60.0, model_error_final_step=False) == [Block(60.0, None)]
    with pytest.raises(AssertionError):
        blocks_to_observation(30.0, 60.0)
