"""The block plan of a run to an observation time with model error.

``CDKLM16.dataAssimilationStep`` (S/CDKLM16.py:742-806, S/ =
src/gpuocean/SWEsimulators) advances a simulator to an observation time in
blocks of ``model_time_step`` seconds and adds the model error after each
block.  The time to the observation is rarely a whole number of blocks, so
one shorter block is taken FIRST (the last block before an observation must be
a full one) and its model error is scaled by sqrt(length / model_time_step);
a first block shorter than a tenth of a model time step is merged with the
next full block, and one shorter than 1e-5 of it is dropped.

Here that plan is computed up front as a list of ``Block``s, which the single
simulator and the batched ensembles then walk.  The rules that decide it (the
rounding of the time left, the two thresholds, which block gets a model
error) are those of the reference, so both take the same steps and perturb
at the same times with the same scales.
"""
from __future__ import annotations

from typing import List, NamedTuple, Optional

import numpy as np

# A first block shorter than this fraction of a model time step is merged
# with the next full block (when there is one to merge with) ...
MERGE_FRACTION = 0.1
# ... and one shorter than this fraction is not taken at all.
DROP_FRACTION = 0.00001
# dt is recomputed from the CFL condition after every DT_REFRESH_BLOCKS-th
# block a simulator has taken in its lifetime (and at the start of each run).
DT_REFRESH_BLOCKS = 5


class Block(NamedTuple):
    """One block of a run to an observation: ``length`` seconds of model
    time, then the model error scaled by ``perturbation`` (None: no model
    error after this block)."""
    length: float
    perturbation: Optional[float]


def blocks_to_observation(time_left, model_time_step, model_error_final_step=True) -> List[Block]:
    """The blocks that take a simulator ``time_left`` seconds ahead.

    The number of full blocks is the time left, rounded to whole seconds,
    over the block length (truncated); what remains of the unrounded time
    becomes a first, shorter block.  Every block is followed by model error
    except, when ``model_error_final_step`` is false, the last one.
    """
    block = model_time_step
    n_full = int(round(time_left) / block)
    first = time_left - n_full * block
    if n_full > 1 and first / block < MERGE_FRACTION:
        # too short on its own: one longer first block instead
        n_full -= 1
        first += block
    if first / block < DROP_FRACTION:
        first = 0
    assert n_full > 0, "There is less than CDKLM16.model_time_step until the observation"
    plan = []
    if first != 0:
        plan.append(Block(first, float(np.sqrt(first / block))))
    last_scale = 1.0 if model_error_final_step else None
    plan.extend(Block(block, 1.0 if k + 1 < n_full else last_scale) for k in range(n_full))
    return plan


def refresh_dt_after(blocks_taken) -> bool:
    """Whether dt is recomputed once a simulator has taken ``blocks_taken``
    blocks in total."""
    return blocks_taken % DT_REFRESH_BLOCKS == 0


def check_arrival(observation_time, t):
    """A run must end at the observation time (to the second)."""
    if round(observation_time) != round(t):
        raise AssertionError("run to observation time %r ended at t = %r (off by %r s)"
                             % (observation_time, t, t - observation_time))
