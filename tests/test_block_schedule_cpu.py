"""The batched engine's vectorised block schedule against the per-member
schedule of ``CDKLM16.step`` (S/CDKLM16.py:493-509): the same dt sequences,
bit for bit, for members with different dts, block lengths that are and are
not multiples of dt, and members left out of the block."""
import numpy as np

from gpuocean_gb300.ensembles.BatchedEnsemble import step_schedule, step_schedules


def test_vectorised_schedules_equal_per_member_schedules():
    rng = np.random.default_rng(1)
    for trial in range(100):
        n = 37
        dts = rng.uniform(0.5, 80.0, n).astype(np.float32)
        if trial % 3 == 0:
            dts[:9] = np.float32(60.0) / np.float32(rng.integers(1, 9))
        t_end = float(rng.choice([60.0, 59.99, 600.0, 1.0, 123.456, 0.0]))
        active = rng.random(n) > 0.2
        table, count = step_schedules(dts, t_end, active)
        for m in range(n):
            ref = step_schedule(dts[m], t_end) if active[m] else []
            got = list(table[m, :count[m]])
            assert len(got) == len(ref)
            assert all(np.float32(a).tobytes() == np.float32(b).tobytes() for a, b in zip(ref, got))
            assert not table[m, count[m]:].any()
