"""The drift fixtures (tests/golden/drift_dam32.npz, drift_dam128.npz) are the
single-threaded oracle's trajectories, written by tests/golden/make_drift.py.
The oracle is deterministic, so its first steps from the seeded start must
reproduce the committed 32^3 fixture bit for bit (CPU only)."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_dam32_fixture_matches_oracle_first_steps():
    from fluid_simulator_gb300.scenes import GridSpec, dam_break
    from oracle import oracle as O

    path = os.path.join(HERE, "golden", "drift_dam32.npz")
    if not os.path.exists(path):
        pytest.skip("fixture not present")
    gold = np.load(path)
    O.build_port()
    res, dt, every = 32, float(gold["dt"]), int(gold["sample_every"])
    idx = gold["tracked"]
    o = O.Oracle(O.make_params(res, transfer=O.FLIP, tol=1e-6, max_iters=200),
                 dam_break(GridSpec(res), seed=0).astype(np.float64), lib="port")
    o.set_threads(1)
    for s in range(1, 2 * every + 1):
        its = o.step(dt)
        pos, vel, _ = o.particles()
        assert its == int(gold["flip_stats"][s - 1, 6])
        assert float((o.grid(O.F_FLAGS) == O.WATER).sum()) == gold["flip_stats"][s - 1, 0]
        if s % every == 0:
            k = s // every - 1
            assert np.array_equal(pos[idx].astype(np.float32), gold["flip_pos"][k])
            assert np.array_equal(vel[idx].astype(np.float32), gold["flip_vel"][k])
    o.close()
