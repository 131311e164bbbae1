"""Host logic of the studies: the Strouhal estimate from a lift history
(collision_check.py:27-31 computes the number as the rFFT peak of the lift
times D/U; the estimator here adds a window and a parabolic peak refinement)."""

import numpy as np
import pytest


@pytest.mark.parametrize("st_true", [0.163, 0.2, 0.2137])
def test_strouhal_of_a_sampled_sine(st_true):
    import studies
    every, d, u = 10, 32.0, 0.08
    period_steps = d / (st_true * u)
    t = np.arange(0, 15000, every, dtype=np.float64)
    lift = 0.4 * np.sin(2 * np.pi * t / period_steps + 0.3) + 0.05 + 0.01 * np.cos(2 * np.pi * t / 7000)
    st = studies.strouhal(lift, every, d, u)
    # bin width here is D / (U * 15000) = 0.027; the refined peak is well inside it
    assert abs(st - st_true) < 0.004, st


def test_raw_strouhal_grid_of_collision_check():
    """collision_check.py's raw estimator: second half of the history, rFFT
    peak, St = f D / U on a grid of D / (U * steps / 2) (collision_check.py:27-30).
    With the default Solver (D = 24, U = 0.08, a report every 50 steps) 8000
    steps give a 0.075 grid, on which 0.200 does not lie; 6000 and 12000 steps
    give 0.1 and 0.05. The peak lands on a grid point next to the true value."""
    import studies
    every, d, u = 50, 24.0, 0.08
    for steps, grid in ((8000, 0.075), (6000, 0.1), (12000, 0.05), (24000, 0.025)):
        t = np.arange(every, steps + 1, every, dtype=np.float64)
        for st_true in (0.19, 0.2, 0.22):
            lift = 0.5 * np.sin(2 * np.pi * t * st_true * u / d)
            st, bin_ = studies.raw_strouhal(lift, every, d, u)
            assert bin_ == pytest.approx(grid)
            assert abs(st / grid - round(st / grid)) < 1e-9          # on the grid
            assert abs(st - st_true) <= grid + 1e-12                   # a neighbouring grid point
