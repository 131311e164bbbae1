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
