"""The allocation-free monitor sums (lbm_field_sums_static) against the solver's own.

lbm_field_sums_static serves callers that cannot allocate device memory while
they run (an in-situ pipeline or host framework that owns every device buffer,
or a fixed device footprint): they pass the report fields and an output, and
the scratch lives in a static device array. This file is collected last, so a
run that stops at the first failure has run every other test before it.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SUM_FIELDS = ("r_rho", "r_ux", "r_uy", "r_uz", "r_ke", "fx", "fy", "fz")


def test_static_sums_match_solver_sums_twice():
    import lbm
    import lbm_native as N

    lib = N.load()
    s = lbm.Solver(96, 48, 12, collision="les", obstacle="cylinder", diameter=10.0,
                   lateral="slip", vertical="slip", init="random", seed=11)
    out = lbm.ManagedArray(16)              # 64 bytes the GPU can write: 8 doubles
    sums = out.numpy.view(np.float64)
    ptrs = (ctypes.c_void_p * 8)(*(s.fields[k].ptr for k in SUM_FIELDS))
    for call in range(2):
        for _ in range(3):
            s.step()
        s.step(report=True)
        want = np.array(s.field_sums())     # the solver's own FP64 sums of this report step
        sums[:] = np.nan
        status = lib.lbm_field_sums_static(ptrs, s.lat.n, ctypes.c_void_p(out.ptr), None)
        assert status == N.OK, lib.lbm_last_error()
        s.sync()
        got = sums.copy()
        assert np.all(np.isfinite(got)), f"call {call}"
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-15, err_msg=f"call {call}")
        # and the host-side FP64 sum of the same float32 fields (lbm.py:654)
        host = np.array([s.fields[k].numpy.sum(dtype=np.float64) for k in SUM_FIELDS])
        np.testing.assert_allclose(got, host, rtol=1e-9, atol=1e-15, err_msg=f"call {call}")


def test_static_sums_reject_bad_sizes():
    import lbm
    import lbm_native as N

    lib = N.load()
    a = lbm.ManagedArray(4)
    out = lbm.ManagedArray(16)
    ptrs = (ctypes.c_void_p * 8)(*([a.ptr] * 8))
    for n in (0, -1, (1 << 28) + 1):
        assert lib.lbm_field_sums_static(ptrs, n, ctypes.c_void_p(out.ptr), None) == N.ERR_ARG
        assert b"2^28" in lib.lbm_last_error()
