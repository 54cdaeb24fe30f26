"""Failure path of the split-precision engine, exercised without a GPU fault.

Every barrier wait of the tcgen05 grouped GEMM is bounded.  Here the main-loop
waits get a budget of one clock cycle (vmps_ctx_set_wait_budget), far below the
time a tile's copies and MMAs take, so waits run out: the kernel stops issuing
work, the copies and MMAs already in flight drain under the normal ~2 s budget,
tensor memory is released and the call returns VMPS_E_TIMEOUT.  The context must
stay usable: with the default budget restored the same HxV gives the same bits
as before."""
import ctypes as C

import numpy as np
import pytest

from vmps_gb300 import _native as N
from vmps_gb300.pivot import PivotMatrix2

from helpers import pivot2_case

pytestmark = pytest.mark.gpu


def test_wait_timeout_is_reported_and_context_survives(gpu_ctx):
    model, mps, Lenv, Renv, W1, W2, V = pivot2_case("hubb", L=16, D=256, site=7, seed=22, profile="gaussian")
    H = PivotMatrix2(gpu_ctx, model.sym, Lenv, Renv, W1, W2, V)
    v = np.random.default_rng(8).standard_normal(V.data.size)
    good = H.apply(v, "bf16x3")
    good64 = H.apply(v, "fp64")
    lib = N.lib()
    try:
        assert lib.vmps_ctx_set_wait_budget(gpu_ctx._h, 1) == 0
        with pytest.raises(N.VmpsError) as exc:
            H.apply(v, "bf16x3")
        assert exc.value.code == -5, exc.value   # VMPS_E_TIMEOUT
        assert "wait" in str(exc.value)
    finally:
        assert lib.vmps_ctx_set_wait_budget(gpu_ctx._h, 0) == 0
    # the context still works, and the results are the same bits as before
    assert np.array_equal(H.apply(v, "bf16x3"), good)
    assert np.array_equal(H.apply(v, "fp64"), good64)
    assert lib.vmps_ctx_set_wait_budget(gpu_ctx._h, -1) == -1
    H.close()
