"""The phase profiler (tn_profile_enable / tn_profile_read) around real work, and the
context's workspace arena growing between profiled phases: the profiler's events are
independent of the arena, so growth (which drops the cached CUDA graphs) must leave them
usable, however often it happens."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_profiler_survives_repeated_workspace_growth():
    import tenetgb

    ctx = tenetgb.Context(0)
    rng = np.random.default_rng(3)

    def contract(n):
        a = tenetgb.DeviceTensor.from_numpy(ctx, rng.standard_normal((n, n)) + 0j, ["i", "k"])
        b = tenetgb.DeviceTensor.from_numpy(ctx, rng.standard_normal((n, n)) + 0j, ["k", "j"])
        return tenetgb.binary_einsum(a, b, out_inds=["j", "i"])  # permuted output: workspace

    ctx.profile(True)
    contract(64)
    first = ctx.profile_read()
    assert first["gemm_fp64"]["launches"] >= 1 and first["gemm_fp64"]["ms"] > 0
    ctx.profile(False)
    for n in (256, 512, 1024, 1536):  # each step needs a larger arena
        contract(n)
    ctx.sync()
    ctx.profile(True)
    c = contract(96)
    prof = ctx.profile_read()
    ctx.profile(False)
    assert prof["gemm_fp64"]["launches"] >= 1 and prof["gemm_fp64"]["ms"] > 0
    assert np.all(np.isfinite(c.numpy()))
