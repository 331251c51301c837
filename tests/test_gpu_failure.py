"""Failure detection without a GPU fault: a bounded device-side wait that runs out.

The line adjoint's consumers wait on mbarriers for staged data; every wait has an iteration
limit, after which the kernel sets a mapped error word and returns.  Here a self-test kernel
waits on an mbarrier that nothing arrives on (a short limit), and the host must report
KORG_ETIMEOUT once, clear it, and keep the context usable for real work.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KORG_ETIMEOUT = 6


def test_bounded_wait_reports_timeout_and_context_stays_usable(gpu_lib):
    from korg_gb300 import synthetic
    from korg_gb300.api import synthesize_prepared
    ctx = gpu_lib.Context(0)
    ctx.ensure_stark()
    lib = ctx.lib
    assert lib.korg_device_status(ctx.h) == 0
    assert lib.korg_selftest_wait_timeout(ctx.h, 64) == KORG_ETIMEOUT
    assert b"ran past its limit" in lib.korg_last_error(ctx.h)
    assert lib.korg_device_status(ctx.h) == 0  # reported once, then cleared
    # the context still synthesises, and the result matches a fresh context's
    inp = synthetic.prepare(synthetic.config0(n_lines=300))
    r1 = synthesize_prepared(inp, precision="mixed", ctx=ctx)
    ctx2 = gpu_lib.Context(0)
    ctx2.ensure_stark()
    r2 = synthesize_prepared(inp, precision="mixed", ctx=ctx2)
    np.testing.assert_array_equal(r1.flux, r2.flux)
    assert lib.korg_device_status(ctx.h) == 0
    ctx2.close()
    ctx.close()
