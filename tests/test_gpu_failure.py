"""Failure detection on the GPU without a fault: a bounded device wait that expires.

The split GEMM's pipeline waits (TMA, MMA, drain) are bounded by %globaltimer; on expiry a
kernel raises a timeout flag and returns, and the host turns the flag into JUES_ETIMEOUT.  The
test entry point runs the same bounded wait on a barrier phase that nothing completes, so the
wait runs out (after its ~2 s limit); the call must report JUES_ETIMEOUT and leave the context
usable.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_context_stays_usable():
    from juesgpu import _lib
    ctx = _lib.context(0)
    t0 = time.perf_counter()
    st = ctx.lib.jues_debug_expired_wait(ctx.h)
    dt = time.perf_counter() - t0
    assert st == _lib.ETIMEOUT
    assert "bounded device-side wait expired" in _lib.last_error()
    assert 1.5 < dt < 60.0
    # the flag was cleared and the context still computes
    rng = np.random.default_rng(0)
    A, B = rng.normal(size=(200, 300)), rng.normal(size=(300, 100))
    got = _lib.gemm(A, B, precision="split_bf16")
    assert np.linalg.norm(got - A @ B) < 1e-5 * np.linalg.norm(A @ B)
