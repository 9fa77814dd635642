"""The timeout path of the library's bounded device waits, driven to expiry on the GPU.

Every spin-wait in the kernels (mbarrier waits of the tensor-core GEMMs, the grid
barrier of the tridiagonalisation) gives up after a bounded number of polls, raises the
context's device error flag and returns; the public call then reports NSG_ERR_TIMEOUT.
nsg_ctx_wait_probe runs that pattern on a device flag that nothing sets, with a short
limit, so the give-up path runs for real.  No fault, trap or endless loop is involved.
"""
import time

import numpy as np
import pytest

from networksolvers_gb300 import _native

pytestmark = pytest.mark.gpu


def test_wait_runs_out_and_returns_timeout(nsg_ctx):
    t0 = time.perf_counter()
    rc = nsg_ctx.L.nsg_ctx_wait_probe(nsg_ctx.h, 20000)
    dt = time.perf_counter() - t0
    assert rc == _native.ERR_TIMEOUT, rc
    assert b"timed out" in nsg_ctx.L.nsg_last_error(nsg_ctx.h)
    assert dt < 5.0
    # the flag was cleared when it was reported: the context keeps working
    nsg_ctx.synchronize()
    from networksolvers_gb300.itensors import DTensor, Index
    x = np.arange(12.0).reshape(3, 4)
    t = DTensor.from_numpy(x, [Index(3), Index(4)])
    assert np.array_equal(t.to_numpy(), x)
    assert abs(t.norm() - np.linalg.norm(x)) < 1e-12 * np.linalg.norm(x)


def test_wait_probe_rejects_unbounded_limits(nsg_ctx):
    assert nsg_ctx.L.nsg_ctx_wait_probe(nsg_ctx.h, 0) == _native.ERR_INVALID
    assert nsg_ctx.L.nsg_ctx_wait_probe(nsg_ctx.h, 1 << 30) == _native.ERR_INVALID
