"""The allocation-free GEMM entry point (nsg_gemm_tf32x3_noalloc), through the C ABI.

It serves callers that must not allocate device memory themselves — for example a
Julia program whose CUDA.jl pool owns the GPU — by keeping its scratch in a static
device array.  Its results must equal those of the allocating entry point that runs the
same TF32x3 tensor-core GEMM (nsg_contract in the "tf32x3" precision mode), within the
2e-6 relative tolerance of the split-precision tests, on two calls in a row (the static
scratch is shared and keeps the previous call's contents).  This file is collected last
so a failure here leaves every other test already run; it also passes on its own in a
fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from networksolvers_gb300.itensors import DTensor, Index, contract

pytestmark = pytest.mark.gpu


def _dptr(t):
    p = C.c_void_p()
    t.ctx.check(t.ctx.L.nsg_tensor_device_ptr(t.st.h, C.byref(p)))
    return p


def _noalloc(ctx, A, transA, B, transB, Cout, m, n, k, alpha, beta):
    err = C.create_string_buffer(512)
    lda = A.shape[0]
    ldb = B.shape[0]
    ctx.synchronize()  # inputs were written on the context's stream
    rc = ctx.L.nsg_gemm_tf32x3_noalloc(_dptr(A), lda, int(transA), _dptr(B), ldb, int(transB), _dptr(Cout), m,
                                       m, n, k, alpha, beta, None, err, 512)
    assert rc == 0, err.value.decode()


def _reference(ctx, a, b):
    m, k = a.shape
    n = b.shape[1]
    i, l, j = Index(m), Index(k), Index(n)
    ctx.set_precision("tf32x3")
    try:
        return contract([DTensor.from_numpy(a, [i, l]), DTensor.from_numpy(b, [l, j])], out=[i, j]).to_numpy()
    finally:
        ctx.set_precision("fp64")


def test_noalloc_matches_allocating_entry_point_twice(nsg_ctx):
    rng = np.random.default_rng(42)
    # first call: plain orientation; second call: transposed operands, other sizes, beta != 0
    m, k, n = 384, 320, 256
    a, b = rng.standard_normal((m, k)), rng.standard_normal((k, n))
    ref1 = _reference(nsg_ctx, a, b)
    A, B = DTensor.from_numpy(a, [Index(m), Index(k)]), DTensor.from_numpy(b, [Index(k), Index(n)])
    Cd = DTensor.zeros([Index(m), Index(n)])
    _noalloc(nsg_ctx, A, False, B, False, Cd, m, n, k, 1.0, 0.0)
    c1 = Cd.to_numpy()
    assert np.linalg.norm(c1 - ref1) / np.linalg.norm(ref1) < 2e-6

    m2, k2, n2 = 200, 500, 130
    a2, b2 = rng.standard_normal((m2, k2)), rng.standard_normal((k2, n2))
    ref2 = _reference(nsg_ctx, a2, b2)
    c0 = rng.standard_normal((m2, n2))
    A2 = DTensor.from_numpy(a2.T.copy(), [Index(k2), Index(m2)])  # stored as A^T
    B2 = DTensor.from_numpy(b2.T.copy(), [Index(n2), Index(k2)])  # stored as B^T
    C2 = DTensor.from_numpy(c0, [Index(m2), Index(n2)])
    _noalloc(nsg_ctx, A2, True, B2, True, C2, m2, n2, k2, 2.0, -0.5)
    c2 = C2.to_numpy()
    want = 2.0 * ref2 - 0.5 * c0
    assert np.linalg.norm(c2 - want) / np.linalg.norm(want) < 2e-6


def test_noalloc_rejects_sizes_beyond_its_static_scratch(nsg_ctx):
    err = C.create_string_buffer(512)
    # 8192 x 8192 x 8192 would need 1 GiB of slices: rejected before any device work
    dummy = C.c_void_p(1)
    rc = nsg_ctx.L.nsg_gemm_tf32x3_noalloc(dummy, 8192, 0, dummy, 8192, 0, dummy, 8192, 8192, 8192, 8192, 1.0, 0.0,
                                           None, err, 512)
    assert rc == 7 and b"static" in err.value
