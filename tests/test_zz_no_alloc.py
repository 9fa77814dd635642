"""The allocation-free GEMM entry point (nsg_gemm_tf32x3_noalloc), through the C ABI.

Some callers cannot let a library allocate device memory: a Julia program whose CUDA.jl
pool has reserved the GPU, a host whose caching allocator must account for every byte,
or a latency-bound loop that cannot absorb the synchronisation of cudaMalloc/cudaFree.
This entry point keeps its scratch in a static device array instead.  Checked here:

* its results are bitwise those of the allocating entry point that runs the same TF32x3
  tensor-core GEMM (nsg_contract in the "tf32x3" precision mode), on two calls in a row
  (the static scratch is shared and keeps the previous call's contents);
* both stay within the TF32x3 error bound of an FP64 product: |C - AB| <= 2^-20 |A||B|
  elementwise (split operands keep 21 mantissa bits; the dropped low x low product and
  the FP32 chunk sums are below that);
* a warmed-up call changes neither the device's free memory nor the high-water marks of
  the device's default stream-ordered pool (no allocation, transient or lasting, through
  either route);
* sizes beyond the static maximum are rejected before any device work.

This file is collected last so a failure here leaves every other test already run; it
also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from networksolvers_gb300.itensors import DTensor, Index, contract

pytestmark = pytest.mark.gpu

TF32X3_BOUND = 2.0 ** -20


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


def _allocating(ctx, a_stored, a_labels, b_stored, b_labels, out):
    """The allocating entry point (nsg_contract) in the TF32x3 mode."""
    ctx.set_precision("tf32x3")
    try:
        return contract([DTensor.from_numpy(a_stored, a_labels), DTensor.from_numpy(b_stored, b_labels)],
                        out=out).to_numpy()
    finally:
        ctx.set_precision("fp64")


def _within_tf32x3_bound(c, a, b):
    err = np.abs(c - a @ b)
    return bool(np.all(err <= TF32X3_BOUND * (np.abs(a) @ np.abs(b))))


class _DriverPool:
    """High-water marks of the device's default stream-ordered memory pool, read and
    reset through the CUDA driver API (the pool the library's contexts allocate from)."""
    RESERVED_MEM_HIGH, USED_MEM_HIGH = 6, 8

    def __init__(self, device=0):
        self.cu = C.CDLL("libcuda.so.1")
        assert self.cu.cuInit(0) == 0
        dev = C.c_int()
        assert self.cu.cuDeviceGet(C.byref(dev), device) == 0
        self.pool = C.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def reset(self):
        for attr in (self.RESERVED_MEM_HIGH, self.USED_MEM_HIGH):
            zero = C.c_uint64(0)  # setting a high-water mark to zero resets it to the current value
            assert self.cu.cuMemPoolSetAttribute(self.pool, attr, C.byref(zero)) == 0

    def highs(self):
        out = []
        for attr in (self.RESERVED_MEM_HIGH, self.USED_MEM_HIGH):
            v = C.c_uint64()
            assert self.cu.cuMemPoolGetAttribute(self.pool, attr, C.byref(v)) == 0
            out.append(v.value)
        return out


def test_noalloc_matches_allocating_entry_point_twice(nsg_ctx):
    from networksolvers_gb300._native import device_free_bytes
    rng = np.random.default_rng(42)
    # first call: plain orientation
    m, k, n = 384, 320, 256
    a, b = rng.standard_normal((m, k)), rng.standard_normal((k, n))
    i, l, j = Index(m), Index(k), Index(n)
    ref1 = _allocating(nsg_ctx, a, [i, l], b, [l, j], [i, j])
    A, B = DTensor.from_numpy(a, [Index(m), Index(k)]), DTensor.from_numpy(b, [Index(k), Index(n)])
    Cd = DTensor.zeros([Index(m), Index(n)])
    _noalloc(nsg_ctx, A, False, B, False, Cd, m, n, k, 1.0, 0.0)
    c1 = Cd.to_numpy()
    assert np.array_equal(c1, ref1)
    assert _within_tf32x3_bound(c1, a, b)

    # second call: transposed operands, other sizes, alpha and beta != 0
    m2, k2, n2 = 200, 500, 130
    a2, b2 = rng.standard_normal((m2, k2)), rng.standard_normal((k2, n2))
    i2, l2, j2 = Index(m2), Index(k2), Index(n2)
    ref2 = _allocating(nsg_ctx, a2.T.copy(), [l2, i2], b2.T.copy(), [j2, l2], [i2, j2])
    assert _within_tf32x3_bound(ref2, a2, b2)
    c0 = rng.standard_normal((m2, n2))
    A2 = DTensor.from_numpy(a2.T.copy(), [Index(k2), Index(m2)])  # stored as A^T
    B2 = DTensor.from_numpy(b2.T.copy(), [Index(n2), Index(k2)])  # stored as B^T
    C2 = DTensor.from_numpy(c0, [Index(m2), Index(n2)])
    _noalloc(nsg_ctx, A2, True, B2, True, C2, m2, n2, k2, 2.0, -0.5)
    c2 = C2.to_numpy()
    want = 2.0 * ref2 - 0.5 * c0
    assert np.max(np.abs(c2 - want)) <= 1e-15 * np.max(np.abs(want)) * 4
    assert _within_tf32x3_bound(c2 + 0.5 * c0, 2.0 * a2, b2)

    # a third, warmed-up call allocates nothing: the device's free memory and the default
    # pool's high-water marks are unchanged across it, and it repeats the first result
    Cd3 = DTensor.zeros([Index(m), Index(n)])
    nsg_ctx.synchronize()
    pool = _DriverPool(0)
    pool.reset()
    free_before, highs_before = device_free_bytes(0), pool.highs()
    _noalloc(nsg_ctx, A, False, B, False, Cd3, m, n, k, 1.0, 0.0)
    free_after, highs_after = device_free_bytes(0), pool.highs()
    assert free_after == free_before, (free_before, free_after)
    assert highs_after == highs_before, (highs_before, highs_after)
    assert np.array_equal(Cd3.to_numpy(), c1)


def test_noalloc_rejects_sizes_beyond_its_static_scratch(nsg_ctx):
    err = C.create_string_buffer(512)
    # 8192 x 8192 x 8192 would need 1 GiB of slices: rejected before any device work
    dummy = C.c_void_p(1)
    rc = nsg_ctx.L.nsg_gemm_tf32x3_noalloc(dummy, 8192, 0, dummy, 8192, 0, dummy, 8192, 8192, 8192, 8192, 1.0, 0.0,
                                           None, err, 512)
    assert rc == 7 and b"static" in err.value
    # extents whose padded product would wrap 64 bits are rejected by the extent bound
    big = 1 << 40
    rc = nsg_ctx.L.nsg_gemm_tf32x3_noalloc(dummy, big, 0, dummy, big, 0, dummy, big, big, big, big, 1.0, 0.0,
                                           None, err, 512)
    assert rc == 7 and b"extent" in err.value
