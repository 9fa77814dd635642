"""Split-precision (TF32x3, FP32 accumulate) GEMMs on the tcgen05 tensor cores, checked
against the FP64 path on the same inputs.  Tolerance: 2e-6 relative (Frobenius) —
the error of FP32 accumulation over K up to a few thousand."""
import numpy as np
import pytest

from networksolvers_gb300.itensors import DTensor, Index, contract

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("m,k,n", [(128, 32, 128), (256, 256, 128), (200, 100, 300), (1024, 1024, 1024),
                                   (130, 4000, 70), (5120, 1024, 4096)])
def test_tf32x3_gemm_orientations(nsg_ctx, m, k, n):
    rng = np.random.default_rng(m + k + n)
    i, j, l = Index(m), Index(n), Index(k)
    a = rng.standard_normal((m, k))
    b = rng.standard_normal((k, n))
    ref = a @ b
    for (ia, aa), (ib, bb) in [(((i, l), a), ((l, j), b)), (((l, i), a.T.copy()), ((l, j), b)),
                               (((i, l), a), ((j, l), b.T.copy())), (((l, i), a.T.copy()), ((j, l), b.T.copy()))]:
        A, B = DTensor.from_numpy(aa, ia), DTensor.from_numpy(bb, ib)
        nsg_ctx.set_precision("tf32x3")
        try:
            c = contract([A, B], out=[i, j]).to_numpy()
        finally:
            nsg_ctx.set_precision("fp64")
        assert rel(c, ref) < 2e-6, (ia, ib)


def test_tf32x3_path_is_the_one_that_ran(nsg_ctx):
    """The tensor-core path runs (two split passes + one tcgen05 GEMM launch)."""
    rng = np.random.default_rng(5)
    m, k, n = 256, 192, 160
    i, l, j = Index(m), Index(k), Index(n)
    a, b = rng.standard_normal((m, k)), rng.standard_normal((k, n))
    A, B = DTensor.from_numpy(a, [i, l]), DTensor.from_numpy(b, [l, j])
    nsg_ctx.set_precision("tf32x3")
    try:
        before = nsg_ctx.counters()["launches"]
        c = contract([A, B], out=[i, j]).to_numpy()
        after = nsg_ctx.counters()["launches"]
    finally:
        nsg_ctx.set_precision("fp64")
    assert rel(c, a @ b) < 2e-6
    assert after - before == 3


@pytest.mark.parametrize("m,k,n", [(128, 64, 64), (200, 100, 300), (1024, 1024, 1024), (130, 4000, 70),
                                   (5120, 1024, 4096)])
def test_ozaki_gemm_fp64_level(nsg_ctx, m, k, n):
    """Six 7-bit BF16 slices per operand, exact FP32 chunk accumulation: FP64-level
    products (1e-12 relative) in every operand orientation, including rows with a wide
    dynamic range (one large entry per row, as the environment blocks carry)."""
    rng = np.random.default_rng(m * 3 + k + n)
    i, j, l = Index(m), Index(n), Index(k)
    a = rng.standard_normal((m, k))
    a[:, 0] *= 1e4
    b = rng.standard_normal((k, n))
    ref = a @ b
    for (ia, aa), (ib, bb) in [(((i, l), a), ((l, j), b)), (((l, i), a.T.copy()), ((l, j), b)),
                               (((i, l), a), ((j, l), b.T.copy())), (((l, i), a.T.copy()), ((j, l), b.T.copy()))]:
        A, B = DTensor.from_numpy(aa, ia), DTensor.from_numpy(bb, ib)
        nsg_ctx.set_precision("ozaki")
        try:
            c = contract([A, B], out=[i, j]).to_numpy()
        finally:
            nsg_ctx.set_precision("fp64")
        scale = np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :] * k
        # the method's bound is relative to the row/column scales (one wide row here)
        assert np.max(np.abs(c - ref) / scale) < 1e-13, (ia, ib)
        assert rel(c, ref) < 5e-11


@pytest.mark.parametrize("m,k,n", [(200, 100, 300), (1024, 1024, 1024), (130, 4000, 70)])
def test_ozaki8_gemm_fp64_accuracy(nsg_ctx, m, k, n):
    """Eight slices (36 products): slicing error 2^-57 of the row and column scales per
    product; the double-float (2 x FP32) chunk accumulation sets the floor near 1e-15 of
    the scales, with one wide-range column as in the environments."""
    rng = np.random.default_rng(m + 5 * k + n)
    i, j, l = Index(m), Index(n), Index(k)
    a = rng.standard_normal((m, k))
    a[:, 0] *= 1e4
    b = rng.standard_normal((k, n))
    ref = a @ b
    A, B = DTensor.from_numpy(a, (i, l)), DTensor.from_numpy(b, (l, j))
    nsg_ctx.set_precision("ozaki8")
    try:
        c = contract([A, B], out=[i, j]).to_numpy()
    finally:
        nsg_ctx.set_precision("fp64")
    scale = np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :] * k
    assert np.max(np.abs(c - ref) / scale) < 1e-15
    assert rel(c, ref) < 1e-13


@pytest.mark.parametrize("precision,bound", [("ozaki", 1e-13), ("ozaki8", 1e-15)])
def test_complex_ozaki_gemm(nsg_ctx, precision, bound):
    """The split form for complex tensors: four real slice products on the interleaved
    real and imaginary parts (Re C = Ar Br - sa sb Ai Bi, Im C = sb Ar Bi + sa Ai Br, the
    signs from conjugated operands), in every operand orientation and with conjugation;
    within the real products' bound relative to the row and column scales, and on the
    tensor cores (the tcgen05 class launches)."""
    rng = np.random.default_rng(11)
    m, k, n = 200, 130, 96
    i, j, l = Index(m), Index(n), Index(k)
    a = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
    b = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
    a[:, 0] *= 1e3
    scale = np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :] * k
    cases = [(((i, l), a), ((l, j), b), False, False), (((l, i), a.T.copy()), ((l, j), b), False, False),
             (((i, l), a), ((j, l), b.T.copy()), False, False), (((i, l), a), ((l, j), b), True, False),
             (((l, i), a.T.copy()), ((j, l), b.T.copy()), True, True)]
    for (ia, aa), (ib, bb), ca, cb in cases:
        A, B = DTensor.from_numpy(aa, ia), DTensor.from_numpy(bb, ib)
        A = A.dag() if ca else A
        B = B.dag() if cb else B
        ref = (np.conj(a) if ca else a) @ (np.conj(b) if cb else b)
        nsg_ctx.set_precision(precision)
        nsg_ctx.profile(True)
        try:
            c = contract([A, B], out=[i, j]).to_numpy()
            prof = nsg_ctx.profile_read()
        finally:
            nsg_ctx.profile(False)
            nsg_ctx.set_precision("fp64")
        assert prof["tc_gemm"]["launches"] == 4, prof
        assert np.max(np.abs(c - ref) / scale) < bound, (ia, ib, ca, cb)


@pytest.mark.parametrize("precision,bound", [("ozaki", 1e-13), ("ozaki8", 1e-15)])
@pytest.mark.parametrize("m,k,n", [(100, 3000, 70), (300, 1000, 200)])
def test_ozaki_split_k_small_outputs(nsg_ctx, precision, bound, m, k, n):
    """Products whose 128 x 64 output tiles would leave most SMs idle split K over whole
    exact chunks (up to 16 splits; the partial products added in order, then alpha and
    beta): the same bound relative to the row and column scales as one pass over K."""
    rng = np.random.default_rng(m + k + n)
    i, j, l = Index(m), Index(n), Index(k)
    a = rng.standard_normal((m, k))
    a[:, 1] *= 1e4
    b = rng.standard_normal((k, n))
    ref = a @ b
    A, B = DTensor.from_numpy(a, (i, l)), DTensor.from_numpy(b, (l, j))
    nsg_ctx.set_precision(precision)
    try:
        before = nsg_ctx.counters()["launches"]
        c = contract([A, B], out=[i, j]).to_numpy()
        launches = nsg_ctx.counters()["launches"] - before
    finally:
        nsg_ctx.set_precision("fp64")
    scale = np.abs(a).max(axis=1)[:, None] * np.abs(b).max(axis=0)[None, :] * k
    assert np.max(np.abs(c - ref) / scale) < bound
    assert launches >= 6  # two operands sliced (2 launches each), the product and its split reduction
