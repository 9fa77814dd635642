"""Per-context launch-choice overrides (nsg_ctx_set_tuning), which the autotuner uses:
invalid values are rejected, and every tridiagonalisation path, divide-and-conquer leaf
order and split-K count gives the same results (eigenvalues 1e-12, products 1e-13
relative)."""
import numpy as np
import pytest

from networksolvers_gb300 import _native
from networksolvers_gb300.itensors import DTensor, Index, contract, factorize

pytestmark = pytest.mark.gpu


def test_set_tuning_rejects_invalid_values(nsg_ctx):
    L = nsg_ctx.L
    assert L.nsg_ctx_set_tuning(nsg_ctx.h, 0, 65) == _native.ERR_INVALID
    assert L.nsg_ctx_set_tuning(nsg_ctx.h, 1, 3) == _native.ERR_INVALID
    assert L.nsg_ctx_set_tuning(nsg_ctx.h, 2, 3) == _native.ERR_INVALID
    assert L.nsg_ctx_set_tuning(nsg_ctx.h, 2, 33) == _native.ERR_INVALID
    assert L.nsg_ctx_set_tuning(nsg_ctx.h, 7, 0) == _native.ERR_INVALID


@pytest.mark.parametrize("n", [40, 150, 300])
def test_tridiag_paths_agree(nsg_ctx, n):
    rng = np.random.default_rng(n)
    M = rng.standard_normal((n, n))
    ref = np.linalg.svd(M, compute_uv=False) ** 2
    l, r = Index(n), Index(n)
    T = DTensor.from_numpy(M, [l, r])
    try:
        for path in (-1, 2, 4, 8, 16):
            nsg_ctx.set_tuning("tridiag", path)
            U, C, info = factorize(T, [l], cutoff=0.0, maxdim=n, spectrum=True)
            assert np.max(np.abs(info["spectrum"][:n] - ref)) < 1e-12 * ref[0], path
            u, c = U.to_numpy(), C.to_numpy()
            assert np.linalg.norm(u @ c - M) < 1e-11 * np.linalg.norm(M), path
    finally:
        nsg_ctx.set_tuning("tridiag", 0)


@pytest.mark.parametrize("n", [64, 300])
def test_dc_leaf_orders_agree(nsg_ctx, n):
    rng = np.random.default_rng(n + 1)
    M = rng.standard_normal((n, n))
    ref = np.linalg.svd(M, compute_uv=False) ** 2
    l, r = Index(n), Index(n)
    T = DTensor.from_numpy(M, [l, r])
    try:
        for leaf in (4, 16, 32, 0):
            nsg_ctx.set_tuning("dc_leaf", leaf)
            U, C, info = factorize(T, [l], cutoff=0.0, maxdim=n, spectrum=True)
            assert np.max(np.abs(info["spectrum"][:n] - ref)) < 1e-12 * ref[0], leaf
            u, c = U.to_numpy(), C.to_numpy()
            assert np.linalg.norm(u @ c - M) < 1e-11 * np.linalg.norm(M), leaf
    finally:
        nsg_ctx.set_tuning("dc_leaf", 0)


def test_splitk_counts_agree(nsg_ctx):
    rng = np.random.default_rng(1)
    m, k = 64, 1024
    a, b = rng.standard_normal((m, k)), rng.standard_normal((k, m))
    i, j, l = Index(m), Index(m), Index(k)
    A, B = DTensor.from_numpy(a, [i, l]), DTensor.from_numpy(b, [l, j])
    ref = a @ b
    try:
        for sp in (0, 1, 2, 8, 64):
            nsg_ctx.set_tuning("splitk", sp)
            c = contract([A, B], out=[i, j]).to_numpy()
            assert np.linalg.norm(c - ref) < 1e-13 * np.linalg.norm(ref), sp
    finally:
        nsg_ctx.set_tuning("splitk", 0)
