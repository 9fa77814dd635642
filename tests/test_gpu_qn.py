"""U(1) block-sparse (QN) tensors on the GPU against dense arithmetic: block-pair
contraction, the sector-wise truncated factorization (spectrum, bond dimension,
orthonormal U, discarded weight), and QN two-site DMRG against the dense chain driver
region by region on a model without degeneracies (XXZ with random longitudinal fields)."""
import numpy as np
import pytest

import oracle.linalg as ol
from networksolvers_gb300 import models as m
from networksolvers_gb300 import qn
from networksolvers_gb300.chain import dmrg_chain

pytestmark = pytest.mark.gpu


def _rand_block(rng, inds, flux, cplx):
    arr = np.zeros(tuple(q.dim for q in inds), dtype=np.complex128 if cplx else np.float64)
    for combo in qn.allowed_sectors(inds, flux):
        sl = tuple(slice(q.offsets[s], q.offsets[s] + q.sectors[s][1]) for q, s in zip(inds, combo))
        shape = arr[sl].shape
        arr[sl] = rng.standard_normal(shape) + (1j * rng.standard_normal(shape) if cplx else 0)
    return arr, qn.BlockTensor.from_dense(arr, inds, flux)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("cplx", [False, True])
def test_qcontract_matches_dense(nsg_ctx, cplx):
    rng = np.random.default_rng(5)
    i = qn.QNIndex([(-1, 2), (1, 3)], +1)
    j = qn.QNIndex([(-2, 1), (0, 2), (2, 2)], +1)
    k = qn.QNIndex([(-1, 3), (1, 2), (3, 1)], +1)
    l = qn.QNIndex([(0, 2), (2, 3)], +1)
    a_arr, A = _rand_block(rng, [i, j, k.dag()], 0, cplx)
    b_arr, B = _rand_block(rng, [k, l.dag()], -2, cplx)
    Cq = qn.qcontract(A, B)
    assert Cq.flux == -2 and [q.key() for q in Cq.inds] == [i.key(), j.key(), l.key()]
    assert rel(Cq.to_dense(), np.einsum("ijk,kl->ijl", a_arr, b_arr)) < 1e-13
    # two shared indices, one of them primed on both sides
    c_arr, Cc = _rand_block(rng, [j.dag(), k, i.prime()], 0, cplx)
    D = qn.qcontract(A, Cc)
    assert rel(D.to_dense(), np.einsum("ijk,jkp->ip", a_arr, c_arr)) < 1e-13


@pytest.mark.parametrize("cplx", [False, True])
def test_qfactorize_matches_dense_svd(nsg_ctx, cplx):
    rng = np.random.default_rng(9)
    a = qn.QNIndex([(-2, 3), (0, 5), (2, 4), (4, 2)], +1)
    s1 = qn.QNIndex([(-1, 1), (1, 1)], +1)
    s2 = qn.QNIndex([(-1, 1), (1, 1)], +1)
    b = qn.QNIndex([(-2, 4), (0, 6), (2, 3), (4, 2)], +1)
    t_arr, _ = _rand_block(rng, [a, s1, s2, b.dag()], 0, cplx)
    # spread the spectrum over decades (as a DMRG spectrum) by scaling the rows of each
    # sector of a: the block structure is untouched
    for sec, f in enumerate([1.0, 3e-2, 1e-3, 3e-5]):
        t_arr[a.offsets[sec]:a.offsets[sec] + a.sectors[sec][1]] *= f
    T = qn.BlockTensor.from_dense(t_arr, [a, s1, s2, b.dag()], 0)
    dense = T.to_dense().reshape(a.dim * 2, 2 * b.dim)
    s = np.linalg.svd(dense, compute_uv=False)
    # (cutoff 1e-14 keeps every non-zero singular value: the sectors hold
    # sum_q min(rows_q, cols_q) of them, the dense SVD pads with structural zeros)
    for cutoff, maxdim in [(1e-14, None), (1e-8, None), (1e-4, 9)]:
        U, Cm, info = qn.qfactorize(T, [a, s1], cutoff=cutoff, maxdim=maxdim)
        kref, errref = ol.truncate_spectrum(s ** 2, cutoff, maxdim)
        assert info["newdim"] == kref
        assert rel(info["spectrum"], (s ** 2)[:kref]) < 1e-12
        assert abs(info["truncerr"] - errref) <= 1e-12 * max(errref, 1e-16) + 1e-15
        ud = U.to_dense().reshape(a.dim * 2, kref)
        assert np.abs(ud.conj().T @ ud - np.eye(kref)).max() < 1e-12
        recon = qn.qcontract(U, Cm).to_dense().reshape(a.dim * 2, 2 * b.dim)
        assert abs(np.linalg.norm(dense - recon) ** 2 / np.linalg.norm(dense) ** 2 - errref) < 1e-12
        assert U.flux == 0 and Cm.flux == 0


def _xxz_fields(n, delta, seed):
    rng = np.random.default_rng(seed)
    os = m.OpSum()
    for j in range(1, n):
        os += (delta, "Sz", j, "Sz", j + 1)
        os += (0.5, "S+", j, "S-", j + 1)
        os += (0.5, "S-", j, "S+", j + 1)
    for j in range(1, n + 1):
        os += (float(rng.uniform(-0.5, 0.5)), "Sz", j)
    return m.chain_mpo(os, n)


def test_qn_dmrg_matches_dense_dmrg_region_by_region(nsg_ctx):
    """XXZ (Delta 1.5) with random longitudinal fields, N=12, from the Neel state:
    per-region energies within 1e-10 and identical bond dimensions, QN against dense."""
    n = 12
    H = _xxz_fields(n, 1.5, 4)
    g = m.chain_graph(n)
    neel = {v: ("Up" if v % 2 else "Dn") for v in g.vertices}
    psi0 = m.product_state(g, neel)
    kw = dict(maxdim=[8, 16, 32, 32], cutoff=1e-10, krylovdim=3, maxiter=1)
    Ed, _, rd = dmrg_chain(H, psi0, 4, **kw)
    Eq, A, rq = qn.qn_dmrg_chain(H, [0 if v % 2 else 1 for v in range(1, n + 1)], 4, **kw)
    rd, rq = np.array(rd, dtype=float), np.array(rq, dtype=float)
    assert np.array_equal(rd[:, 3], rq[:, 3])
    assert np.max(np.abs(rq[:, 2] - rd[:, 2]) / np.abs(rd[:, 2])) < 1e-10
    assert abs(Eq - Ed) / abs(Ed) < 1e-10
    # the state keeps the Neel state's total charge and is normalised
    assert all(t.flux == 0 for t in A)
