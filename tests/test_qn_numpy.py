"""The QN layer's block bookkeeping (networksolvers_gb300/qn.py, unchanged) run on the
CPU with numpy stand-ins for its device calls (tests/_qn_numpy.py): block-pair
contraction and the sector-wise factorization against dense numpy, and QN two-site DMRG
against the dense oracle DMRG region by region.  No GPU."""
import numpy as np
import pytest

import oracle.linalg as ol
from oracle import sweep as osw
from networksolvers_gb300 import models as m
from networksolvers_gb300 import qn

from _qn_numpy import numpy_backend


def _rand_block(rng, inds, flux, cplx, ctx):
    arr = np.zeros(tuple(q.dim for q in inds), dtype=np.complex128 if cplx else np.float64)
    for combo in qn.allowed_sectors(inds, flux):
        sl = tuple(slice(q.offsets[s], q.offsets[s] + q.sectors[s][1]) for q, s in zip(inds, combo))
        shape = arr[sl].shape
        arr[sl] = rng.standard_normal(shape) + (1j * rng.standard_normal(shape) if cplx else 0)
    return arr, qn.BlockTensor.from_dense(arr, inds, flux, ctx=ctx)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("cplx", [False, True])
def test_block_contraction_and_factorization(cplx):
    with numpy_backend() as ctx:
        rng = np.random.default_rng(5)
        i = qn.QNIndex([(-1, 2), (1, 3)], +1)
        j = qn.QNIndex([(-2, 1), (0, 2), (2, 2)], +1)
        k = qn.QNIndex([(-1, 3), (1, 2), (3, 1)], +1)
        l = qn.QNIndex([(0, 2), (2, 3)], +1)
        a_arr, A = _rand_block(rng, [i, j, k.dag()], 0, cplx, ctx)
        b_arr, B = _rand_block(rng, [k, l.dag()], -2, cplx, ctx)
        assert rel(qn.qcontract(A, B).to_dense(), np.einsum("ijk,kl->ijl", a_arr, b_arr)) < 1e-13
        a = qn.QNIndex([(-2, 3), (0, 5), (2, 4), (4, 2)], +1)
        s1 = qn.QNIndex([(-1, 1), (1, 1)], +1)
        s2 = qn.QNIndex([(-1, 1), (1, 1)], +1)
        b = qn.QNIndex([(-2, 4), (0, 6), (2, 3), (4, 2)], +1)
        t_arr, _ = _rand_block(rng, [a, s1, s2, b.dag()], 0, cplx, ctx)
        for sec, f in enumerate([1.0, 3e-2, 1e-3, 3e-5]):
            t_arr[a.offsets[sec]:a.offsets[sec] + a.sectors[sec][1]] *= f
        T = qn.BlockTensor.from_dense(t_arr, [a, s1, s2, b.dag()], 0, ctx=ctx)
        dense = t_arr.reshape(a.dim * 2, 2 * b.dim)
        s = np.linalg.svd(dense, compute_uv=False)
        for cutoff, maxdim in [(1e-14, None), (1e-8, None), (1e-4, 9)]:
            U, Cm, info = qn.qfactorize(T, [a, s1], cutoff=cutoff, maxdim=maxdim)
            kref, errref = ol.truncate_spectrum(s ** 2, cutoff, maxdim)
            assert info["newdim"] == kref and rel(info["spectrum"], (s ** 2)[:kref]) < 1e-12
            ud = U.to_dense().reshape(a.dim * 2, kref)
            assert np.abs(ud.conj().T @ ud - np.eye(kref)).max() < 1e-12
            recon = qn.qcontract(U, Cm).to_dense().reshape(a.dim * 2, 2 * b.dim)
            assert abs(np.linalg.norm(dense - recon) ** 2 / np.linalg.norm(dense) ** 2 - errref) < 1e-12


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


def test_qn_dmrg_matches_the_dense_oracle():
    """XXZ (Delta 1.5) with random longitudinal fields, N=10, from the Neel state, maxdim
    [8, 16, 32], cutoff 1e-10: per-region energies 1e-10 and identical bond dimensions."""
    n = 10
    H = _xxz_fields(n, 1.5, 2)
    g = m.chain_graph(n)
    psi0 = m.product_state(g, {v: ("Up" if v % 2 else "Dn") for v in g.vertices})
    trunc = dict(cutoff=1e-10, maxdim=[8, 16, 32])
    ref = []
    Eo, _ = osw.dmrg(H, psi0, 3, nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
                     inserter_kwargs=dict(trunc=trunc),
                     region_callback=lambda prob, sweep, region, which, **k: ref.append(
                         (prob.eigenvalue, prob.last_insert.get("newdim", -1))))
    with numpy_backend() as ctx:
        Eq, A, rq = qn.qn_dmrg_chain(H, [0 if v % 2 else 1 for v in range(1, n + 1)], 3, maxdim=trunc["maxdim"],
                                     cutoff=1e-10, ctx=ctx)
    ref = np.array(ref, dtype=float)
    got = np.array([(r[2], r[3]) for r in rq], dtype=float)
    assert np.array_equal(got[:, 1], ref[:, 1])
    assert np.max(np.abs(got[:, 0] - ref[:, 0]) / np.abs(ref[:, 0])) < 1e-10
    assert abs(Eq - Eo) / abs(Eo) < 1e-10
