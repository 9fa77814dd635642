"""Kernel-level parity on the GPU, through the C ABI (libnsg.so via ctypes):
contractions (every GEMM orientation, batched forms, conjugation, permutes),
truncated factorisation, QR, Hermitian eigen, Lanczos, Krylov exponential and RK4,
each against numpy / the oracle on the same seeded inputs.
Tolerances: FP64 contractions 1e-12 relative; eigenvalues 1e-12 relative;
truncated bond dimensions exact."""
import numpy as np
import pytest

from networksolvers_gb300 import itensors as it
from networksolvers_gb300.itensors import DTensor, Index, contract
from oracle import krylov as ok, linalg as ol

pytestmark = pytest.mark.gpu


def rnd(rng, shape, cplx=False):
    a = rng.standard_normal(shape)
    if cplx:
        a = a + 1j * rng.standard_normal(shape)
    return a


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("cplx", [False, True])
def test_contract_layouts(nsg_ctx, cplx):
    rng = np.random.default_rng(1)
    i, j, k, l, m_ = (Index(d) for d in (7, 5, 6, 4, 3))
    cases = [
        ((i, k), (k, j)),          # N N
        ((k, i), (k, j)),          # T N
        ((i, k), (j, k)),          # N T
        ((k, i), (j, k)),          # T T
        ((i, k, l), (k, j)),       # A batched over l
        ((i, k, l), (j, k)),
        ((i, j), (m_, k, j, l)),   # B batched
        ((k, l, i), (l, j, k)),    # K order mismatch -> permute
        ((i, k, j, l), (l, k)),    # K interleaved -> permute
        ((i,), (i, j)),            # vector
    ]
    for ia, ib in cases:
        a = rnd(rng, [x.dim for x in ia], cplx)
        b = rnd(rng, [x.dim for x in ib], cplx)
        for conj_a in (False, True):
            A = DTensor.from_numpy(a, ia)
            B = DTensor.from_numpy(b, ib)
            if conj_a:
                A = A.dag()
            Cd = A * B
            aa = np.conj(a) if (conj_a and cplx) else a
            lab = {}
            for x in list(ia) + list(ib):
                lab.setdefault(x, len(lab))
            ref = np.einsum(aa, [lab[x] for x in ia], b, [lab[x] for x in ib], [lab[x] for x in Cd.inds])
            assert rel(Cd.to_numpy(), ref) < 1e-12, (ia, ib, conj_a)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("conj", [False, True])
def test_site_operator_step(nsg_ctx, cplx, conj):
    """The H_eff middle step: T[a', w1, s1, s2, b] . W[w1, s1, s2, x] over (w1, s1, s2),
    a batched tall-skinny product (N, K <= 32) run by the one-row-per-thread kernel,
    with and without conjugated operands."""
    rng = np.random.default_rng(5)
    a, w1, s1, s2, b, x = (Index(d) for d in (300, 5, 2, 2, 70, 20))
    T = rnd(rng, (300, 5, 2, 2, 70), cplx)
    W = rnd(rng, (5, 2, 2, 20), cplx)
    At = DTensor.from_numpy(T, [a, w1, s1, s2, b])
    Wt = DTensor.from_numpy(W, [w1, s1, s2, x])
    if conj:
        At, T = At.dag(), T.conj()
    got = contract([At, Wt], out=[a, x, b]).to_numpy()
    ref = np.einsum("awstb,wstx->axb", T, W)
    assert rel(got, ref) < 1e-13


def test_contract_network_and_output_order(nsg_ctx):
    rng = np.random.default_rng(2)
    chi, w, d = 9, 5, 2
    a, ap, b, bp = Index(chi), Index(chi), Index(chi), Index(chi)
    w1, w2, w3 = Index(w), Index(w), Index(w)
    s1, s2 = Index(d), Index(d)
    L = rnd(rng, (chi, w, chi)); R = rnd(rng, (chi, w, chi))
    W1 = rnd(rng, (w, d, d, w)); W2 = rnd(rng, (w, d, d, w)); x = rnd(rng, (chi, d, d, chi))
    t = [DTensor.from_numpy(L, [ap, w1, a]), DTensor.from_numpy(W1, [w1, s1.prime(), s1, w2]),
         DTensor.from_numpy(W2, [w2, s2.prime(), s2, w3]), DTensor.from_numpy(R, [bp, w3, b]),
         DTensor.from_numpy(x, [a, s1, s2, b])]
    out = [ap, s1.prime(), s2.prime(), bp]
    y = contract(t, out=out).to_numpy()
    ref = np.einsum("pwa,wtsv,vuxz,qzb,asxb->ptuq", L, W1, W2, R, x)
    assert rel(y, ref) < 1e-12


@pytest.mark.parametrize("perm", [(1, 0, 2), (2, 0, 1), (0, 2, 1, 3), (3, 1, 0, 2), (1, 2, 0, 3)])
def test_permute(nsg_ctx, perm):
    rng = np.random.default_rng(3)
    shape = [5, 33, 7, 40][: len(perm)]
    a = rnd(rng, shape, True)
    inds = [Index(s) for s in shape]
    T = DTensor.from_numpy(a, inds)
    P = T.permute([inds[p] for p in perm])
    assert np.array_equal(P.to_numpy(), np.transpose(a, perm))
    Pc = T.dag().permute([inds[p] for p in perm])
    assert np.array_equal(Pc.to_numpy(), np.conj(np.transpose(a, perm)))


def _spectrum_matrix(rng, m, n, decay, cplx):
    k = min(m, n)
    U, _ = np.linalg.qr(rnd(rng, (m, k), cplx))
    V, _ = np.linalg.qr(rnd(rng, (n, k), cplx))
    s = decay ** np.arange(k)
    return (U * s) @ V.conj().T


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("m,n", [(16, 16), (24, 10), (10, 24), (128, 128), (200, 24), (300, 20)])
def test_factorize_truncation(nsg_ctx, cplx, m, n):
    """Singular values 0.55^i.  The tall shapes take the tall route (Gram matrix of the
    narrow side, re-orthogonalised U) whenever the kept spectrum is resolved well above
    the Gram matrix's rounding, the M M^H route otherwise."""
    rng = np.random.default_rng(m * 100 + n)
    M = _spectrum_matrix(rng, m, n, 0.55, cplx)
    l, r = Index(m), Index(n)
    T = DTensor.from_numpy(M, [l, r])
    for cutoff, maxdim in [(0.0, None), (1e-10, None), (1e-6, 8), (1e-3, None)]:
        U, Cc, info = it.factorize(T, [l], cutoff=cutoff, maxdim=maxdim, spectrum=True)
        s = np.linalg.svd(M, compute_uv=False)
        kref, errref = ol.truncate_spectrum(s ** 2, cutoff, maxdim)
        assert info["newdim"] == kref
        # the Gram route fixes each discarded sigma^2 to ~1e-15 of ||M||^2 (absolute)
        assert abs(info["truncerr"] - errref) <= 1e-6 * errref + 1e-14
        u = U.to_numpy()
        c = Cc.to_numpy()
        assert np.allclose(u.conj().T @ u, np.eye(kref), atol=1e-12)
        Pk = u @ c
        s2 = s[:kref]
        assert rel(np.linalg.svd(Pk, compute_uv=False)[:kref], s2) < 1e-10
        assert abs(np.linalg.norm(M - Pk) ** 2 / np.linalg.norm(M) ** 2 - errref) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("m,n,decay", [(600, 200, 0.88), (1500, 700, 0.965), (400, 100, 0.7)])
def test_factorize_tall_unresolved_tail(nsg_ctx, cplx, m, n, decay, precision):
    """Tall M whose kept spectrum reaches below what U = M V S^-1 resolves (kept sigma^2
    down to ~1e-13 of the largest, 3 to 49 such columns): orthonormal U, exact bond
    dimension (or one either side at a cutoff tie: the Gram matrix fixes partial sums of
    the spectrum to ~eps sqrt(n) of the largest weight), discarded weight and
    reconstruction.  Cutoffs far below that resolution (1e-15) leave the kept count itself
    undetermined for any Gram-based factorization and are not used."""
    rng = np.random.default_rng(m + n)
    M = _spectrum_matrix(rng, m, n, decay, cplx)
    l, r = Index(m), Index(n)
    T = DTensor.from_numpy(M, [l, r])
    s = np.linalg.svd(M, compute_uv=False)
    for cutoff, maxdim in [(1e-12, None), (1e-13, n // 2), (3e-13, None)]:
        nsg_ctx.set_precision(precision)
        try:
            U, Cc, info = it.factorize(T, [l], cutoff=cutoff, maxdim=maxdim, spectrum=True)
        finally:
            nsg_ctx.set_precision("fp64")
        kref, errref = ol.truncate_spectrum(s ** 2, cutoff, maxdim)
        if info["newdim"] != kref and _cutoff_tie(s ** 2, kref, cutoff, resolution=5e-14):
            assert abs(info["newdim"] - kref) == 1
            kref = info["newdim"]
            errref = float((s ** 2)[kref:].sum() / (s ** 2).sum())
        assert info["newdim"] == kref, (cutoff, maxdim)
        u = U.to_numpy().reshape(m, -1)
        assert np.abs(u.conj().T @ u - np.eye(kref)).max() < 1e-12
        Pk = u @ Cc.to_numpy().reshape(kref, n)
        assert abs(np.linalg.norm(M - Pk) ** 2 / np.linalg.norm(M) ** 2 - errref) < 1e-13
        # a Gram matrix carries ~eps sqrt(n) sigma_max^2 of rounding, so a Gram-based
        # factorization (either side, this library's or numpy's own) resolves kept singular
        # values only to ~sqrt(eps sqrt(n)) sigma_max absolute; the part well above that is
        # checked relatively
        sp = np.linalg.svd(Pk, compute_uv=False)[:kref]
        assert np.abs(sp - s[:kref]).max() < 4 * np.sqrt(np.finfo(float).eps * np.sqrt(n)) * s[0]
        res = s[:kref] ** 2 > 1e-11 * s[0] ** 2
        assert rel(sp[res], s[:kref][res]) < 1e-10


def test_factorize_tensor_axes(nsg_ctx):
    rng = np.random.default_rng(5)
    a, s1, s2, b = Index(6), Index(2), Index(2), Index(5)
    x = rnd(rng, (6, 2, 2, 5))
    T = DTensor.from_numpy(x, [a, s1, s2, b])
    U, Cc, info = it.factorize(T, [s1, a], cutoff=0.0)
    recon = contract([U, Cc], out=[a, s1, s2, b]).to_numpy()
    assert rel(recon, x) < 1e-12
    Q, R = it.qr(T, [a, s1])
    assert Q.inds[-1].dim == 10
    assert rel(contract([Q, R], out=[a, s1, s2, b]).to_numpy(), x) < 1e-12


@pytest.mark.parametrize("cplx", [False, True])
def test_eigh_truncated(nsg_ctx, cplx):
    rng = np.random.default_rng(6)
    a0, s = Index(7), Index(2)
    S = rnd(rng, (14, 9), cplx)
    rho = (S @ S.conj().T).reshape(7, 2, 7, 2)
    T = DTensor.from_numpy(rho, [a0.prime(), s.prime(), a0, s])
    D, U, u = it.eigen_hermitian(T, [a0, s], cutoff=1e-8, maxdim=5)
    w = np.sort(np.linalg.eigvalsh(S @ S.conj().T))[::-1]
    kref, _ = ol.truncate_spectrum(w, 1e-8, 5)
    assert len(D) == kref and rel(D, w[:kref]) < 1e-12
    Um = U.to_numpy().reshape(14, kref)
    M = S @ S.conj().T
    assert rel(M @ Um, Um * D) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("cplx", [False, True])
def test_factorize_complement_and_reduced_expansion(nsg_ctx, cplx, precision):
    """nsg_factorize_complement: Uperp [left..., rows - k] orthonormal and orthogonal to U,
    U and C as nsg_factorize gives them, none from the narrow-side route; and the
    densitymatrix eigenproblem solved in Uperp (R = Y Y^H, Y = Uperp^H sqrt_rho) gives the
    eigenvalues and the eigenvector subspace of the full rho = X X^H, X = (1 - U U^H) sqrt_rho."""
    rng = np.random.default_rng(21)
    a, s, b = Index(40), Index(2), Index(96)
    M = _dmrg_like(rng, 80, 96, cplx).reshape(40, 2, 96)
    T = DTensor.from_numpy(M, [a, s, b])
    nsg_ctx.set_precision(precision)
    try:
        U, Cc, info = it.factorize(T, [a, s], cutoff=1e-10, maxdim=50, complement=True)
        U0, C0, info0 = it.factorize(T, [a, s], cutoff=1e-10, maxdim=50)
        perp = info["complement"]
        k = info["newdim"]
        assert perp is not None and list(perp.inds[:2]) == [a, s] and perp.inds[2].dim == 80 - k
        u, q = U.to_numpy().reshape(80, k), perp.to_numpy().reshape(80, 80 - k)
        assert np.abs(q.conj().T @ q - np.eye(80 - k)).max() < 1e-12
        assert np.abs(u.conj().T @ q).max() < 1e-12
        assert info0["newdim"] == k and rel(u, U0.to_numpy().reshape(80, k)) < 1e-12
        assert rel(Cc.to_numpy(), C0.to_numpy()) < 1e-12
        # reduced expansion against the full one
        w_, o = Index(3), Index(30)
        S = rnd(rng, (40, 2, 3, 30), cplx)
        sq = DTensor.from_numpy(S, [a.prime(), s.prime(), w_, o])
        Y = perp.prime().dag() * sq
        R = Y * Y.noprime().dag()
        D, Z, _ = it.eigen_hermitian(R, [perp.inds[2]], cutoff=1e-14, maxdim=20)
        Ue = (perp * Z).to_numpy().reshape(80, -1)
        X = S.reshape(80, 90)
        X = X - u @ (u.conj().T @ X)
        wf, Vf = np.linalg.eigh(X @ X.conj().T)
        wf, Vf = wf[::-1][: len(D)], Vf[:, ::-1][:, : len(D)]
        assert rel(np.array(D), wf) < 1e-12
        # same subspace: the projector difference
        assert np.abs(Ue @ Ue.conj().T - Vf @ Vf.conj().T).max() < 1e-10
        # the narrow-side route (tall M, cutoff > 0) returns no complement
        Mt = _dmrg_like(rng, 200, 40, cplx)
        lt, rt = Index(200), Index(40)
        _, _, it_info = it.factorize(DTensor.from_numpy(Mt, [lt, rt]), [lt], cutoff=1e-12, complement=True)
        assert it_info["complement"] is None
    finally:
        nsg_ctx.set_precision("fp64")


def _chain_heff(rng, chi_l, chi_r, w=5, d=2, cplx=False):
    """A Hermitian 2-site H_eff: L, W1, W2, R hermitised so that the map is Hermitian."""
    def herm_env(chi):
        E = rnd(rng, (chi, w, chi), cplx)
        return E + np.conj(np.transpose(E, (2, 1, 0)))
    def herm_op():
        W = rnd(rng, (w, d, d, w), cplx)
        return W + np.conj(np.transpose(W, (0, 2, 1, 3)))
    return herm_env(chi_l), herm_op(), herm_op(), herm_env(chi_r)


def _heff_numpy(L, W1, W2, R):
    return lambda x: np.einsum("pwa,wtsv,vuxz,qzb,asxb->ptuq", L, W1, W2, R, x)


def _device_map(L, W1, W2, R):
    from networksolvers_gb300.network import LinearMap
    chi_l, chi_r = L.shape[0], R.shape[0]
    w, d = W1.shape[0], W1.shape[1]
    a, b = Index(chi_l, "Link"), Index(chi_r, "Link")
    w1, w2, w3 = Index(w), Index(w), Index(w)
    s1, s2 = Index(d, "Site"), Index(d, "Site")

    class P:
        def map_tensors(self):
            return [DTensor.from_numpy(L, [a.prime(), w1, a]), DTensor.from_numpy(W1, [w1, s1.prime(), s1, w2]),
                    DTensor.from_numpy(W2, [w2, s2.prime(), s2, w3]), DTensor.from_numpy(R, [b.prime(), w3, b])]
    return LinearMap(P(), [a, s1, s2, b]), [a, s1, s2, b]


@pytest.mark.parametrize("cplx", [False, True])
def test_linmap_matches_numpy(nsg_ctx, cplx):
    rng = np.random.default_rng(7)
    L, W1, W2, R = _chain_heff(rng, 11, 13, cplx=cplx)
    lm, inds = _device_map(L, W1, W2, R)
    x = rnd(rng, (11, 2, 2, 13), cplx)
    y = lm(DTensor.from_numpy(x, inds)).to_numpy()
    assert rel(y, _heff_numpy(L, W1, W2, R)(x)) < 1e-12
    assert lm.flops() > 0


@pytest.mark.parametrize("krylovdim,maxiter", [(3, 1), (6, 3)])
def test_lanczos_matches_oracle(nsg_ctx, krylovdim, maxiter):
    from networksolvers_gb300.sweep import eigsolve_solver
    rng = np.random.default_rng(8)
    L, W1, W2, R = _chain_heff(rng, 12, 10)
    lm, inds = _device_map(L, W1, W2, R)
    x0 = rnd(rng, (12, 2, 2, 10))
    lam, x = eigsolve_solver(lm, DTensor.from_numpy(x0, inds), krylovdim=krylovdim, maxiter=maxiter)
    lam_o, x_o = ok.eigsolve_lanczos(_heff_numpy(L, W1, W2, R), x0, krylovdim=krylovdim, maxiter=maxiter)
    assert abs(lam - lam_o) <= 1e-12 * abs(lam_o)
    assert abs(abs(np.vdot(x.to_numpy(), x_o)) - 1) < 1e-12


def test_lanczos_breakdown_small_space(nsg_ctx):
    """Local space smaller than krylovdim (chain end): the factorisation stops on breakdown."""
    from networksolvers_gb300.sweep import eigsolve_solver
    rng = np.random.default_rng(9)
    L, W1, W2, R = _chain_heff(rng, 1, 1)
    lm, inds = _device_map(L, W1, W2, R)
    x0 = rnd(rng, (1, 2, 2, 1))
    lam, x = eigsolve_solver(lm, DTensor.from_numpy(x0, inds), krylovdim=8, maxiter=1)
    H = _heff_numpy(L, W1, W2, R)
    dense = np.stack([H(e.reshape(1, 2, 2, 1)).ravel() for e in np.eye(4)], axis=1)
    assert abs(lam - np.linalg.eigvalsh(dense)[0]) < 1e-11


def test_exponentiate_and_rk4(nsg_ctx):
    from networksolvers_gb300.sweep import exponentiate_solver, runge_kutta_solver
    import scipy.linalg as sla
    rng = np.random.default_rng(10)
    L, W1, W2, R = _chain_heff(rng, 5, 4, cplx=True)
    lm, inds = _device_map(L, W1, W2, R)
    H = _heff_numpy(L, W1, W2, R)
    n = 5 * 2 * 2 * 4
    dense = np.stack([H(e.reshape(5, 2, 2, 4)).ravel() for e in np.eye(n)], axis=1)
    x0 = rnd(rng, (5, 2, 2, 4), True)
    x0 /= np.linalg.norm(x0)
    t = -0.05j
    y, info = exponentiate_solver(lm, t, DTensor.from_numpy(x0, inds))
    exact = (sla.expm(t * dense) @ x0.ravel()).reshape(x0.shape)
    assert rel(y.to_numpy(), exact) < 1e-10
    y_o, _ = ok.exponentiate(H, t, x0)
    assert rel(y.to_numpy(), y_o) < 1e-11
    z, _ = runge_kutta_solver(lm, t, DTensor.from_numpy(x0, inds), order=4)
    assert rel(z.to_numpy(), ok.runge_kutta_4(H, t, x0)) < 1e-12
    z2, _ = runge_kutta_solver(lm, t, DTensor.from_numpy(x0, inds), order=2)
    assert rel(z2.to_numpy(), ok.runge_kutta_2(H, t, x0)) < 1e-12


def test_concat_directsum(nsg_ctx):
    rng = np.random.default_rng(11)
    a0, s, a, u = Index(4), Index(2), Index(3), Index(2)
    A = rnd(rng, (4, 2, 3)); U = rnd(rng, (4, 2, 2))
    Ax, ax = it.directsum(DTensor.from_numpy(A, [a0, s, a]), a, DTensor.from_numpy(U, [a0, s, u]), u)
    assert np.array_equal(Ax.to_numpy(), np.concatenate([A, U], axis=2))


def test_errors_are_reported(nsg_ctx):
    from networksolvers_gb300._native import NsgError
    a, b = Index(3), Index(4)
    T = DTensor.from_numpy(np.ones((3, 4)), [a, b])
    with pytest.raises(NsgError):
        it.factorize(T, [], cutoff=0.0)


def _dmrg_like(rng, m, n, cplx):
    """Singular values with exact triple degeneracies and a long tail (an SU(2)-like
    entanglement spectrum), as the Gram matrices of a DMRG bond have."""
    k = min(m, n)
    s = np.repeat(np.exp(-0.12 * np.arange((k + 2) // 3)), 3)[:k]
    s[2 * k // 3:] *= 1e-7
    U, _ = np.linalg.qr(rnd(rng, (m, k), cplx))
    V, _ = np.linalg.qr(rnd(rng, (n, k), cplx))
    return (U * s) @ V.conj().T


def _cutoff_tie(P, k, cutoff, resolution=1e-14):
    """True when the cutoff rule decides the kept count k by a margin of at most
    `resolution` of the total weight: the discarded weight at k, or at k - 1, lies that
    close to cutoff * sum(P).  FP64-level Gram products and eigensolvers resolve the
    spectrum's partial sums to about 1e-15 of the total, so such a boundary can land on
    either side."""
    if cutoff <= 0:
        return False
    tot = float(P.sum())
    return any(abs(float(P[j:].sum()) - cutoff * tot) <= resolution * tot for j in (k, k - 1) if 0 <= j < len(P))


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("m,n", [(1, 3), (33, 33), (64, 40), (200, 260), (513, 513), (1100, 900)])
def test_eigensolver_large_and_degenerate(nsg_ctx, cplx, m, n, precision):
    """Exact bond dimensions, orthonormal U (1e-12) and the discarded weight, in the plain
    form and with C = U^H M on the Ozaki tensor-core path."""
    rng = np.random.default_rng(m + 7 * n)
    M = _dmrg_like(rng, m, n, cplx)
    l, r = Index(m), Index(n)
    T = DTensor.from_numpy(M, [l, r])
    for cutoff, maxdim in [(0.0, None), (1e-12, None), (1e-8, 3 * min(m, n) // 4 + 1)]:
        nsg_ctx.set_precision(precision)
        try:
            U, Cc, info = it.factorize(T, [l], cutoff=cutoff, maxdim=maxdim, spectrum=True)
        finally:
            nsg_ctx.set_precision("fp64")
        s = np.linalg.svd(M, compute_uv=False)
        kref, errref = ol.truncate_spectrum(s ** 2, cutoff, maxdim)
        if info["newdim"] != kref and _cutoff_tie(s ** 2, kref, cutoff):
            # the cutoff decides kref by a margin below FP64 resolution of the total
            # weight: one state more or fewer is the same truncation
            assert abs(info["newdim"] - kref) == 1, (cutoff, maxdim)
            kref = info["newdim"]
            errref = float((s ** 2)[kref:].sum() / (s ** 2).sum())
        assert info["newdim"] == kref, (cutoff, maxdim)
        u = U.to_numpy().reshape(m, -1)
        assert np.abs(u.conj().T @ u - np.eye(kref)).max() < 1e-12
        Pk = u @ Cc.to_numpy().reshape(kref, n)
        assert abs(np.linalg.norm(M - Pk) ** 2 / np.linalg.norm(M) ** 2 - errref) < 1e-12
        assert rel(info["spectrum"][:kref], s[:kref] ** 2) < 1e-12


@pytest.mark.parametrize("n", [24, 200, 700])
def test_eigh_exact_multiplets(nsg_ctx, n):
    """Spectra with exact multiplets (the Heisenberg chain's SU(2) structure in the extreme)
    make the divide and conquer deflate by close poles: its rotation sweep and the merges
    around rotated poles run.  Eigenvalues 1e-12 of the largest, orthonormal eigenvectors,
    reconstruction of the kept part."""
    rng = np.random.default_rng(n)
    mult = rng.integers(1, 6, size=n)
    lam = np.repeat(np.linspace(1.0, 0.01, n), mult)[:n]
    lam[rng.random(n) < 0.2] = 0.0  # and an exact null space
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    k = Index(n)
    T = DTensor.from_numpy(A, [k.prime(), k])
    D, U, u = it.eigen_hermitian(T, [k], cutoff=0.0, maxdim=n)
    ref = np.sort(np.linalg.eigvalsh(A))[::-1]
    assert np.max(np.abs(D - ref[: len(D)])) < 1e-12 * ref[0]
    Un = U.to_numpy().reshape(n, -1)
    assert np.abs(Un.T @ Un - np.eye(Un.shape[1])).max() < 1e-12
    assert np.linalg.norm((Un * D) @ Un.T - A) < 1e-12 * n * np.linalg.norm(A)


def test_fused_region_step_matches_call_by_call(nsg_ctx):
    """nsg_region_step (product, Lanczos, truncated factorization in one call) against
    the same region step taken entry point by entry point."""
    import networksolvers_gb300.models as models
    from kernelbench import _FixedMap
    from networksolvers_gb300.network import LinearMap
    from networksolvers_gb300.sweep import eigsolve_solver, region_step
    rng = np.random.default_rng(11)
    chi, d = 40, 2
    W = models.heisenberg_chain(4).tensors[2]
    w = W.shape[0]
    a, b, cc, s1, s2 = Index(chi), Index(chi), Index(chi), Index(d), Index(d)
    w1, w2, w3 = Index(w), Index(w), Index(w)
    Ln = rng.standard_normal((chi, w, chi))
    Rn = rng.standard_normal((chi, w, chi))
    L = DTensor.from_numpy(Ln + Ln.transpose(2, 1, 0), [a.prime(), w1, a])
    R = DTensor.from_numpy(Rn + Rn.transpose(2, 1, 0), [b.prime(), w3, b])
    W1 = DTensor.from_numpy(W, [w1, s1.prime(), s1, w2])
    W2 = DTensor.from_numpy(W, [w2, s2.prime(), s2, w3])
    p1 = DTensor.from_numpy(rng.standard_normal((chi, d, chi)), [a, s1, cc])
    p2 = DTensor.from_numpy(rng.standard_normal((chi, d, chi)), [cc, s2, b])
    E1, U1, C1, info1 = region_step(L, W1, W2, R, p1, p2, direction=0, krylovdim=3, maxiter=1, cutoff=1e-10,
                                    maxdim=30)
    local = contract([p1, p2], out=[a, s1, s2, b])
    lm = LinearMap(_FixedMap([L, R, W1, W2]), [a, s1, s2, b])
    E2, x = eigsolve_solver(lm, local, krylovdim=3, maxiter=1)
    U2, C2, info2 = it.factorize(x, [a, s1], cutoff=1e-10, maxdim=30)
    assert abs(E1 - E2) <= 1e-13 * abs(E2)
    assert info1["newdim"] == info2["newdim"] == 30
    assert abs(info1["truncerr"] - info2["truncerr"]) <= 1e-14
    k = info1["newdim"]
    P1 = U1.to_numpy().reshape(chi * d, k) @ C1.to_numpy().reshape(k, d * chi)
    P2 = U2.to_numpy().reshape(chi * d, k) @ C2.to_numpy().reshape(k, d * chi)
    assert rel(P1, P2) < 1e-12
