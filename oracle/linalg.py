"""Restated factorizations of ITensors/NDTensors (test infrastructure).

`truncate_spectrum` restates NDTensors' truncation rule for a descending spectrum
P (σ² for SVD, λ for Hermitian eigen): zero negative tail entries; discard down to
maxdim; then keep discarding from the end while (discarded + P[n] < cutoff·ΣP) and
n > mindim; the discarded weight is reported relative to ΣP.  Call sites in the
reference: inserter.jl:23 (`factorize`), subspace/densitymatrix.jl:53 (`eigen`),
truncation parameters from truncation_parameters.jl:7-14.
"""
from __future__ import annotations

import numpy as np

from .tensor import Index, Tensor


def truncate_spectrum(P, cutoff=0.0, maxdim=None, mindim=1):
    P = np.array(P, dtype=np.float64)
    origm = len(P)
    for n in range(origm - 1, -1, -1):
        if P[n] >= 0:
            break
        P[n] = 0.0
    maxdim = origm if maxdim is None else min(int(maxdim), origm)
    n = origm
    truncerr = 0.0
    while n > maxdim:
        truncerr += P[n - 1]
        n -= 1
    scale = float(P.sum())
    if scale == 0.0:
        scale = 1.0
    while n > mindim and (truncerr + P[n - 1] < cutoff * scale):
        truncerr += P[n - 1]
        n -= 1
    n = max(n, 1)
    return n, truncerr / scale


def _matricize(T: Tensor, left):
    left = [i for i in T.inds if i in left]
    right = [i for i in T.inds if i not in left]
    M = T.permute(left + right).data
    ml = int(np.prod([i.dim for i in left])) if left else 1
    return M.reshape(ml, -1), left, right


def factorize(T: Tensor, left, cutoff=0.0, maxdim=None, mindim=1, tags="Link", return_gap=False):
    """U·C = T truncated; U an isometry on `left` (ortho="left"), C = S·V†.
    Returns (U, C, truncerr, spectrum_kept), and with return_gap the relative gap of the
    cut, (s_k^2 - s_{k+1}^2) / s_k^2 between the last kept and the first discarded weight
    (inf when nothing is discarded): near zero, the cut runs through a (near-)degenerate
    multiplet and the kept subspace is fixed only up to rotations inside it."""
    M, L, R = _matricize(T, left)
    u, s, vh = np.linalg.svd(M, full_matrices=False)
    n, err = truncate_spectrum(s * s, cutoff, maxdim, mindim)
    link = Index(n, tags)
    U = Tensor(u[:, :n].reshape([i.dim for i in L] + [n]), L + [link])
    C = Tensor((s[:n, None] * vh[:n]).reshape([n] + [i.dim for i in R]), [link] + R)
    if return_gap:
        gap = float("inf") if n >= len(s) or s[n - 1] == 0 else float((s[n - 1] ** 2 - s[n] ** 2) / s[n - 1] ** 2)
        return U, C, err, s[:n] ** 2, gap
    return U, C, err, s[:n] ** 2


def qr(T: Tensor, left, tags="Link"):
    M, L, R = _matricize(T, left)
    q, r = np.linalg.qr(M, mode="reduced")
    k = q.shape[1]
    link = Index(k, tags)
    Q = Tensor(q.reshape([i.dim for i in L] + [k]), L + [link])
    Rt = Tensor(r.reshape([k] + [i.dim for i in R]), [link] + R)
    return Q, Rt


def eigen_hermitian(rho: Tensor, ket_inds, cutoff=0.0, maxdim=None, mindim=1, tags="Link"):
    """rho has inds (ket_inds', ket_inds).  Returns (D, U) with U[ket_inds..., new],
    eigenvalues descending, truncated by `truncate_spectrum`."""
    bra = [i.prime() for i in ket_inds]
    M = rho.permute(bra + list(ket_inds)).data
    m = int(np.prod([i.dim for i in ket_inds]))
    M = M.reshape(m, m)
    M = 0.5 * (M + M.conj().T)
    w, V = np.linalg.eigh(M)
    order = np.argsort(-w, kind="stable")
    w, V = w[order], V[:, order]
    n, err = truncate_spectrum(w, cutoff, maxdim, mindim)
    link = Index(n, tags)
    U = Tensor(V[:, :n].reshape([i.dim for i in ket_inds] + [n]), list(ket_inds) + [link])
    return w[:n], U, link


def directsum(A: Tensor, a: Index, U: Tensor, u: Index, tags="Link"):
    """[A | U] along a new index of dim(a)+dim(u) (ITensors `directsum(A=>a, U=>u)`)."""
    other = [i for i in A.inds if i != a]
    Ad = A.permute(other + [a]).data
    Ud = U.permute(other + [u]).data
    ax = Index(a.dim + u.dim, tags)
    return Tensor(np.concatenate([Ad, Ud], axis=-1), other + [ax]), ax
