"""Exact diagonalisation on small graphs (test infrastructure).

Builds the many-body Hamiltonian directly from the model definition with scipy
sparse Kronecker products — independent of the tree/chain operator builders — and
plays the role of test/utilities/simple_ed_methods.jl:4-42 (`ed_ground_state`,
`ed_time_evolution`).  The basis is ordered with the first vertex as the most
significant factor.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _site_op(op, k, n):
    mats = [sp.identity(2, format="csr")] * n
    mats = list(mats)
    mats[k] = sp.csr_matrix(op)
    out = mats[0]
    for m in mats[1:]:
        out = sp.kron(out, m, format="csr")
    return out


def hamiltonian(vertices, bond_terms, site_terms=None):
    """bond_terms: list of (i, j, coef, A, B); site_terms: dict v -> matrix."""
    n = len(vertices)
    pos = {v: k for k, v in enumerate(vertices)}
    H = sp.csr_matrix((2 ** n, 2 ** n))
    for (i, j, c, A, B) in bond_terms:
        H = H + c * (_site_op(A, pos[i], n) @ _site_op(B, pos[j], n))
    for v, h in (site_terms or {}).items():
        H = H + _site_op(h, pos[v], n)
    return H.tocsr()


def heisenberg_terms(edges, J=1.0, delta=1.0):
    sz = np.diag([0.5, -0.5])
    spl = np.array([[0.0, 1.0], [0.0, 0.0]])
    smi = spl.T
    out = []
    for (i, j) in edges:
        out += [(i, j, J * delta, sz, sz), (i, j, 0.5 * J, spl, smi), (i, j, 0.5 * J, smi, spl)]
    return out


def ground_energy(H):
    if H.shape[0] <= 64:
        return float(np.linalg.eigvalsh(H.toarray())[0])
    w = spla.eigsh(H, k=1, which="SA", tol=1e-13, maxiter=100000)[0]
    return float(w[0])


def ground_state(H):
    if H.shape[0] <= 64:
        w, V = np.linalg.eigh(H.toarray())
        return float(w[0]), V[:, 0]
    w, V = spla.eigsh(H, k=1, which="SA", tol=1e-13, maxiter=100000)
    return float(w[0]), V[:, 0]


def evolve(H, psi, t):
    """exp(-i H t) psi."""
    return spla.expm_multiply(-1j * t * H, psi)
