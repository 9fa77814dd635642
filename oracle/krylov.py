"""Restated local solvers (test infrastructure).

* `eigsolve_lanczos` — KrylovKit `eigsolve(A, x0, 1, :SR; krylovdim, maxiter, tol,
  ishermitian=true)` as called by local_solvers/eigsolve.jl:16-27: Lanczos with full
  reorthogonalisation (restated as the three-term recurrence followed by two full
  classical Gram-Schmidt passes; alpha is the sum of the two projections on the newest
  vector.  This spans the same Krylov space as KrylovKit's ModifiedGramSchmidtIR), Ritz pair of the
  smallest Ritz value.  A factorisation of dimension k costs k operator applications.
  Restarts (maxiter > 1) restart from the Ritz vector; every workload here uses
  maxiter = 1, the reference default.
* `exponentiate` — Lanczos exponential integrator for exp(t·A)·x with A Hermitian
  (local_solvers/exponentiate.jl:16-27): grow the basis one vector at a time
  (eager), accept the full remaining step when the estimate
  ‖x‖·|β_k|·|[exp(τT_k)]_{k,1}| ≤ tol; at krylovdim take the largest fraction of the
  remaining step (bisection, 50 halvings) whose estimate is ≤ tol·|τ_step|/|t| and
  restart from the advanced vector.
* `runge_kutta_2/4`, `runge_kutta_solver` — runge_kutta.jl:2-25, verbatim algebra.
"""
from __future__ import annotations

import numpy as np


def _tridiag(alpha, beta):
    k = len(alpha)
    T = np.diag(np.asarray(alpha, dtype=np.float64))
    for i in range(k - 1):
        T[i, i + 1] = T[i + 1, i] = beta[i]
    return T


def _dot(a, b):
    return np.vdot(a.ravel(), b.ravel())


def _norm(a):
    return float(np.linalg.norm(a.ravel()))


def lanczos_factorization(A, v0, kmax, breakdown, eager_check=None):
    """Grow a Lanczos factorisation from unit vector v0.  Returns (V, alpha, beta, r).
    beta[k-1] is the residual norm after the k-th vector; `eager_check(V, alpha, beta)`
    may stop the growth early by returning True."""
    V = [v0]
    alpha, beta = [], []
    while True:
        w = A(V[-1])
        # three-term recurrence, then two full classical Gram-Schmidt passes;
        # the projections onto the newest vector correct alpha
        if len(V) > 1:
            w = w - beta[-1] * V[-2]
        a = 0.0
        for _pass in range(2):
            coeffs = [_dot(v, w) for v in V]
            for c, v in zip(coeffs, V):
                w = w - c * v
            a = a + coeffs[-1]
        alpha.append(float(np.real(a)))
        b = _norm(w)
        beta.append(b)
        if eager_check is not None and eager_check(V, alpha, beta):
            return V, alpha, beta, w
        if len(V) >= kmax or b <= breakdown:
            return V, alpha, beta, w
        V.append(w / b)


def eigsolve_lanczos(A, x0, krylovdim=3, maxiter=1, tol=1e-14):
    x = x0 / _norm(x0)
    lam = None
    for it in range(maxiter):
        V, alpha, beta, _ = lanczos_factorization(A, x, krylovdim, breakdown=tol)
        T = _tridiag(alpha, beta[:-1])
        w, Y = np.linalg.eigh(T)
        lam = float(w[0])
        y = Y[:, 0]
        x = sum(c * v for c, v in zip(y, V))
        x = x / _norm(x)
        if abs(beta[-1] * y[-1]) <= tol:
            break
    return lam, x


def expm_small(A):
    """exp(A) of a small complex matrix: scaling and squaring with a degree-18 Taylor
    polynomial on A/2^s, ||A/2^s||_1 <= 1/2.  Entries that are tiny (the Krylov error
    corner [k-1, 0]) keep their relative accuracy, which an eigendecomposition does not."""
    A = np.asarray(A, dtype=np.complex128)
    k = A.shape[0]
    nrm = np.abs(A).sum(axis=0).max() if k else 0.0
    s = 0 if nrm <= 0.5 else int(np.ceil(np.log2(nrm / 0.5)))
    X = A / (2.0 ** s)
    E = np.eye(k, dtype=np.complex128)
    term = np.eye(k, dtype=np.complex128)
    for j in range(1, 19):
        term = (term @ X) / j
        E = E + term
    for _ in range(s):
        E = E @ E
    return E


def _expm_sym_tridiag(T, tau):
    return expm_small(tau * T)


def exponentiate(A, t, x, krylovdim=30, maxiter=100, tol=1e-12):
    """exp(t·A)·x, t complex scalar, A Hermitian.  Returns (y, info)."""
    t = complex(t)
    if t == 0:
        return x.copy(), {"converged": True, "numops": 0}
    dtype = np.result_type(x.dtype, np.complex128 if t.imag != 0 else x.dtype)
    w = x.astype(dtype)
    remaining = t
    numops = 0
    for it in range(maxiter):
        beta0 = _norm(w)
        if beta0 == 0.0:
            return w, {"converged": True, "numops": numops}
        state = {}

        def check(V, alpha, beta):
            k = len(alpha)
            T = _tridiag(alpha, beta[:-1])
            E = _expm_sym_tridiag(T, remaining)
            err = beta0 * abs(beta[-1]) * abs(E[k - 1, 0])
            state["E"], state["err"] = E, err
            return err <= tol

        V, alpha, beta, _ = lanczos_factorization(A, w / beta0, krylovdim, breakdown=tol * 1e-3,
                                                  eager_check=check)
        numops += len(alpha)
        k = len(alpha)
        if state["err"] <= tol or beta[-1] <= tol * 1e-3:
            step = remaining
            E = state["E"]
        else:
            # largest fraction s of the remaining time whose estimate is within the
            # per-unit-time budget tol*|step|/|t| (bisection, 50 halvings)
            T = _tridiag(alpha, beta[:-1])

            def est(s):
                Es = expm_small(remaining * s * T)[:, 0]
                return Es, beta0 * abs(beta[-1]) * abs(Es[k - 1])

            lo, hi = 0.0, 1.0
            for _ in range(50):
                mid = 0.5 * (lo + hi)
                if est(mid)[1] <= tol * mid * abs(remaining) / abs(t):
                    lo = mid
                else:
                    hi = mid
            if lo <= 0.0:
                return w, {"converged": False, "numops": numops}
            step = remaining * lo
            E = est(lo)[0][:, None]
        coef = beta0 * E[:, 0]
        w = sum(c * v for c, v in zip(coef, V))
        remaining = remaining - step
        if abs(remaining) <= 1e-15 * abs(t):
            return w, {"converged": True, "numops": numops}
    return w, {"converged": False, "numops": numops}


def runge_kutta_2(H, t, psi0):
    Hpsi = H(psi0)
    H2psi = H(Hpsi)
    return psi0 + t * Hpsi + (t ** 2 / 2) * H2psi


def runge_kutta_4(H, t, psi0):
    k1 = H(psi0)
    k2 = k1 + (t / 2) * H(k1)
    k3 = k1 + (t / 2) * H(k2)
    k4 = k1 + t * H(k3)
    return psi0 + (t / 6) * (k1 + 2 * k2 + 2 * k3 + k4)


def runge_kutta_solver(H, time, psi, order=4):
    if order == 4:
        return runge_kutta_4(H, time, psi), {}
    if order == 2:
        return runge_kutta_2(H, time, psi), {}
    raise ValueError("For runge_kutta_solver, must specify `order` keyword")
