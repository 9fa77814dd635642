"""U(1) quantum-number (QN) block-sparse tensors on the device, and two-site DMRG on a
chain with them — the `conserve_qns=true` path of the reference's tensor stack (NDTensors
BlockSparse storage: one dense block per allowed combination of index sectors;
contraction block pair by block pair; SVD / eigen per QN sector of the row space with the
truncation applied to all sectors' values together).

Index arrows and flux: every index carries a direction (+1 / -1) and a list of sectors
(qn, dim); a block with sectors (s_1, ..., s_r) exists only when
sum_i dir_i * qn_i(s_i) equals the tensor's flux.  A bond shared by two tensors appears
with opposite directions, so fluxes add under contraction.

Storage: a block is a dense device tensor (`DTensor`) whose indices are the per-sector
indices `QNIndex.sec(s)` (id = (QN index id, s), same prime level), so the device
contraction engine pairs blocks of shared QN indices by label.  The host keeps the
block dictionary and issues one device contraction per matching block pair, one device
factorization per row-space sector (assembled with `nsg_copy_submatrix`), and block-wise
vector algebra for the Lanczos solver.

Chain conventions (two-site DMRG): A_j [a_{j-1} (+1), s_j (+1), a_j (-1)] with flux 0 and
the total QN on the last link; W_j [w_{j-1} (+1), s_j' (+1), s_j (-1), w_j (-1)] with
flux 0 (its link QNs inferred from the dense MPO, `qn_mpo`); environments
L_j [a_j' (+1), w_j (-1), a_j (-1)] and R_j [a_{j-1}' (-1), w_{j-1} (+1), a_{j-1} (+1)].
"""
from __future__ import annotations

import ctypes as C
import itertools
import math
from collections import defaultdict

import numpy as np

from . import _native as N
from .itensors import DTensor, Index, contract, factorize, inner

__all__ = ["QNIndex", "BlockTensor", "qcontract", "qfactorize", "qn_lanczos", "qn_mpo", "qn_product_state",
           "qn_dmrg_chain", "allowed_sectors", "truncate_sectors", "infer_link_qns", "site_qns"]

_qn_ids = itertools.count(1)


class QNIndex:
    """An index with U(1) sectors ((qn, dim), ...) and a direction (+1 / -1)."""

    __slots__ = ("sectors", "dir", "tags", "plev", "id", "dim", "offsets", "_sec")

    def __init__(self, sectors, dir=1, tags="", plev=0, id=None):
        self.sectors = tuple((int(q), int(d)) for q, d in sectors)
        self.dir = int(dir)
        self.tags = tags
        self.plev = plev
        self.id = ("qn", next(_qn_ids)) if id is None else id
        self.dim = sum(d for _, d in self.sectors)
        offs, o = [], 0
        for _, d in self.sectors:
            offs.append(o)
            o += d
        self.offsets = tuple(offs)
        self._sec = {}

    def prime(self, n=1):
        return QNIndex(self.sectors, self.dir, self.tags, self.plev + n, self.id)

    def noprime(self):
        return QNIndex(self.sectors, self.dir, self.tags, 0, self.id)

    def dag(self):
        return QNIndex(self.sectors, -self.dir, self.tags, self.plev, self.id)

    def key(self):
        return (self.id, self.plev)

    def __eq__(self, o):
        return isinstance(o, QNIndex) and self.key() == o.key()

    def __hash__(self):
        return hash(self.key())

    def qn(self, s):
        return self.sectors[s][0]

    def sec(self, s):
        """The dense index of sector s (the label the device contraction sees)."""
        ix = self._sec.get(s)
        if ix is None:
            ix = self._sec[s] = Index(self.sectors[s][1], self.tags, self.plev, (self.id, s))
        return ix

    def __repr__(self):
        return f"QNIndex({list(self.sectors)},dir={self.dir},id={self.id}{chr(39) * self.plev})"


def allowed_sectors(inds, flux):
    """Every sector combination of `inds` whose arrowed QN sum equals `flux`."""
    out = []
    for combo in itertools.product(*[range(len(q.sectors)) for q in inds]):
        if sum(q.dir * q.qn(s) for q, s in zip(inds, combo)) == flux:
            out.append(combo)
    return out


class BlockTensor:
    """Block-sparse tensor: `blocks` maps sector tuples (one sector position per index)
    to dense device blocks with indices [inds[k].sec(s_k)]."""

    __slots__ = ("inds", "blocks", "flux")

    def __init__(self, inds, blocks, flux=0):
        self.inds = tuple(inds)
        self.blocks = dict(blocks)
        self.flux = int(flux)

    # -- construction / inspection --------------------------------------------------
    @classmethod
    def from_dense(cls, arr, inds, flux=0, ctx=None, tol=0.0, keep_zero=False):
        """Blocks of the dense array `arr` (index order `inds`); allowed blocks that are
        exactly zero are left out unless `keep_zero`.  Entries outside the allowed blocks
        must vanish (|x| <= tol * max|arr|): the array conserves the QN."""
        arr = np.asarray(arr)
        assert arr.shape == tuple(q.dim for q in inds), (arr.shape, inds)
        mask = np.zeros(arr.shape, dtype=bool)
        blocks = {}
        for combo in allowed_sectors(inds, flux):
            sl = tuple(slice(q.offsets[s], q.offsets[s] + q.sectors[s][1]) for q, s in zip(inds, combo))
            mask[sl] = True
            if keep_zero or np.any(arr[sl]):
                blocks[combo] = DTensor.from_numpy(arr[sl], [q.sec(s) for q, s in zip(inds, combo)], ctx=ctx)
        outside = np.abs(arr[~mask]).max() if (~mask).any() else 0.0
        scale = np.abs(arr).max() if arr.size else 0.0
        if outside > tol * scale:
            raise ValueError(f"BlockTensor.from_dense: the array does not conserve the QN (|outside| = {outside:.3e})")
        return cls(inds, blocks, flux)

    def to_dense(self):
        dt = np.complex128 if any(b.is_complex() for b in self.blocks.values()) else np.float64
        out = np.zeros(tuple(q.dim for q in self.inds), dtype=dt)
        for combo, b in self.blocks.items():
            sl = tuple(slice(q.offsets[s], q.offsets[s] + q.sectors[s][1]) for q, s in zip(self.inds, combo))
            out[sl] = b.to_numpy()
        return out

    def is_complex(self):
        return any(b.is_complex() for b in self.blocks.values())

    def nnz(self):
        return sum(b.size for b in self.blocks.values())

    # -- index metadata -------------------------------------------------------------
    def prime(self):
        return BlockTensor([q.prime() for q in self.inds], {k: b.prime() for k, b in self.blocks.items()}, self.flux)

    def noprime(self):
        return BlockTensor([q.noprime() for q in self.inds], {k: b.noprime() for k, b in self.blocks.items()},
                           self.flux)

    def dag(self):
        return BlockTensor([q.dag() for q in self.inds], {k: b.dag() for k, b in self.blocks.items()}, -self.flux)

    def permute(self, inds):
        inds = list(inds)
        pos = [self.inds.index(q) for q in inds]
        blocks = {}
        for combo, b in self.blocks.items():
            nc = tuple(combo[p] for p in pos)
            blocks[nc] = b.permute([b.inds[p] for p in pos])
        return BlockTensor([self.inds[p] for p in pos], blocks, self.flux)

    def replaceind(self, old, new):
        """Swap QN index `old` for `new` (same sectors): blocks relabelled."""
        k = self.inds.index(old)
        assert new.sectors == old.sectors
        inds = list(self.inds)
        inds[k] = new
        blocks = {}
        for combo, b in self.blocks.items():
            blocks[combo] = b.replaceind(old.sec(combo[k]), new.sec(combo[k]))
        return BlockTensor(inds, blocks, self.flux)

    # -- vector algebra (Lanczos) ---------------------------------------------------
    def copy(self):
        return BlockTensor(self.inds, {k: b.copy() for k, b in self.blocks.items()}, self.flux)

    def scale_(self, s):
        for b in self.blocks.values():
            b.scale_(s)
        return self

    def axpy_(self, a, x):
        """self += a x (x with the same indices, possibly in another order or with other
        blocks present)."""
        xx = x if tuple(x.inds) == tuple(self.inds) else x.permute(self.inds)
        for combo, b in xx.blocks.items():
            if combo in self.blocks:
                self.blocks[combo].axpy_(a, b)
            else:
                nb = b.materialize().copy()
                nb.scale_(a)
                self.blocks[combo] = nb
        return self

    def norm(self):
        return math.sqrt(sum(b.norm() ** 2 for b in self.blocks.values()))


def qinner(a: BlockTensor, b: BlockTensor):
    """<a, b> = sum conj(a) b over the blocks both hold."""
    bb = b if tuple(b.inds) == tuple(a.inds) else b.permute(a.inds)
    s = 0.0
    for combo, blk in a.blocks.items():
        if combo in bb.blocks:
            s += inner(blk, bb.blocks[combo])
    return s


def qcontract(a: BlockTensor, b: BlockTensor):
    """Contract two block tensors over their shared QN indices: one device contraction per
    pair of blocks that agree on the shared sectors, summed into the output block of the
    remaining sectors.  Result indices: a's free ones, then b's."""
    shared = [(i, b.inds.index(q)) for i, q in enumerate(a.inds) if q in b.inds]
    sa = [i for i, _ in shared]
    sb = [j for _, j in shared]
    fa = [i for i in range(len(a.inds)) if i not in sa]
    fb = [j for j in range(len(b.inds)) if j not in sb]
    out_inds = [a.inds[i] for i in fa] + [b.inds[j] for j in fb]
    bykey = defaultdict(list)
    for combo, blk in b.blocks.items():
        bykey[tuple(combo[j] for j in sb)].append((combo, blk))
    out = {}
    for ca, ba in a.blocks.items():
        for cb, bb in bykey.get(tuple(ca[i] for i in sa), ()):
            oc = tuple(ca[i] for i in fa) + tuple(cb[j] for j in fb)
            res = contract([ba, bb], out=[q.sec(s) for q, s in zip(out_inds, oc)])
            if oc in out:
                out[oc].axpy_(1.0, res)
            else:
                out[oc] = res
    return BlockTensor(out_inds, out, a.flux + b.flux)


def truncate_sectors(spectra, cutoff=0.0, maxdim=None, mindim=1):
    """Global truncation of per-sector spectra (each descending): the NDTensors rule
    (negative tail zeroed; cut to maxdim; then drop from the end while the discarded
    weight plus the next value stays below cutoff * total, keeping at least mindim) on
    the union of all sectors' values.  Returns (kept count per sector, relative discarded
    weight, kept values descending)."""
    vals = [(v, q, i) for q, sp in enumerate(spectra) for i, v in enumerate(sp)]
    vals.sort(key=lambda t: (-t[0], t[1], t[2]))
    P = np.array([max(v, 0.0) for v, _, _ in vals], dtype=np.float64)
    n = len(P)
    md = n if maxdim is None or maxdim <= 0 else min(int(maxdim), n)
    err = float(P[md:].sum())
    n = md
    total = float(P.sum()) or 1.0
    while n > mindim and err + P[n - 1] < cutoff * total:
        err += P[n - 1]
        n -= 1
    n = max(n, 1) if len(P) else 0
    keep = [0] * len(spectra)
    for _, q, _ in vals[:n]:
        keep[q] += 1
    return keep, err / total, P[:n]


def qfactorize(t: BlockTensor, left, cutoff=0.0, maxdim=None, mindim=1, tags="Link"):
    """it.factorize(t, left; ortho="left") for a block tensor (inserter.jl:23): the
    matricised tensor is block diagonal in the QN of its row space; each sector's
    (rows x cols) matrix is assembled on the device and factorized there (all its
    singular values kept), the truncation runs over all sectors' values together, and
    U [left..., link (-1)], C [link (+1), right...] are cut back into blocks."""
    if not t.blocks:
        raise ValueError("qfactorize: the tensor has no blocks (it is zero)")
    ctx = next(iter(t.blocks.values())).ctx
    lp = [t.inds.index(q) for q in left]
    rp = [i for i in range(len(t.inds)) if i not in lp]
    linds, rinds = [t.inds[i] for i in lp], [t.inds[i] for i in rp]
    groups = defaultdict(list)
    for combo, blk in t.blocks.items():
        ql = sum(t.inds[i].dir * t.inds[i].qn(combo[i]) for i in lp)
        groups[ql].append(combo)
    sector_qns = sorted(groups)
    fulls, spectra, layout = [], [], []
    for ql in sector_qns:
        rkeys = sorted({tuple(c[i] for i in lp) for c in groups[ql]})
        ckeys = sorted({tuple(c[i] for i in rp) for c in groups[ql]})
        rsz = {k: int(np.prod([linds[n].sectors[s][1] for n, s in enumerate(k)])) for k in rkeys}
        csz = {k: int(np.prod([rinds[n].sectors[s][1] for n, s in enumerate(k)])) for k in ckeys}
        roff, o = {}, 0
        for k in rkeys:
            roff[k], o = o, o + rsz[k]
        rows = o
        coff, o = {}, 0
        for k in ckeys:
            coff[k], o = o, o + csz[k]
        cols = o
        ri, ci = Index(rows), Index(cols)
        M = DTensor.zeros([ri, ci], dtype=N.C128 if t.is_complex() else N.F64, ctx=ctx)
        for combo in groups[ql]:
            blk = t.blocks[combo]
            order = [blk.inds[i] for i in lp + rp]
            bm = blk if (list(blk.inds) == order and not blk.conj) else blk.permute(order)
            rk, ck = tuple(combo[i] for i in lp), tuple(combo[i] for i in rp)
            ctx.check(ctx.L.nsg_copy_submatrix(ctx.h, bm.st.h, rsz[rk], 0, 0, M.st.h, rows, roff[rk], coff[ck],
                                               rsz[rk], csz[ck], 0))
        U, Cm, info = factorize(M, [ri], cutoff=0.0, spectrum=True)
        fulls.append((U, Cm, info["newdim"]))
        spectra.append(list(info["spectrum"]))
        layout.append((rkeys, ckeys, rsz, csz, roff, coff, rows))
    keep, err, kept_vals = truncate_sectors(spectra, cutoff, maxdim, mindim)
    link_secs = [(ql, k) for ql, k in zip(sector_qns, keep) if k > 0]
    link = QNIndex(link_secs, dir=+1, tags=tags)
    linkU = link.dag()
    ublocks, cblocks = {}, {}
    pos = 0
    dt = N.C128 if t.is_complex() else N.F64
    for (ql, k), (U, Cm, r), (rkeys, ckeys, rsz, csz, roff, coff, rows) in zip(zip(sector_qns, keep), fulls, layout):
        if k == 0:
            continue
        ls = pos
        pos += 1
        for rk in rkeys:
            inds = [linds[n].sec(s) for n, s in enumerate(rk)] + [linkU.sec(ls)]
            blk = DTensor.zeros(inds, dtype=dt, ctx=ctx)
            ctx.check(ctx.L.nsg_copy_submatrix(ctx.h, U.st.h, rows, roff[rk], 0, blk.st.h, rsz[rk], 0, 0, rsz[rk], k,
                                               0))
            ublocks[rk + (ls,)] = blk
        for ck in ckeys:
            inds = [link.sec(ls)] + [rinds[n].sec(s) for n, s in enumerate(ck)]
            blk = DTensor.zeros(inds, dtype=dt, ctx=ctx)
            ctx.check(ctx.L.nsg_copy_submatrix(ctx.h, Cm.st.h, r, 0, coff[ck], blk.st.h, k, 0, 0, k, csz[ck], 0))
            cblocks[(ls,) + ck] = blk
    Ut = BlockTensor(linds + [linkU], ublocks, 0)
    Ct = BlockTensor([link] + rinds, cblocks, t.flux)
    return Ut, Ct, dict(truncerr=err, newdim=int(sum(keep)), spectrum=np.asarray(kept_vals), sectors=link_secs)


def _tridiag_lowest(alpha, beta):
    k = len(alpha)
    T = np.diag(np.asarray(alpha, dtype=np.float64))
    for i in range(k - 1):
        T[i, i + 1] = T[i + 1, i] = beta[i]
    w, V = np.linalg.eigh(T)
    return w[0], V[:, 0]


def qn_lanczos(apply, x0: BlockTensor, krylovdim=3, maxiter=1, tol=1e-14):
    """KrylovKit `eigsolve(A, x0, 1, :SR; krylovdim, maxiter, tol)` (Lanczos) on block
    vectors, the same steps as the device solver for dense vectors: w = A v_j -
    beta_{j-1} v_{j-1}, two full classical Gram-Schmidt passes (alpha_j their summed
    projections on v_j), beta_j = ||w||; the lowest Ritz pair of the tridiagonal.
    Returns (eigenvalue, normalised eigenvector, number of applications)."""
    x = x0.copy()
    nx = x.norm()
    if not (nx > 0 and math.isfinite(nx)):
        raise ValueError("qn_lanczos: zero or non-finite start vector")
    x.scale_(1.0 / nx)
    ops = 0
    lam = None
    for it in range(maxiter):
        V = [x]
        alpha, beta = [], []
        for j in range(krylovdim):
            w = apply(V[j])
            ops += 1
            if j > 0:
                w.axpy_(-beta[j - 1], V[j - 1])
            a = 0.0
            for _ in range(2):
                co = [qinner(V[i], w) for i in range(j + 1)]
                for i in range(j + 1):
                    w.axpy_(-co[i], V[i])
                a += float(np.real(co[j]))
            b = w.norm()
            if not (math.isfinite(a) and math.isfinite(b)):
                raise FloatingPointError("qn_lanczos: non-finite scalar")
            alpha.append(a)
            beta.append(b)
            if j + 1 == krylovdim or b <= tol:
                break
            V.append(w.scale_(1.0 / b))
        lam, y = _tridiag_lowest(alpha, beta[: len(alpha) - 1])
        k = len(alpha)
        xn = V[0].copy().scale_(y[0])
        for j in range(1, k):
            xn.axpy_(y[j], V[j])
        xn.scale_(1.0 / xn.norm())
        x = xn
        if abs(beta[k - 1] * y[k - 1]) <= tol or it + 1 == maxiter:
            break
    return lam, x, ops


# ----------------------------------------------------------------------------
# chain models with U(1) conservation
# ----------------------------------------------------------------------------


def site_qns(H):
    """2 S^z of the local basis states (the diagonal of the model's Sz operator)."""
    from .models import SITE_OPS
    sz = np.real(np.diag(SITE_OPS["Sz"]))
    return [int(round(2 * v)) for v in sz]


def infer_link_qns(Ws, sq):
    """Link charges of a chain MPO W_j [w_{j-1}, s', s, w_j] (boundary links of dimension
    1) that conserves the U(1) charge with site charges `sq`: q(w_j) = q(w_{j-1}) + q(s') -
    q(s) for every non-zero entry whose left link state is reachable from the left
    boundary, propagated from q(w_0) = 0.  Entries of unreachable states never receive
    weight from the left boundary (they do not contribute to the operator).  Raises if a
    contributing entry breaks the rule (the operator does not conserve the charge).
    Returns (charges q(w_0), ..., q(w_N); reachable-state masks)."""
    unset = np.iinfo(np.int64).min
    qs = [np.zeros(1, dtype=np.int64)]
    live = [np.ones(1, dtype=bool)]
    for j, W in enumerate(Ws):
        ql, ll = qs[-1], live[-1]
        qr = np.full(W.shape[3], unset, dtype=np.int64)
        for a, sp, s, b in np.argwhere(np.abs(W) > 0):
            if not ll[a]:
                continue
            q = ql[a] + sq[sp] - sq[s]
            if qr[b] == unset:
                qr[b] = q
            elif qr[b] != q:
                raise ValueError(f"infer_link_qns: site {j + 1} breaks U(1) conservation at link state {b}")
        lr = qr != unset
        qr[~lr] = 0
        qs.append(qr)
        live.append(lr)
    return qs, live


def _sectors_and_perm(qvec):
    """Group states by charge (ascending): ((qn, dim), ...) and the permutation that
    makes each charge's states contiguous."""
    order = np.argsort(qvec, kind="stable")
    secs = []
    for q in qvec[order]:
        if secs and secs[-1][0] == int(q):
            secs[-1][1] += 1
        else:
            secs.append([int(q), 1])
    return [tuple(s) for s in secs], order


def qn_mpo(H, ctx=None):
    """Block-sparse chain MPO from a dense one (models.Network on chain_graph(N)).
    Returns (W list of BlockTensor [w_{j-1}, s_j', s_j, w_j], site QN indices, link QN
    indices)."""
    from .chain import _pad_op
    n = len(H.graph.vertices)
    Ws = [_pad_op(H.tensors[j], j, n) for j in range(1, n + 1)]
    sq = site_qns(H)
    qs, live = infer_link_qns(Ws, sq)
    # entries leaving an unreachable link state contribute nothing: drop them
    Ws = [np.where(live[j][:, None, None, None], W, 0.0) for j, W in enumerate(Ws)]
    ssec, sperm = _sectors_and_perm(np.array(sq))
    sites = [QNIndex(ssec, dir=+1, tags=f"Site,n={j}") for j in range(1, n + 1)]
    links, perms = [], []
    for j, qv in enumerate(qs):
        secs, perm = _sectors_and_perm(qv)
        links.append(QNIndex(secs, dir=+1, tags=f"OpLink,l={j}"))
        perms.append(perm)
    out = []
    for j in range(n):
        W = Ws[j][np.ix_(perms[j], sperm, sperm, perms[j + 1])]
        s = sites[j]
        out.append(BlockTensor.from_dense(W, [links[j], s.prime(), s.dag(), links[j + 1].dag()], 0, ctx=ctx))
    return out, sites, links


def qn_product_state(sites, states, ctx=None):
    """MPS of the product state `states` (basis index per site, in the model's basis
    order) as block tensors A_j [a_{j-1}, s_j, a_j] with bond dimension 1; the last link
    carries the total charge."""
    from .models import SITE_OPS
    sq = [int(round(2 * v)) for v in np.real(np.diag(SITE_OPS["Sz"]))]
    ssec, sperm = _sectors_and_perm(np.array(sq))
    pos_in_sorted = {int(b): i for i, b in enumerate(sperm)}
    q = 0
    left = QNIndex([(0, 1)], dir=+1, tags="Link,l=0")
    out = []
    for j, (s, st) in enumerate(zip(sites, states)):
        q += sq[st]
        right = QNIndex([(q, 1)], dir=+1, tags=f"Link,l={j + 1}")
        arr = np.zeros((1, s.dim, 1))
        arr[0, pos_in_sorted[st], 0] = 1.0
        out.append(BlockTensor.from_dense(arr, [left, s, right.dag()], 0, ctx=ctx))
        left = right
    return out


def _qheff(L, W1, W2, R):
    def apply(x: BlockTensor):
        t = qcontract(L, x)
        t = qcontract(t, W1)
        t = qcontract(t, W2)
        t = qcontract(t, R).noprime()
        return t.permute(x.inds)
    return apply


def qn_dmrg_chain(H, states, nsweeps, maxdim=None, cutoff=0.0, mindim=1, krylovdim=3, maxiter=1, tol=1e-14,
                  ctx=None, region_callback=None):
    """Two-site DMRG with U(1) conservation on a chain (eigsolve.jl:45-76 with the chain's
    Euler-tour plan, euler_plans.jl:4-13) from the product state `states`: per region the
    block-sparse H_eff (optimal_map, operator_map.jl:3-10), the Lanczos updater
    (eigsolve.jl:14-28) and the QN-sector truncated factorization (inserter.jl:23), with
    the environments rebuilt across the bond just left.  `maxdim` / `cutoff` / `mindim`
    are scalars or per-sweep lists.  Returns (energy, MPS block tensors, records) with
    records = [(sweep, region index, energy, new bond dimension), ...]."""
    from .sweep import get_or_last
    ctx = ctx or N.default_context()
    Ws, sites, _ = qn_mpo(H, ctx=ctx)
    A = qn_product_state(sites, states, ctx=ctx)
    n = len(A)
    wl = Ws[0].inds[0]
    wr = Ws[-1].inds[3]
    a0 = A[0].inds[0]
    aN = A[-1].inds[2]
    one = np.ones((1, 1, 1))
    Lenv = {0: BlockTensor.from_dense(one, [a0.prime(), wl.dag(), a0.dag()], 0, ctx=ctx)}
    Renv = {n + 1: BlockTensor.from_dense(one, [aN.prime(), wr.dag(), aN.dag()], 0, ctx=ctx)}

    def env(prev, j):
        a = A[j - 1]
        t = qcontract(prev, a)
        t = qcontract(t, Ws[j - 1])
        return qcontract(t, a.dag().prime())

    for j in range(n, 2, -1):
        Renv[j] = env(Renv[j + 1], j)
    records = []
    energy = None
    for sweep in range(1, nsweeps + 1):
        md = get_or_last(maxdim, sweep) if maxdim is not None else None
        co = get_or_last(cutoff, sweep)
        mi = get_or_last(mindim, sweep)
        regions = [(j, 0) for j in range(1, n)] + [(j, 1) for j in range(n - 1, 0, -1)]
        for k, (j, direction) in enumerate(regions):
            # the two-site tensor in [left link, site j, site j+1, right link] order (the
            # factorizations leave the site tensors' indices in varying orders)
            s1, s2 = sites[j - 1], sites[j]
            a_left = [q for q in A[j - 1].inds if q != s1 and q not in A[j].inds][0]
            b_right = [q for q in A[j].inds if q != s2 and q not in A[j - 1].inds][0]
            psi = qcontract(A[j - 1], A[j])
            psi = psi.permute([q for r in (a_left, s1, s2, b_right) for q in psi.inds if q == r])
            apply = _qheff(Lenv[j - 1], Ws[j - 1], Ws[j], Renv[j + 2])
            energy, psi, _ = qn_lanczos(apply, psi, krylovdim=krylovdim, maxiter=maxiter, tol=tol)
            a_left, s1, s2, b_right = psi.inds
            if direction == 0:
                U, Cc, info = qfactorize(psi, [a_left, s1], cutoff=co, maxdim=md, mindim=mi,
                                         tags=f"Link,l={j}")
                A[j - 1], A[j] = U, Cc
                if j < n - 1:
                    Lenv[j] = env(Lenv[j - 1], j)
            else:
                U, Cc, info = qfactorize(psi, [s2, b_right], cutoff=co, maxdim=md, mindim=mi,
                                         tags=f"Link,l={j}")
                A[j - 1], A[j] = Cc, U
                if j > 1:
                    Renv[j + 1] = env(Renv[j + 2], j + 1)
            records.append((sweep, k, energy, info["newdim"]))
            if region_callback is not None:
                region_callback(sweep, k, energy, info)
    return energy, A, records


def qn_to_dense_mps(A):
    """Dense numpy site tensors [left, site, right] of a block MPS, each index in its
    sector-sorted basis order (tests compare states through basis-independent
    quantities)."""
    return [a.to_dense() for a in A]
