"""Device-resident dense tensors with ITensor index semantics.

A `DTensor` is a handle to device memory (column-major, in the order of its indices)
plus a tuple of `Index` objects.  `A * B` contracts every index the two share (same
id and prime level) through `nsg_contract`; `dag()` and `prime()` are free (they
only change metadata; conjugation is folded into the next GEMM).  This is the
surface the reference's plugins use from ITensors (`*`, `prime`, `dag`, `noprime`,
`norm`, `inds`, `commonind`, `uniqueinds`).
"""
from __future__ import annotations

import ctypes as C
import itertools

import numpy as np

from . import _native as N

_ids = itertools.count(1)


class Index:
    __slots__ = ("id", "dim", "plev", "tags")

    def __init__(self, dim, tags="", plev=0, id=None):
        self.id = next(_ids) if id is None else id
        self.dim = int(dim)
        self.plev = plev
        self.tags = tags

    def prime(self, n=1):
        return Index(self.dim, self.tags, self.plev + n, self.id)

    def noprime(self):
        return Index(self.dim, self.tags, 0, self.id)

    def key(self):
        return (self.id, self.plev)

    def __eq__(self, o):
        return isinstance(o, Index) and self.key() == o.key()

    def __hash__(self):
        return hash(self.key())

    def __repr__(self):
        return f"Index({self.dim},{self.tags!r},id={self.id}{chr(39) * self.plev})"


class Storage:
    """Owns one nsg_tensor handle; released when the last DTensor drops it."""

    __slots__ = ("ctx", "h", "dtype", "dims")

    def __init__(self, ctx, h, dtype, dims):
        self.ctx, self.h, self.dtype, self.dims = ctx, h, dtype, tuple(dims)

    @classmethod
    def from_handle(cls, ctx, h):
        dt, rk = C.c_int(), C.c_int()
        dims = (C.c_int64 * 16)()
        ctx.check(ctx.L.nsg_tensor_shape(h, C.byref(dt), C.byref(rk), dims))
        return cls(ctx, h, dt.value, [dims[k] for k in range(rk.value)])

    def __del__(self):
        try:
            if self.h and self.ctx.h:
                self.ctx.L.nsg_tensor_release(self.ctx.h, self.h)
        except Exception:
            pass
        self.h = None


def _dims_arr(dims):
    return (C.c_int64 * max(1, len(dims)))(*dims)


class DTensor:
    __slots__ = ("st", "inds", "conj")

    def __init__(self, st: Storage, inds, conj=False):
        self.st = st
        self.inds = tuple(inds)
        self.conj = conj
        assert tuple(i.dim for i in self.inds) == st.dims, (self.inds, st.dims)

    # -- construction --------------------------------------------------------
    @classmethod
    def from_numpy(cls, arr, inds, ctx=None, dtype=None):
        ctx = ctx or N.default_context()
        a = np.asarray(arr)
        if dtype is None:
            dtype = N.C128 if np.iscomplexobj(a) else N.F64
        npdt = np.complex128 if dtype == N.C128 else np.float64
        buf = np.asfortranarray(a.astype(npdt, copy=False))
        h = C.c_void_p()
        dims = list(a.shape)
        ctx.check(ctx.L.nsg_tensor_upload(ctx.h, dtype, len(dims), _dims_arr(dims),
                                          buf.ctypes.data_as(C.c_void_p), C.byref(h)))
        return cls(Storage(ctx, h, dtype, dims), inds)

    @classmethod
    def zeros(cls, inds, dtype=N.F64, ctx=None):
        ctx = ctx or N.default_context()
        dims = [i.dim for i in inds]
        h = C.c_void_p()
        ctx.check(ctx.L.nsg_tensor_create(ctx.h, dtype, len(dims), _dims_arr(dims), C.byref(h)))
        return cls(Storage(ctx, h, dtype, dims), inds)

    @property
    def ctx(self):
        return self.st.ctx

    @property
    def dtype(self):
        return self.st.dtype

    @property
    def shape(self):
        return self.st.dims

    @property
    def size(self):
        return int(np.prod(self.st.dims)) if self.st.dims else 1

    def is_complex(self):
        return self.st.dtype == N.C128

    def to_numpy(self):
        npdt = np.complex128 if self.dtype == N.C128 else np.float64
        out = np.empty(self.shape, dtype=npdt, order="F")
        self.ctx.check(self.ctx.L.nsg_tensor_download(self.ctx.h, self.st.h, out.ctypes.data_as(C.c_void_p)))
        return np.conj(out) if self.conj else out

    def materialize(self):
        """A tensor owning fresh storage with conjugation applied."""
        if not self.conj:
            return self
        return self.permute(self.inds)

    def copy(self):
        if self.conj:
            return self.materialize()
        h = C.c_void_p()
        self.ctx.check(self.ctx.L.nsg_tensor_copy(self.ctx.h, self.st.h, C.byref(h)))
        return DTensor(Storage(self.ctx, h, self.dtype, self.shape), self.inds)

    # -- index metadata ------------------------------------------------------
    def prime(self, *which):
        if not which:
            return DTensor(self.st, [i.prime() for i in self.inds], self.conj)
        w = set(which)
        return DTensor(self.st, [i.prime() if i in w else i for i in self.inds], self.conj)

    def noprime(self):
        return DTensor(self.st, [i.noprime() for i in self.inds], self.conj)

    def dag(self):
        return DTensor(self.st, self.inds, not self.conj if self.is_complex() else False)

    def replaceind(self, old, new):
        return DTensor(self.st, [new if i == old else i for i in self.inds], self.conj)

    # -- algebra -------------------------------------------------------------
    def permute(self, inds):
        inds = list(inds)
        perm = (C.c_int * len(inds))(*[self.inds.index(i) for i in inds])
        h = C.c_void_p()
        self.ctx.check(self.ctx.L.nsg_permute(self.ctx.h, self.st.h, perm, int(self.conj), C.byref(h)))
        return DTensor(Storage(self.ctx, h, self.dtype, [i.dim for i in inds]), inds)

    def __mul__(self, other):
        if np.isscalar(other):
            out = self.copy()
            out.scale_(other)
            return out
        return contract([self, other])

    __rmul__ = lambda self, s: self * s

    def __truediv__(self, s):
        return self * (1.0 / s)

    def scale_(self, s):
        assert not self.conj
        s = complex(s)
        if s.imag != 0 and not self.is_complex():
            raise ValueError("complex scale of a real tensor")
        self.ctx.check(self.ctx.L.nsg_axpby(self.ctx.h, s.real, s.imag, self.st.h, 0.0, 0.0, self.st.h))
        return self

    def axpy_(self, a, x):
        """self += a * x (x aligned to self's index order)."""
        assert not self.conj
        xx = x if (tuple(x.inds) == tuple(self.inds) and not x.conj) else x.permute(self.inds)
        a = complex(a)
        self.ctx.check(self.ctx.L.nsg_axpby(self.ctx.h, a.real, a.imag, xx.st.h, 1.0, 0.0, self.st.h))
        return self

    def __add__(self, other):
        return self.materialize().copy().axpy_(1.0, other)

    def __sub__(self, other):
        return self.materialize().copy().axpy_(-1.0, other)

    def norm(self):
        out = C.c_double()
        self.ctx.check(self.ctx.L.nsg_norm(self.ctx.h, self.st.h, C.byref(out)))
        return out.value

    def __repr__(self):
        return f"DTensor{self.shape}{list(self.inds)}{'*' if self.conj else ''}"


def contract(tensors, out=None):
    """Contract a list of tensors over shared indices (optimal pairwise order on the
    device).  Result indices: uncontracted ones in order of first appearance, or `out`."""
    tensors = list(tensors)
    ctx = tensors[0].ctx
    counts = {}
    for t in tensors:
        for i in t.inds:
            counts[i] = counts.get(i, 0) + 1
    lab = {}
    for t in tensors:
        for i in t.inds:
            lab.setdefault(i, len(lab))
    free = [i for i in lab if counts[i] == 1] if out is None else list(out)
    dtype = N.C128 if any(t.is_complex() for t in tensors) else N.F64
    ts = []
    for t in tensors:
        if dtype == N.C128 and not t.is_complex():
            t = promote(t)
        ts.append(t)
    handles = (C.c_void_p * len(ts))(*[t.st.h for t in ts])
    flat = [lab[i] for t in ts for i in t.inds]
    labels = (C.c_int32 * max(1, len(flat)))(*flat)
    conj = (C.c_int * len(ts))(*[int(t.conj) for t in ts])
    outl = (C.c_int32 * max(1, len(free)))(*[lab[i] for i in free])
    h = C.c_void_p()
    ctx.check(ctx.L.nsg_contract(ctx.h, len(ts), handles, labels, conj, len(free), outl, C.byref(h)))
    return DTensor(Storage(ctx, h, dtype, [i.dim for i in free]), free)


def promote(t: DTensor):
    """Real tensor -> complex copy (host round trip is avoided: 0*i added on device)."""
    arr = t.to_numpy().astype(np.complex128)
    return DTensor.from_numpy(arr, t.inds, ctx=t.ctx)


def inner(a: DTensor, b: DTensor):
    bb = b if tuple(b.inds) == tuple(a.inds) else b.permute(a.inds)
    aa = a.materialize() if a.conj else a
    re, im = C.c_double(), C.c_double()
    a.ctx.check(a.ctx.L.nsg_dot(a.ctx.h, aa.st.h, bb.st.h, C.byref(re), C.byref(im)))
    return complex(re.value, im.value) if a.is_complex() else re.value


def commoninds(a, b):
    return [i for i in a.inds if i in b.inds]


def uniqueinds(a, b):
    return [i for i in a.inds if i not in b.inds]


def commonind(a, b):
    c = commoninds(a, b)
    return c[0] if c else None


def _axes(t, inds):
    return [t.inds.index(i) for i in inds]


def factorize(T: DTensor, left, cutoff=0.0, maxdim=None, mindim=1, tags="Link", spectrum=False, complement=False):
    """ITensors `factorize(T, left; ortho="left", cutoff, maxdim, mindim)` on device.
    Returns (U, C, info) with U[left..., link], C[link, right...].  With complement=True
    (and spectrum=False), info["complement"] is an orthonormal basis Uperp[left..., perp] of
    the complement of U's columns when the factorization produced one
    (nsg_factorize_complement), else None."""
    T = T.materialize()
    ctx = T.ctx
    left = [i for i in T.inds if i in left]
    right = [i for i in T.inds if i not in left]
    ax = (C.c_int * len(left))(*_axes(T, left))
    U, Cc = C.c_void_p(), C.c_void_p()
    k, err = C.c_int64(), C.c_double()
    md = -1 if maxdim is None else int(maxdim)
    perp = None
    if complement and not spectrum:
        Up = C.c_void_p()
        ctx.check(ctx.L.nsg_factorize_complement(ctx.h, T.st.h, ax, len(left), float(cutoff), md, int(mindim),
                                                 C.byref(U), C.byref(Cc), C.byref(Up), C.byref(k), C.byref(err)))
        if Up.value:
            rows = int(np.prod([i.dim for i in left]))
            perp = DTensor(Storage(ctx, Up, T.dtype, [i.dim for i in left] + [rows - k.value]),
                           left + [Index(rows - k.value, "Link,perp")])
    else:
        cap = int(min(np.prod([i.dim for i in left]), np.prod([i.dim for i in right])))
        spec = (C.c_double * cap)() if spectrum else None
        ctx.check(ctx.L.nsg_factorize(ctx.h, T.st.h, ax, len(left), float(cutoff), md, int(mindim),
                                      C.byref(U), C.byref(Cc), C.byref(k), C.byref(err), spec,
                                      cap if spectrum else 0))
    link = Index(k.value, tags)
    Ut = DTensor(Storage(ctx, U, T.dtype, [i.dim for i in left] + [k.value]), left + [link])
    Ct = DTensor(Storage(ctx, Cc, T.dtype, [k.value] + [i.dim for i in right]), [link] + right)
    info = dict(truncerr=err.value, newdim=k.value)
    if spectrum:
        info["spectrum"] = np.array(spec[: k.value])
    if complement:
        info["complement"] = perp
    return Ut, Ct, info


def qr(T: DTensor, left, tags="Link"):
    T = T.materialize()
    ctx = T.ctx
    left = [i for i in T.inds if i in left]
    right = [i for i in T.inds if i not in left]
    ax = (C.c_int * len(left))(*_axes(T, left))
    Q, R = C.c_void_p(), C.c_void_p()
    ctx.check(ctx.L.nsg_qr(ctx.h, T.st.h, ax, len(left), C.byref(Q), C.byref(R)))
    Qs = Storage.from_handle(ctx, Q)
    k = Qs.dims[-1]
    link = Index(k, tags)
    Qt = DTensor(Qs, left + [link])
    Rt = DTensor(Storage(ctx, R, T.dtype, [k] + [i.dim for i in right]), [link] + right)
    return Qt, Rt


def eigen_hermitian(rho: DTensor, ket_inds, cutoff=0.0, maxdim=None, mindim=1, tags="Link"):
    """rho has inds (ket', ket); eigenvectors U[ket..., link], eigenvalues descending."""
    rho = rho.materialize()
    ctx = rho.ctx
    bra = [i.prime() for i in ket_inds]
    rows = _axes(rho, bra)
    # column axes must be in ket order for the eigenvector layout
    rho = rho.permute(bra + list(ket_inds))
    ax = (C.c_int * len(bra))(*range(len(bra)))
    U = C.c_void_p()
    m = int(np.prod([i.dim for i in ket_inds]))
    ev = (C.c_double * m)()
    k, err = C.c_int64(), C.c_double()
    md = -1 if maxdim is None else int(maxdim)
    ctx.check(ctx.L.nsg_eigh(ctx.h, rho.st.h, ax, len(bra), float(cutoff), md, int(mindim), C.byref(U),
                             ev, m, C.byref(k), C.byref(err)))
    link = Index(k.value, tags)
    Ut = DTensor(Storage(ctx, U, rho.dtype, [i.dim for i in ket_inds] + [k.value]), list(ket_inds) + [link])
    return np.array(ev[: k.value]), Ut, link


def directsum(A: DTensor, a: Index, U: DTensor, u: Index, tags="Link"):
    """[A | U] along a new index of dim(a)+dim(u) (ITensors `directsum(A=>a, U=>u)`)."""
    other = [i for i in A.inds if i != a]
    Ap = A.permute(other + [a]) if (list(A.inds) != other + [a] or A.conj) else A
    Up = U.permute(other + [u]) if (list(U.inds) != other + [u] or U.conj) else U
    ctx = A.ctx
    h = C.c_void_p()
    ctx.check(ctx.L.nsg_concat(ctx.h, Ap.st.h, Up.st.h, len(other), C.byref(h)))
    ax = Index(a.dim + u.dim, tags)
    return DTensor(Storage(ctx, h, A.dtype, [i.dim for i in other] + [ax.dim]), other + [ax]), ax
