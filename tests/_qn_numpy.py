"""Test-only numpy stand-ins for the device calls the QN layer makes (DTensor storage,
label-based contraction, inner product, truncated factorization, nsg_copy_submatrix),
so that the block bookkeeping of networksolvers_gb300/qn.py runs unchanged on the CPU
and can be checked against the dense oracle.  Never used by the library itself."""
import contextlib

import numpy as np

from networksolvers_gb300 import _native as N
from networksolvers_gb300 import qn
from networksolvers_gb300.itensors import Index


class _Lib:
    """The one library call qn.py issues directly."""

    @staticmethod
    def nsg_copy_submatrix(h, src, lds, r0s, c0s, dst, ldd, r0d, c0d, rows, cols, acc):
        for j in range(cols):
            s0, d0 = r0s + (c0s + j) * lds, r0d + (c0d + j) * ldd
            if acc:
                dst.flat[d0:d0 + rows] += src.flat[s0:s0 + rows]
            else:
                dst.flat[d0:d0 + rows] = src.flat[s0:s0 + rows]
        return 0


class FakeCtx:
    h = None
    L = _Lib()

    @staticmethod
    def check(rc):
        assert rc == 0


class _Store:
    """Column-major flat buffer; `h` is the handle qn.py passes to the library."""

    def __init__(self, arr, ctx):
        arr = np.asarray(arr)
        self.dims = tuple(arr.shape)
        self.flat = np.array(arr.reshape(-1, order="F"), dtype=arr.dtype)
        self.ctx = ctx
        self.h = self

    def array(self):
        return self.flat.reshape(self.dims, order="F")


class NpTensor:
    """The DTensor interface qn.py relies on, on a numpy buffer."""

    def __init__(self, st, inds, conj=False):
        self.st, self.inds, self.conj = st, tuple(inds), conj
        assert tuple(i.dim for i in self.inds) == st.dims

    @classmethod
    def from_numpy(cls, arr, inds, ctx=None, dtype=None):
        a = np.asarray(arr)
        a = a.astype(np.complex128 if (np.iscomplexobj(a) or dtype == N.C128) else np.float64)
        return cls(_Store(a, ctx or FakeCtx()), inds)

    @classmethod
    def zeros(cls, inds, dtype=N.F64, ctx=None):
        dt = np.complex128 if dtype == N.C128 else np.float64
        return cls(_Store(np.zeros([i.dim for i in inds], dtype=dt), ctx or FakeCtx()), inds)

    @property
    def ctx(self):
        return self.st.ctx

    @property
    def size(self):
        return int(np.prod(self.st.dims)) if self.st.dims else 1

    def is_complex(self):
        return np.iscomplexobj(self.st.flat)

    def to_numpy(self):
        a = self.st.array().copy()
        return np.conj(a) if self.conj else a

    def materialize(self):
        return NpTensor(_Store(self.to_numpy(), self.ctx), self.inds) if self.conj else self

    def copy(self):
        return NpTensor(_Store(self.to_numpy(), self.ctx), self.inds)

    def prime(self, *which):
        w = set(which)
        return NpTensor(self.st, [i.prime() if (not which or i in w) else i for i in self.inds], self.conj)

    def noprime(self):
        return NpTensor(self.st, [i.noprime() for i in self.inds], self.conj)

    def dag(self):
        return NpTensor(self.st, self.inds, (not self.conj) if self.is_complex() else False)

    def replaceind(self, old, new):
        return NpTensor(self.st, [new if i == old else i for i in self.inds], self.conj)

    def permute(self, inds):
        perm = [self.inds.index(i) for i in inds]
        return NpTensor(_Store(np.transpose(self.to_numpy(), perm), self.ctx), inds)

    def scale_(self, s):
        self.st.flat *= s
        return self

    def axpy_(self, a, x):
        xx = x.to_numpy() if tuple(x.inds) == tuple(self.inds) else x.permute(self.inds).to_numpy()
        if np.iscomplexobj(xx) and not self.is_complex():
            self.st.flat = self.st.flat.astype(np.complex128)
        self.st.flat += a * xx.reshape(-1, order="F")
        return self

    def norm(self):
        return float(np.linalg.norm(self.st.flat))


def contract(tensors, out=None):
    keys, letters = {}, iter("abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ")
    counts = {}
    for t in tensors:
        for i in t.inds:
            counts[i] = counts.get(i, 0) + 1
            if i not in keys:
                keys[i] = next(letters)
    free = [i for i in keys if counts[i] == 1] if out is None else list(out)
    spec = ",".join("".join(keys[i] for i in t.inds) for t in tensors) + "->" + "".join(keys[i] for i in free)
    arr = np.einsum(spec, *[t.to_numpy() for t in tensors])
    return NpTensor(_Store(arr, tensors[0].ctx), free)


def inner(a, b):
    bb = b if tuple(b.inds) == tuple(a.inds) else b.permute(a.inds)
    v = np.vdot(a.to_numpy(), bb.to_numpy())
    return v if a.is_complex() else float(np.real(v))


def factorize(T, left, cutoff=0.0, maxdim=None, mindim=1, tags="Link", spectrum=False, complement=False):
    """Keep-everything factorization (the only form qn.py requests): U [left, link],
    C [link, right] from numpy's SVD, the spectrum sigma^2."""
    assert cutoff == 0.0 and maxdim is None and spectrum
    left = [i for i in T.inds if i in left]
    right = [i for i in T.inds if i not in left]
    a = T.permute(left + right).to_numpy()
    m = int(np.prod([i.dim for i in left]))
    M = a.reshape(m, -1, order="F")
    u, s, vh = np.linalg.svd(M, full_matrices=False)
    k = len(s)
    link = Index(k, tags)
    U = NpTensor(_Store(u.reshape([i.dim for i in left] + [k], order="F"), T.ctx), left + [link])
    Cm = (s[:, None] * vh).reshape([k] + [i.dim for i in right], order="F")
    C = NpTensor(_Store(Cm, T.ctx), [link] + right)
    return U, C, dict(newdim=k, truncerr=0.0, spectrum=s ** 2)


@contextlib.contextmanager
def numpy_backend():
    """Route qn.py's device calls to the stand-ins above for the duration."""
    saved = (qn.DTensor, qn.contract, qn.inner, qn.factorize)
    qn.DTensor, qn.contract, qn.inner, qn.factorize = NpTensor, contract, inner, factorize
    try:
        yield FakeCtx()
    finally:
        qn.DTensor, qn.contract, qn.inner, qn.factorize = saved
