"""Minimal dense ITensor semantics in numpy (test infrastructure).

Indices carry an id and a prime level; contraction with ``*`` sums over every index
the two tensors share (same id and prime level), as ITensors does.  The result keeps
A's uncontracted indices followed by B's.
"""
from __future__ import annotations

import itertools
import numpy as np

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

    def __eq__(self, other):
        return isinstance(other, Index) and self.key() == other.key()

    def __hash__(self):
        return hash(self.key())

    def __repr__(self):
        return f"Index({self.dim},{self.tags!r},id={self.id}{chr(39) * self.plev})"


class Tensor:
    __slots__ = ("data", "inds")

    def __init__(self, data, inds):
        self.data = np.asarray(data)
        self.inds = tuple(inds)
        assert self.data.ndim == len(self.inds), (self.data.shape, self.inds)
        for k, i in enumerate(self.inds):
            assert self.data.shape[k] == i.dim, (self.data.shape, self.inds)

    # -- index manipulation -------------------------------------------------
    def prime(self, *which):
        if not which:
            return Tensor(self.data, [i.prime() for i in self.inds])
        w = set(which)
        return Tensor(self.data, [i.prime() if i in w else i for i in self.inds])

    def noprime(self):
        return Tensor(self.data, [i.noprime() for i in self.inds])

    def dag(self):
        return Tensor(np.conj(self.data), self.inds)

    def permute(self, inds):
        inds = list(inds)
        perm = [self.inds.index(i) for i in inds]
        return Tensor(self.data.transpose(perm), inds)

    def replaceind(self, old, new):
        return Tensor(self.data, [new if i == old else i for i in self.inds])

    # -- algebra ------------------------------------------------------------
    def __mul__(self, other):
        if np.isscalar(other):
            return Tensor(self.data * other, self.inds)
        common = [i for i in self.inds if i in other.inds]
        ia = [self.inds.index(i) for i in common]
        ib = [other.inds.index(i) for i in common]
        data = np.tensordot(self.data, other.data, axes=(ia, ib))
        inds = [i for i in self.inds if i not in common] + [i for i in other.inds if i not in common]
        return Tensor(data, inds)

    __rmul__ = lambda self, s: self * s

    def __truediv__(self, s):
        return Tensor(self.data / s, self.inds)

    def __add__(self, other):
        o = other.permute(self.inds)
        return Tensor(self.data + o.data, self.inds)

    def __sub__(self, other):
        o = other.permute(self.inds)
        return Tensor(self.data - o.data, self.inds)

    def norm(self):
        return float(np.linalg.norm(self.data.ravel()))

    def scalar(self):
        assert self.data.ndim == 0
        return self.data[()]

    def __repr__(self):
        return f"Tensor{self.data.shape}{list(self.inds)}"


def inner(a: Tensor, b: Tensor):
    """<a|b> with a conjugated; a and b have the same index set."""
    bb = b.permute(a.inds)
    return np.vdot(a.data.ravel(), bb.data.ravel())


def commoninds(a, b):
    return [i for i in a.inds if i in b.inds]


def uniqueinds(a, b):
    return [i for i in a.inds if i not in b.inds]


def commonind(a, b):
    c = commoninds(a, b)
    return c[0] if c else None


def contract(tensors, out=None):
    """Contract a list of tensors over every shared index (einsum with an optimal
    pairwise order, the role of `itn.contract(list; sequence)` in operator_map.jl:7-8).
    Output index order: uncontracted indices in order of first appearance, or `out`."""
    counts = {}
    for t in tensors:
        for i in t.inds:
            counts[i] = counts.get(i, 0) + 1
    lab = {}
    for t in tensors:
        for i in t.inds:
            if i not in lab:
                lab[i] = len(lab)
    free = [i for i in lab if counts[i] == 1]
    if out is not None:
        free = list(out)
    args = []
    for t in tensors:
        args += [t.data, [lab[i] for i in t.inds]]
    args.append([lab[i] for i in free])
    sig = tuple((t.data.shape, tuple(lab[i] for i in t.inds)) for t in tensors) + (
        tuple(lab[i] for i in free),)
    path = _paths.get(sig)
    if path is None:
        path = np.einsum_path(*args, optimize=("optimal", float(2 ** 62)))[0][1:]
        _paths[sig] = path
    # pairwise contractions in the optimal order, each one a BLAS tensordot
    work = list(tensors)
    for pair in path:
        picked = [work[k] for k in pair]
        for k in sorted(pair, reverse=True):
            del work[k]
        t = picked[0]
        for o in picked[1:]:
            t = t * o
        work.append(t)
    t = work[0]
    for o in work[1:]:
        t = t * o
    return t.permute(free)


_paths = {}
