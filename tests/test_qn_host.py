"""Host logic of the U(1) block-sparse (QN) layer (networksolvers_gb300/qn.py): the
global truncation over sectors against the NDTensors rule on the union of the spectra
(oracle), link-charge inference of chain MPOs, and sector enumeration.  No GPU."""
import numpy as np
import pytest

import oracle.linalg as ol
from networksolvers_gb300 import models as m
from networksolvers_gb300 import qn
from networksolvers_gb300.chain import _pad_op


def _spectra(rng):
    nsec = int(rng.integers(1, 7))
    out = []
    for _ in range(nsec):
        k = int(rng.integers(1, 14))
        v = rng.exponential(1.0, k) * 10.0 ** (-rng.uniform(0, 14, k))
        out.append(np.sort(v)[::-1])
    return out


def test_truncate_sectors_is_the_rule_on_the_union():
    rng = np.random.default_rng(3)
    for _ in range(300):
        spectra = _spectra(rng)
        union = np.sort(np.concatenate(spectra))[::-1]
        cutoff = float(10.0 ** -rng.uniform(2, 14))
        maxdim = None if rng.random() < 0.4 else int(rng.integers(1, len(union) + 3))
        mindim = int(rng.integers(1, 4))
        keep, err, vals = qn.truncate_sectors(spectra, cutoff, maxdim, mindim)
        k, e = ol.truncate_spectrum(union, cutoff, maxdim, mindim)
        assert sum(keep) == k
        assert abs(err - e) <= 1e-14 * max(e, 1e-300) + 1e-300
        kept = np.sort(np.concatenate([sp[:kq] for sp, kq in zip(spectra, keep)]))[::-1]
        assert np.array_equal(kept, union[:k]) and np.array_equal(vals, union[:k])


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


@pytest.mark.parametrize("model", ["heisenberg", "xxz", "j1j2", "opsum_fields"])
def test_mpo_link_charges(model):
    n = 10
    H = {"heisenberg": lambda: m.heisenberg_chain(n), "xxz": lambda: m.xxz_chain(n, 1.7),
         "j1j2": lambda: m.j1j2_chain(n, 0.35), "opsum_fields": lambda: _xxz_fields(n, 1.5, 0)}[model]()
    Ws = [_pad_op(H.tensors[j], j, n) for j in range(1, n + 1)]
    sq = qn.site_qns(H)
    assert sq == [1, -1]
    qs, live = qn.infer_link_qns(Ws, sq)
    assert list(qs[0]) == [0] and list(qs[-1]) == [0] and live[-1].all()
    for j, W in enumerate(Ws):
        for a, sp, s, b in np.argwhere(np.abs(W) > 0):
            if live[j][a]:
                assert live[j + 1][b] and qs[j + 1][b] == qs[j][a] + sq[sp] - sq[s]
    # dropping the entries of unreachable states leaves the operator unchanged
    mps = [np.where(live[j][:, None, None, None], W, 0.0) for j, W in enumerate(Ws)]
    def dense(ws):
        t = ws[0][0]
        for W in ws[1:]:
            t = np.einsum("...a,aijb->...ijb", t, W)
        return t
    assert np.array_equal(dense(mps), dense(Ws))


def test_mpo_link_charges_reject_a_transverse_field():
    n = 6
    os = m.OpSum()
    for j in range(1, n):
        os += (1.0, "Sz", j, "Sz", j + 1)
    for j in range(1, n + 1):
        os += (0.3, "Sx", j)
    H = m.chain_mpo(os, n)
    Ws = [_pad_op(H.tensors[j], j, n) for j in range(1, n + 1)]
    with pytest.raises(ValueError):
        qn.infer_link_qns(Ws, qn.site_qns(H))


def test_allowed_sectors_and_index_keys():
    a = qn.QNIndex([(-1, 2), (1, 3)], dir=+1)
    b = qn.QNIndex([(0, 1), (2, 2)], dir=-1)
    combos = qn.allowed_sectors([a, b], -1)
    assert combos == [(0, 0), (1, 1)]
    assert a.prime().key() != a.key() and a.dag().key() == a.key() and a.dag().dir == -1
    assert a.sec(1) == a.dag().sec(1) and a.sec(1).dim == 3 and a.prime().sec(1) != a.sec(1)
