"""Generate the committed golden fixtures from the oracle (FP64 CPU restatement) and
scipy exact diagonalisation.  Run from the repository root:
    python tests/golden/make_golden.py
Fixtures:
  c1_heisenberg_n20.npz — config "plain 2-site DMRG, Heisenberg N=20, random MPS χ=10
      seed 0, 5 sweeps, maxdim 64, cutoff 1e-10, krylovdim 3, maxiter 1":
      per-region eigenvalues and kept bond dimensions, final energy, ED ground energy.
  tree_dmrg.npz — the reference's 10-site tree test (test_tree_dmrg.jl): ED energy and
      oracle energies for 2-site and 1-site+densitymatrix.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import networksolvers_gb300.models as m  # noqa: E402
from oracle import sweep, ed  # noqa: E402

OUT = Path(__file__).resolve().parent


def c1():
    H, psi0 = m.config_heisenberg_chain(20, 10, 0)
    rec = []

    def cb(prob, sweep, region, which, **k):
        rec.append((sweep, which, prob.eigenvalue, prob.last_insert.get("newdim", -1)))

    E, psi = sweep.dmrg(H, psi0, nsweeps=5, nsites=2, updater_kwargs=dict(krylovdim=3, maxiter=1),
                        inserter_kwargs=dict(trunc=dict(cutoff=1e-10, maxdim=64)), region_callback=cb)
    Hx = ed.hamiltonian(H.graph.vertices, ed.heisenberg_terms(H.graph.edges))
    Eed = ed.ground_energy(Hx)
    rec = np.array(rec, dtype=np.float64)
    np.savez_compressed(OUT / "c1_heisenberg_n20.npz", sweep=rec[:, 0], which=rec[:, 1], eigenvalue=rec[:, 2],
                        newdim=rec[:, 3], energy=E, ed_energy=Eed,
                        linkdims=np.array([psi.linkdims()[e] for e in H.graph.edges]))
    print("c1", E, Eed)


def tree():
    g = m.build_tree_graph(3, 3)
    H, p0 = m.heisenberg_tree(g), m.neel_state(g)
    Ex = ed.ground_energy(ed.hamiltonian(g.vertices, ed.heisenberg_terms(g.edges)))
    trunc = dict(cutoff=1e-5, maxdim=40)
    E2, _ = sweep.dmrg(H, p0, nsweeps=5, nsites=2, inserter_kwargs=dict(trunc=trunc))
    E1, _ = sweep.dmrg(H, p0, nsweeps=5, nsites=1, extracter_kwargs=dict(trunc=trunc, subspace_algorithm="densitymatrix"),
                       inserter_kwargs=dict(trunc=trunc))
    np.savez_compressed(OUT / "tree_dmrg.npz", ed_energy=Ex, e2=E2, e1=E1)
    print("tree", Ex, E2, E1)


if __name__ == "__main__":
    c1()
    tree()
