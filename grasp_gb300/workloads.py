"""Named, seeded synthetic workloads with the shapes of the CI-stage benchmarks.

Every workload is: a 590-point log grid (RNT = 2e-6/Z, H = 0.05), screened
hydrogenic Dirac orbitals (DCBSRW at Z - sigma, SCREENPAR screening), and a
CI block from :func:`grasp_gb300.synth.ci_block` (CSF occupations, mcp.30
structure, T/V lists with seeded coefficients).

Sizes versus the workload descriptions they stand in for:
  ne7   Be-like Ne VII, J = 0 even, refs 1s2 2s2 / 1s2 2p2, SD into n <= 4,
        l <= 3. With 1s kept closed this space has only 26 J = 0 CSFs; the
        described 200-400 CSFs are reached with 1s active (361 CSFs), which is
        what this workload uses.
  fe15  Mg-like Fe XV, J = 0 even, refs 1s2 2s2 2p6 {3s2, 3p2, 3d2}, SD into
        n <= 6, l <= 4 (34 orbitals). With n <= 2 inactive only two
        electrons move (68 CSFs); the described 30k-60k CSFs are reached with
        2s 2p active and 1s inactive: 43,493 CSFs. The natural excitation-rank
        structure has 7.5 % density; it is thinned to the described 1-3 %
        (2 % by default).
  rk40  The R^k table workload: n <= 7, |kappa| <= 4 (40 orbitals), Z = 26,
        screening drawn U[0, Z-1] from the seed, k = 0..8.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import synth as S


@dataclass
class Workload:
    name: str
    z: float
    orbs: list
    n: int
    rnt: float
    h: float
    c: float
    zz: np.ndarray
    orb: S.Orbitals
    block: S.CIBlock | None
    nroots: int
    kmax: int = -1

    def describe(self):
        d = dict(workload=self.name, z=self.z, norb=len(self.orbs), grid_points=self.n)
        if self.block is not None:
            b = self.block
            d.update(ncf=b.ncf, nnz=b.nnz, density=round(b.density, 5), contributions=b.ncontr, nroots=self.nroots)
        return d


def _orbitals(orbs, z, sigma):
    n = S.NNNP
    rnt, r = S.grid(n, z)
    ob = S.hydrogenic_orbitals(orbs, z, sigma, r, n=n)
    return n, rnt, ob


def ne7(seed=3):
    orbs = S.orbital_set(4, 3)

    def occ(d):
        return S.occupation(orbs, d)
    refs = [occ({(1, -1): 2, (2, -1): 2}), occ({(1, -1): 2, (2, 1): 2}), occ({(1, -1): 2, (2, 1): 1, (2, -2): 1}),
            occ({(1, -1): 2, (2, -2): 2})]
    blk = S.ci_block(orbs, refs, [0] * len(orbs), two_j=0, parity=0, seed=seed)
    z = 10.0
    n, rnt, ob = _orbitals(orbs, z, S.screenpar([k for _, k in orbs], 1))
    return Workload("ne7_j0e_361csf", z, orbs, n, rnt, 0.05, S.CVAC, np.full(n, z), ob, blk, 3)


def fe15(density=0.02, seed=11):
    orbs = S.orbital_set(6, 4)

    def occ(d):
        return S.occupation(orbs, d)
    core = {(1, -1): 2, (2, -1): 2, (2, 1): 2, (2, -2): 4}
    refs = []
    for v in [{(3, -1): 2}, {(3, 1): 2}, {(3, 1): 1, (3, -2): 1}, {(3, -2): 2}, {(3, 2): 2}, {(3, 2): 1, (3, -3): 1},
              {(3, -3): 2}]:
        d = dict(core)
        d.update(v)
        refs.append(occ(d))
    frozen = [1 if o == (1, -1) else 0 for o in orbs]
    blk = S.ci_block(orbs, refs, frozen, two_j=0, parity=0, kmaxf=9, density=density, seed=seed)
    z = 26.0
    n, rnt, ob = _orbitals(orbs, z, S.screenpar([k for _, k in orbs], 4))
    return Workload("fe15_j0e_43493csf", z, orbs, n, rnt, 0.05, S.CVAC, np.full(n, z), ob, blk, 10)


def rk40(seed=2024):
    orbs = S.orbital_set(7, 4, kappa_max=4)
    z = 26.0
    sig = np.random.default_rng(seed).uniform(0.0, z - 1.0, size=len(orbs))
    n, rnt, ob = _orbitals(orbs, z, sig)
    return Workload("rk_table_40orb_k8", z, orbs, n, rnt, 0.05, S.CVAC, np.full(n, z), ob, None, 0, kmax=8)
