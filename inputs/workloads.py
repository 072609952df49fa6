"""Named, seeded synthetic workloads with the shapes of the CI-stage benchmarks.

Every workload is: a 590-point log grid (RNT = 2e-6/Z, H = 0.05), screened
hydrogenic Dirac orbitals (DCBSRW at Z - sigma, SCREENPAR screening), and a
CI block from :func:`inputs.synth.ci_block` (CSF occupations, mcp.30
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
  large The large-scale CI workload: Ni-like Z = 40 orbital set (n <= 7,
        l <= 5: 47 orbitals, R^k to k = 10) and a seeded synthetic symmetric
        H of ~3e5 CSFs with ~1e9 stored lower-triangle elements (sorted
        configuration-like diagonal, small random couplings, uniform random
        structure), 5 roots. The Hamiltonian is generated directly (no T/V
        lists: at this size they would be ~2.4e9 contributions), so it
        exercises the tables and the eigensolver, not SETHAM.
  batch The ne7 expansion for every ion Z = 10..40 (31 ions) and every
        2J = 0, 2, 4, 6, 8 of both parities: 310 blocks of 321-1007 CSFs
        (7,027 CSFs and 1.04 M stored elements per ion), 3 roots each. The
        angular lists depend on the CSFs only, so each (J, parity) block's
        T/V lists are generated once and assembled with every ion's orbitals.
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


@dataclass
class LargeWorkload:
    """Orbitals for the R^k table and a lower-triangle-by-rows H (IENDC,
    1-based IROW with the diagonal last in each row, EMT)."""
    name: str
    z: float
    orbs: list
    n: int
    rnt: float
    h: float
    c: float
    zz: np.ndarray
    orb: S.Orbitals
    ncf: int
    iendc: np.ndarray
    irow: np.ndarray
    emt: np.ndarray
    nroots: int
    kmax: int

    @property
    def nnz(self):
        return int(self.iendc[-1])

    def describe(self):
        return dict(workload=self.name, z=self.z, norb=len(self.orbs), kmax=self.kmax, grid_points=self.n,
                    ncf=self.ncf, nnz=self.nnz, density=round(2.0 * self.nnz / (self.ncf * (self.ncf + 1.0)), 5),
                    nroots=self.nroots, hamiltonian="synthetic (seeded), no T/V lists")


def synthetic_h(ncf, nnz, seed=7):
    """Seeded symmetric H in GRASP's lower-triangle-by-rows storage with about
    ``nnz`` stored elements (gs_synthetic_h, inputs/grasp_synth.h): each
    column below the diagonal of row r is present with the same probability;
    diagonal -1000 + 30 sqrt(r / ncf) Eh (sorted, like configuration
    energies) plus N(0, 1e-3), off-diagonal elements N(0, 2e-3) Eh."""
    from .synth import _d, _i32, _i64, ptr
    from .synth import check as check_synth
    p = 2.0 * max(nnz - ncf, 0) / (ncf * (ncf - 1.0))
    iendc = np.zeros(ncf + 1, np.int64)
    lib = S.lib()
    check_synth(lib.gs_synthetic_h(ncf, p, seed, ptr(iendc, _i64), None, None))
    irow = np.empty(int(iendc[-1]), np.int32)
    emt = np.empty(int(iendc[-1]), np.float64)
    check_synth(lib.gs_synthetic_h(ncf, p, seed, ptr(iendc, _i64), ptr(irow, _i32), ptr(emt, _d)))
    return iendc, irow, emt


def large(ncf=300000, nnz=1.0e9, seed=7, nroots=5):
    orbs = S.orbital_set(7, 5)
    z = 40.0
    n, rnt, ob = _orbitals(orbs, z, S.screenpar([k for _, k in orbs], 4))  # n <= 2 core: 1s, 2s, 2p-, 2p
    iendc, irow, emt = synthetic_h(ncf, int(nnz), seed=seed)
    return LargeWorkload(f"ni_like_z40_j1o_{ncf}csf_synthetic", z, orbs, n, rnt, 0.05, S.CVAC, np.full(n, z), ob,
                         ncf, iendc, irow, emt, nroots, 10)


@dataclass
class BatchWorkload:
    name: str
    zs: list
    orbs: list
    blocks: list        # [(two_j, parity, CIBlock)] shared by every ion
    nroots: int

    def describe(self):
        ncf = [b.ncf for _, _, b in self.blocks]
        return dict(workload=self.name, ions=len(self.zs), blocks=len(self.zs) * len(self.blocks),
                    ncf_min=min(ncf), ncf_max=max(ncf), ncf_total=len(self.zs) * sum(ncf),
                    nnz_total=len(self.zs) * sum(b.nnz for _, _, b in self.blocks), nroots=self.nroots)

    def ion(self, z):
        """(n, rnt, orbitals) of ion Z on its own grid (RNT = 2e-6/Z)."""
        return _orbitals(self.orbs, float(z), S.screenpar([k for _, k in self.orbs], 1))


def batch(zs=tuple(range(10, 41)), two_js=(0, 2, 4, 6, 8), parities=(0, 1), max_ncf=0, seed=3, nroots=3):
    orbs = S.orbital_set(4, 3)

    def occ(d):
        return S.occupation(orbs, d)
    refs = [occ({(1, -1): 2, (2, -1): 2}), occ({(1, -1): 2, (2, 1): 2}), occ({(1, -1): 2, (2, 1): 1, (2, -2): 1}),
            occ({(1, -1): 2, (2, -2): 2})]
    blocks = []
    for par in parities:
        for tj in two_js:
            blocks.append((tj, par, S.ci_block(orbs, refs, [0] * len(orbs), two_j=tj, parity=par, max_ncf=max_ncf,
                                               seed=seed)))
    return BatchWorkload(f"ne_like_{len(zs)}ions_{len(zs) * len(blocks)}blocks", list(zs), orbs, blocks, nroots)


def assemble_batch(w, ctx, precision=0):
    """All blocks of all ions on one context: per ion the grid, orbitals,
    R^k (GG_FP64 or the tensor cores) and I(ab) tables, then SETHAM of each
    block. The first ion uploads each block's structure and T/V lists; the
    other ions' blocks are views of them (gg_hmat_create_view), which share
    the lists and the assembly plan. Returns the HMatrix objects in
    (ion, block) order."""
    from grasp_gb300 import HMatrix
    hs, first = [], []
    for iz, z in enumerate(w.zs):
        n, rnt, ob = w.ion(z)
        ctx.set_grid(n, rnt, 0.05, S.CVAC, np.full(n, float(z)))
        ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
        ctx.genintrk(precision=precision)
        ctx.iabint_table()
        for j, (_, _, b) in enumerate(w.blocks):
            if iz == 0:
                H = HMatrix(ctx, b.ncf, b.iendc, b.irow)
                H.setham(b.iq, b.tlist, b.vlists)
                first.append(H)
            else:
                H = HMatrix.view(first[j], ctx)
                H.setham_assemble()
            hs.append(H)
    return hs
