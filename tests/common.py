"""Shared fixtures-in-code: seeded orbital sets and CI blocks for the tests."""
import numpy as np

from inputs import synth as S

CVAC = S.CVAC


def hydrogenic_case(nmax=3, lmax=2, z=10.0, seed=None, c=CVAC, kappa_max=None, sigma=None):
    """Orbitals n <= nmax, l <= lmax as screened hydrogenic spinors at Z - sigma.
    sigma: None -> SCREENPAR with the 1s as core; 'random' -> U[0, Z-1] seeded."""
    orbs = S.orbital_set(nmax, lmax, kappa_max)
    n = S.NNNP
    rnt, r = S.grid(n, z)
    if isinstance(sigma, str) and sigma == "random":
        rng = np.random.default_rng(seed)
        sig = rng.uniform(0.0, z - 1.0, size=len(orbs))
    elif sigma is None:
        sig = S.screenpar([k for _, k in orbs], 1)
    else:
        sig = np.asarray(sigma, dtype=float)
    orb = S.hydrogenic_orbitals(orbs, z, sig, r, n=n, c=c)
    return dict(orbs=orbs, n=n, rnt=rnt, h=0.05, c=c, z=z, zz=np.full(n, float(z)), orb=orb)


def oracle_for(case):
    import oracle
    o = oracle.Oracle(n=case["n"], rnt=case["rnt"], h=case["h"], c=case["c"], zz=case["zz"])
    ob = case["orb"]
    o.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    return o


def ne7_block(max_ncf=0, density=0.0, seed=3):
    """Be-like Ne VII, J = 0 even: 1s2 2s2 and 1s2 2p2 with SD into n <= 4, l <= 3
    (1s active, which gives the 200-400 CSF size of that workload)."""
    orbs = S.orbital_set(4, 3)

    def occ(d):
        return S.occupation(orbs, d)
    refs = [occ({(1, -1): 2, (2, -1): 2}), occ({(1, -1): 2, (2, 1): 2}), occ({(1, -1): 2, (2, 1): 1, (2, -2): 1}),
            occ({(1, -1): 2, (2, -2): 2})]
    frozen = [0] * len(orbs)
    return orbs, S.ci_block(orbs, refs, frozen, two_j=0, parity=0, max_ncf=max_ncf, density=density, seed=seed)
