"""The oracle's SETCOF (rmcdhf90/setcof.f90) on synthetic Ne VII blocks:

- DSUBRS in EOL mode with every CSF its own level (unit eigenvectors) and
  level weights w is DSUBRS in EAL mode with CSF weights w, operation for
  operation, so the two modes give the same lists to the bit;
- every list value is linear in 1/UCF(J) and quadratic in the mixing
  coefficients (scaling the eigenvectors by 2 scales every value by 4);
- the labels decode to valid orbitals, the DACON orbitals are orbitals
  coupled to J by a one-body label of the block."""
import numpy as np

from tests.common import hydrogenic_case, ne7_block, oracle_for

KEY = 215


def _blocks(two_js=(0,), ncf_max=120):
    from inputs import synth as S
    orbs, b0 = ne7_block(max_ncf=ncf_max)
    out = []
    rng = np.random.default_rng(3)
    for t, tj in enumerate(two_js):
        b = b0 if tj == 0 else S.ci_block(orbs, [S.occupation(orbs, {(1, -1): 2, (2, -1): 1, (2, 1): 1})],
                                          [0] * len(orbs), two_j=tj, parity=1, max_ncf=ncf_max, seed=5)
        ev = rng.normal(size=(b.ncf, 2))
        ev /= np.linalg.norm(ev, axis=0)
        out.append(dict(ncf=b.ncf, iendc=b.iendc, irow=b.irow, iq=b.iq, tlist=b.tlist, vlists=b.vlists,
                        evec=ev, wt=np.array([0.7, 0.3])))
    return orbs, out


def test_eol_unit_levels_equal_eal(oracle_mod):
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    o = oracle_for(case)
    orbs, blocks = _blocks()
    b = blocks[0]
    w = np.random.default_rng(1).uniform(0.1, 1.0, b["ncf"])
    eol = [dict(b, evec=np.eye(b["ncf"]), wt=w)]
    eal = [dict(b, wt=w)]
    for j in (1, 3, 5):
        a = o.setcof(eol, True, j, 1.5)
        c = o.setcof(eal, False, j, 1.5)
        for key in a:
            np.testing.assert_array_equal(a[key], c[key])


def test_scaling_and_labels(oracle_mod):
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    o = oracle_for(case)
    nw = len(case["orb"].nak)
    orbs, blocks = _blocks(two_js=(0, 2))
    j = 3
    base = o.setcof(blocks, True, j, 1.0)
    half = o.setcof(blocks, True, j, 2.0)
    double = o.setcof([dict(b, evec=2 * b["evec"]) for b in blocks], True, j, 1.0)
    for key in ("ya", "xa", "da"):
        assert np.abs(half[key] - base[key] / 2).max() <= 1e-15 * max(1e-300, np.abs(base[key]).max())
        assert np.abs(double[key] - 4 * base[key]).max() <= 1e-14 * max(1e-300, np.abs(base[key]).max())
    for l in base["nya"]:
        k, ab = l % KEY, l // KEY
        assert 1 <= ab % KEY <= nw and 1 <= ab // KEY <= nw and k <= 20
    for l in base["nxa"]:
        x = l // KEY
        assert all(1 <= v <= nw for v in (x % KEY, (x // KEY) % KEY, x // KEY // KEY))
    partners = set()
    for b in blocks:
        for v in b["tlist"]["lab"]:
            a, c = int(v % KEY), int(v // KEY)
            if a == j or c == j:
                partners.add(c if a == j else a)
    assert set(int(v) for v in base["nda"]) <= partners
