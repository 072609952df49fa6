"""The oracle's Breit integrals (rci90: BESSEL, ZKF, RKINT, SKINT, BRRA,
BRINTF, TRIANGBREIT1/2, GENINTBREIT1/2) against facts that follow from the
reference's formulas, on hydrogenic orbitals and on GRASP's He orbitals
with the energies of their rwfn file:

- BRRA's type 4 is RKINT(RAC..) + RKINT(RBD..): swapping the pairs (a, b)
  and (c, d) swaps the two terms, so the value is the same to the bit;
- at zero frequency (WFACT = 0) every Bessel factor is zero and type 1's
  four RKINT terms reduce to type 4's two, each twice: type 1 = type 4 to
  rounding, and type 5 = 2 RKINT(RAC..);
- the frequency-dependent integrals tend to the zero-frequency ones as
  WFACT -> 0;
- GENINTBREIT's tables hold, per k, the TRIANGBREIT-admitted indices in the
  reference's loop order (INDTP ascending within each k, which BRINT1/2's
  binary search needs) and the BRINTF values of those indices."""
import numpy as np

from tests import grasp_examples as G
from tests.common import hydrogenic_case, oracle_for


def _hyd():
    case = hydrogenic_case(nmax=3, lmax=2, z=10.0)
    o = oracle_for(case)
    nw = len(case["orb"].nak)
    e = -np.linspace(50.0, 1.0, nw)
    return o, nw, e


def test_type4_pair_swap_is_exact(oracle_mod):
    o, nw, e = _hyd()
    for (a, b, c, d, k) in [(1, 2, 3, 4, 1), (2, 5, 4, 6, 2), (3, 3, 7, 8, 1)]:
        assert o.brintf(4, a, b, c, d, k, 1.0, e) == o.brintf(4, c, d, a, b, k, 1.0, e)


def test_zero_frequency_limits(oracle_mod):
    o, nw, e = _hyd()
    for (a, b, c, d, k) in [(1, 2, 3, 4, 1), (2, 5, 4, 6, 2), (2, 3, 5, 7, 1)]:
        t1 = o.brintf(1, a, b, c, d, k, 0.0, e)
        t4 = o.brintf(4, a, b, c, d, k, 0.0, e)
        assert abs(t1 - t4) <= 1e-14 * abs(t4), (t1, t4)
        # and the frequency-dependent value approaches it
        near = o.brintf(1, a, b, c, d, k, 1e-4, e)
        far = o.brintf(1, a, b, c, d, k, 1.0, e)
        assert abs(near - t1) < abs(far - t1) or far == t1


def test_tables_follow_the_reference_loops(oracle_mod):
    o, nw, e = _hyd()
    key = nw + 1
    for itype in (1, 2):
        ind, val, kst, j2max = o.genintbreit(itype, 1.0, e, nthreads=4)
        assert kst[0] == 1 and kst[-1] == ind.size + 1 and np.all(np.diff(kst) >= 0)
        for k in range(j2max + 1):
            blk = ind[kst[k] - 1:kst[k + 1] - 1]
            assert np.all(np.diff(blk) > 0)
        rng = np.random.default_rng(itype)
        for pos in rng.choice(ind.size, 25, replace=False):
            k = int(np.searchsorted(kst, pos + 1, side="right") - 1)
            x = int(ind[pos])
            d = x % key; x //= key
            c = x % key; x //= key
            b = x % key; a = x // key
            assert val[pos] == o.brintf(itype, a, b, c, d, k, 1.0, e)


def test_grasp_orbitals_all_types(oracle_mod):
    """The six BRINTF types on GRASP's He orbitals with their energies:
    finite, and type 4 symmetric to the bit."""
    d = G.load("He", oracle_mod)
    o = oracle_mod.Oracle(n=d["n"], rnt=d["rnt"], h=d["h"], c=d["c"], zz=d["zz"])
    o.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    for t in range(1, 7):
        v = o.brintf(t, 1, 2, 3, 4, 2, 1.0, d["e"])
        assert np.isfinite(v)
    assert o.brintf(4, 1, 5, 3, 7, 1, 1.0, d["e"]) == o.brintf(4, 3, 7, 1, 5, 1, 1.0, d["e"])
