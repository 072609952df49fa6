"""The oracle's COFPOT tail and SETLAG (rmcdhf90/cofpot.f90:30-33,
lagcon.f90, dacon.f90, setlag.f90) on GRASP's He orbitals, against facts
that follow from their definitions:

- with no LAGCON and no DACON terms COFPOT's potentials are YPOT's and
  XPOT's, bit for bit;
- LAGCON adds WA R(I) QF(I,M) to XP and subtracts WA R(I) PF(I,M) from XQ,
  WA = ECV / (UCF(J) C), for the pairs containing J; a weight below
  0.01 ACCY is skipped;
- DACON is linear in its coefficients;
- SETLAG with empty lists (YP = ZZ, XP = XQ = 0) and orbital M fixed gives
  ECV = (int RPOR (P_M P_J + Q_M Q_J) ZZ - RINTI(M,J,1)) UCF(J), which is
  -I(M,J) UCF(J) with I = RINTI(M,J,0) (its nuclear piece is that integral);
- a pair's ECV does not depend on the pairs before it."""
import numpy as np

from tests import grasp_examples as G
from tests.test_potentials import KEY, _lists


def _setup(oracle_mod):
    d = G.load("He", oracle_mod)
    o = oracle_mod.Oracle(n=d["n"], rnt=d["rnt"], h=d["h"], c=d["c"], zz=d["zz"])
    o.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    return d, o


def _cofs(nw, seed):
    out = []
    for j in range(nw):
        _, _, _, _, nya, nxa, co = _lists(nw, n=8, seed=seed + j)
        rng = np.random.default_rng(seed + 100 + j)
        out.append(dict(nya=nya, ya=co, nxa=nxa, xa=co[::-1].copy(), nda=rng.integers(1, nw + 1, 3),
                        da=rng.normal(size=3) * 0.1))
    return out


def same_kappa_pairs(nak, count, seed):
    rng = np.random.default_rng(seed)
    nw = len(nak)
    pairs = [(i, j) for j in range(2, nw + 1) for i in range(1, j) if nak[i - 1] == nak[j - 1]]
    pick = rng.choice(len(pairs), size=min(count, len(pairs)), replace=False)
    return np.array([pairs[p][0] + KEY * pairs[p][1] for p in sorted(pick)], np.int32)


def test_cofpot_without_extra_terms_is_ypot_xpot(oracle_mod):
    d, o = _setup(oracle_mod)
    nw = len(d["nak"])
    cof = _cofs(nw, 3)[4]
    plain = dict(nya=cof["nya"], ya=cof["ya"], nxa=cof["nxa"], xa=cof["xa"])
    yp, xp, xq = o.cofpot(5, 1.7, plain)
    np.testing.assert_array_equal(yp, o.ypot(cof["nya"], cof["ya"]))
    xp0, xq0 = o.xpot(cof["nxa"], cof["xa"])
    np.testing.assert_array_equal(xp, xp0)
    np.testing.assert_array_equal(xq, xq0)


def test_lagcon_term(oracle_mod):
    d, o = _setup(oracle_mod)
    j, m, ucf = 3, 7, 1.5
    iecc = np.array([j + KEY * m, 1 + KEY * 2], np.int32)  # the second pair does not contain j
    ecv = np.array([0.25, 9.0])
    _, xp0, xq0 = o.cofpot(j, ucf, {})
    _, xp, xq = o.cofpot(j, ucf, {}, iecc, ecv)
    n = d["n"]
    wa = ecv[0] * (1.0 / (ucf * d["c"]))
    r = o.grid()[0][:n]
    mf = d["mf"][m - 1]
    exp_p = np.where(np.arange(1, n + 1) <= mf, wa * r * d["qf"][m - 1, :n], 0.0)
    exp_q = np.where(np.arange(1, n + 1) <= mf, -wa * r * d["pf"][m - 1, :n], 0.0)
    assert np.abs((xp - xp0) - exp_p).max() <= 1e-14 * np.abs(exp_p).max()
    assert np.abs((xq - xq0) - exp_q).max() <= 1e-14 * np.abs(exp_q).max()
    # a weight below 0.01 ACCY is skipped
    _, xp2, _ = o.cofpot(j, ucf, {}, iecc[:1], np.array([1e-30]))
    np.testing.assert_array_equal(xp2, xp0)


def test_dacon_is_linear(oracle_mod):
    d, o = _setup(oracle_mod)
    base = dict(nda=np.array([4], np.int32))
    _, xp0, xq0 = o.cofpot(4, 1.0, dict(base, da=[0.0]))
    _, xp1, xq1 = o.cofpot(4, 1.0, dict(base, da=[1.0]))
    _, xp3, xq3 = o.cofpot(4, 1.0, dict(base, da=[3.0]))
    assert np.abs((xp3 - xp0) - 3 * (xp1 - xp0)).max() <= 1e-13 * np.abs(xp1 - xp0).max()
    assert np.abs((xq3 - xq0) - 3 * (xq1 - xq0)).max() <= 1e-13 * np.abs(xq1 - xq0).max()
    assert np.abs(xp1 - xp0).max() > 0


def test_setlag_with_empty_lists_is_minus_iab(oracle_mod):
    d, o = _setup(oracle_mod)
    nw = len(d["nak"])
    iecc = same_kappa_pairs(d["nak"], 6, 1)
    ucf = np.linspace(1.0, 2.0, nw)
    lfix = np.ones(nw, np.int32)  # every M fixed: the first case
    ecv = o.setlag(iecc, ucf, lfix, [{} for _ in range(nw)])
    for k, code in enumerate(iecc):
        m, j = int(code) // KEY, int(code) % KEY
        expect = -o.rinti(m, j, 0) * ucf[j - 1]
        assert abs(ecv[k] - expect) <= 1e-12 * max(1.0, abs(expect)), (j, m, ecv[k], expect)


def test_setlag_pairs_are_independent(oracle_mod):
    d, o = _setup(oracle_mod)
    nw = len(d["nak"])
    cofs = _cofs(nw, 11)
    iecc = same_kappa_pairs(d["nak"], 8, 2)
    rng = np.random.default_rng(5)
    ucf = rng.uniform(0.5, 2.0, nw)
    lfix = (rng.random(nw) < 0.3).astype(np.int32)
    ecv = o.setlag(iecc, ucf, lfix, cofs)
    for k in range(len(iecc)):
        one = o.setlag(iecc[k:k + 1], ucf, lfix, cofs)
        assert one[0] == ecv[k]
