"""gg_ypot / gg_xpot (rmcdhf's YPOT and XPOT, rmcdhf90/ypot.f90:35-49,
xpot.f90:31-54) on GRASP's own orbitals (He: 220-point grid, 36 subshells;
Ge II: Fermi nucleus, 590 points) against the oracle's YPOT and XPOT for the
same coefficient lists: the device builds every YZK function of the list on
all N points and combines them in the list's order, so the potentials agree
to rounding (bar: 1e-14 of the largest |value|). Labels outside the orbital
set are errors."""
import numpy as np
import pytest

from tests import grasp_examples as G
from tests.test_potentials import KEY, _lists

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("run", ["He", "Ge"])
def test_potentials_match_oracle(gpu_ready, oracle_mod, run):
    from grasp_gb300 import Context, GGError
    d = G.load(run, oracle_mod)
    ctx = Context(0)
    ctx.set_grid(d["n"], d["rnt"], d["h"], d["c"], d["zz"])
    ctx.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    o = oracle_mod.Oracle(n=d["n"], rnt=d["rnt"], h=d["h"], c=d["c"], zz=d["zz"])
    o.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    nw = len(d["nak"])
    # 1500 terms take XPOT's two-pass form (products by all SMs, then the
    # per-point sums in list order)
    for seed, nt in ((4, 60), (5, 60), (6, 1500)):
        k, a, b, io, nya, nxa, co = _lists(nw, n=nt, seed=seed)
        yp, yp0 = ctx.ypot(nya, co), o.ypot(nya, co)
        assert np.abs(yp - yp0).max() <= 1e-14 * np.abs(yp0).max(), np.abs(yp - yp0).max()
        (xp, xq), (xp0, xq0) = ctx.xpot(nxa, co), o.xpot(nxa, co)
        assert np.abs(xp - xp0).max() <= 1e-14 * np.abs(xp0).max()
        assert np.abs(xq - xq0).max() <= 1e-14 * np.abs(xq0).max()
    # an empty list: YP = ZZ, XP = XQ = 0
    np.testing.assert_array_equal(ctx.ypot(np.zeros(0, np.int32), np.zeros(0)), d["zz"][:d["n"]])
    with pytest.raises(GGError):
        ctx.ypot(np.array([(1 * KEY + (nw + 1)) * KEY], np.int32), np.ones(1))
    with pytest.raises(GGError):
        ctx.xpot(np.array([((1 * KEY + 1) * KEY + 1) * KEY + 21], np.int32), np.ones(1))  # K above 20


def _ctx_oracle(run, oracle_mod):
    from grasp_gb300 import Context
    d = G.load(run, oracle_mod)
    ctx = Context(0)
    ctx.set_grid(d["n"], d["rnt"], d["h"], d["c"], d["zz"])
    ctx.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    o = oracle_mod.Oracle(n=d["n"], rnt=d["rnt"], h=d["h"], c=d["c"], zz=d["zz"])
    o.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    return d, ctx, o


@pytest.mark.parametrize("run", ["He", "Ge"])
def test_cofpot_matches_oracle(gpu_ready, oracle_mod, run):
    """COFPOT's device part (YPOT, XPOT, LAGCON, DACON) against the oracle's."""
    from tests.test_lagrange import _cofs, same_kappa_pairs
    d, ctx, o = _ctx_oracle(run, oracle_mod)
    nw = len(d["nak"])
    cofs = _cofs(nw, 21)
    iecc = same_kappa_pairs(d["nak"], 10, 3)
    ecv = np.random.default_rng(8).normal(size=iecc.size)
    for j in sorted({int(c) % KEY for c in iecc} | {1}):
        yp, xp, xq = ctx.cofpot(j, 1.25, cofs[j - 1], iecc, ecv)
        yp0, xp0, xq0 = o.cofpot(j, 1.25, cofs[j - 1], iecc, ecv)
        for a, b in ((yp, yp0), (xp, xp0), (xq, xq0)):
            assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max(), (j, np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("run", ["He", "Ge"])
def test_setlag_matches_oracle(gpu_ready, oracle_mod, run):
    """SETLAG's multipliers (every case: M fixed, J fixed, occupations apart,
    close occupations) against the oracle's, which follows the reference's
    loop over pairs."""
    from grasp_gb300 import GGError
    from tests.test_lagrange import _cofs, same_kappa_pairs
    d, ctx, o = _ctx_oracle(run, oracle_mod)
    nw = len(d["nak"])
    cofs = _cofs(nw, 31)
    iecc = same_kappa_pairs(d["nak"], 16, 4)
    rng = np.random.default_rng(6)
    cases = set()
    for trial in range(3):
        ucf = rng.uniform(0.5, 2.0, nw)
        if trial == 2:
            ucf[:] = 1.0 + rng.uniform(0, 0.05, nw)  # every pair within 10 %
        lfix = (rng.random(nw) < (0.0 if trial else 0.3)).astype(np.int32)
        ecv = ctx.setlag(iecc, ucf, lfix, cofs)
        ecv0 = o.setlag(iecc, ucf, lfix, cofs)
        scale = max(1.0, np.abs(ecv0).max())
        assert np.abs(ecv - ecv0).max() <= 1e-12 * scale, (trial, np.abs(ecv - ecv0).max() / scale)
        for c in iecc:
            m, j = int(c) // KEY, int(c) % KEY
            if lfix[m - 1]:
                cases.add(0)
            elif lfix[j - 1]:
                cases.add(1)
            else:
                cases.add(2 if abs(ucf[j - 1] - ucf[m - 1]) / max(ucf[j - 1], ucf[m - 1]) > 0.1 else 3)
    assert cases == {0, 1, 2, 3}, cases
    # a pair of orbitals with different kappa: RINTI's error
    bad = [(i, j) for j in range(2, nw + 1) for i in range(1, j) if d["nak"][i - 1] != d["nak"][j - 1]][0]
    with pytest.raises(GGError):
        ctx.setlag(np.array([bad[0] + KEY * bad[1]], np.int32), np.ones(nw), np.zeros(nw, np.int32), cofs)


def test_setlag_long_and_short_lists_match_oracle(gpu_ready, oracle_mod):
    """SETLAG where some orbitals' XPOT lists are long (600 to 1,100 terms:
    the joint two-pass rounds over several orbitals) and the others short
    (one joint launch), with YPOT lists of every length modulo the
    prefetch depth, and DACON terms on every orbital: the multipliers equal
    the oracle's (bar 1e-12 of the largest)."""
    from tests.test_lagrange import same_kappa_pairs
    d, ctx, o = _ctx_oracle("Ge", oracle_mod)
    nw = len(d["nak"])
    cofs = []
    for j in range(1, nw + 1):
        nx = 600 + 37 * j if j % 3 == 0 else 5 + j
        ny = 3 + 5 * j
        _, _, _, _, _, nxa, cx = _lists(nw, n=nx, seed=200 + j)
        _, _, _, _, nya, _, cy = _lists(nw, n=ny, seed=300 + j)
        rng = np.random.default_rng(400 + j)
        cofs.append(dict(nya=nya, ya=cy, nxa=nxa, xa=cx, nda=rng.integers(1, nw + 1, 2),
                         da=rng.normal(size=2) * 0.1))
    assert sum(len(c["nxa"]) >= 512 for c in cofs) >= 2
    iecc = same_kappa_pairs(d["nak"], 12, 9)
    ucf = np.random.default_rng(10).uniform(0.5, 2.0, nw)
    lfix = np.zeros(nw, np.int32)
    ecv = ctx.setlag(iecc, ucf, lfix, cofs)
    ecv0 = o.setlag(iecc, ucf, lfix, cofs)
    scale = max(1.0, np.abs(ecv0).max())
    assert np.abs(ecv - ecv0).max() <= 1e-12 * scale, np.abs(ecv - ecv0).max() / scale
    # COFPOT of a long-list orbital with LAGCON terms through the same path
    j = 3
    ecv1 = np.random.default_rng(11).normal(size=iecc.size)
    got = ctx.cofpot(j, 1.25, cofs[j - 1], iecc, ecv1)
    ref = o.cofpot(j, 1.25, cofs[j - 1], iecc, ecv1)
    for a, b in zip(got, ref):
        assert np.abs(a - b).max() <= 1e-14 * max(1e-300, np.abs(b).max())


@pytest.mark.parametrize("run", ["He", "Ge"])
def test_three_pass_y_build_equals_one_pass(gpu_ready, oracle_mod, run):
    """The Y functions of the three-pass build (k_yincr, k_ychain_sum,
    k_yassemble: lists of 32 or more distinct functions) equal the one-pass
    k_ychain's (a single function) to the bit: YPOT over 48 distinct
    functions whose coefficients are zero but one equals YPOT of that one
    term alone, for functions with k = 0 (b = d: the asymptote 1; b != d)
    and k > 0."""
    d, ctx, o = _ctx_oracle(run, oracle_mod)
    nw = len(d["nak"])
    rng = np.random.default_rng(12)
    keys = {(0, 1, 1), (0, 2, 2), (0, 1, 2), (2, 1, 3), (5, 2, nw)}
    while len(keys) < 48:
        keys.add((int(rng.integers(0, 6)), int(rng.integers(1, nw + 1)), int(rng.integers(1, nw + 1))))
    keys = sorted(keys)
    nya = np.array([(b * KEY + a) * KEY + k for k, a, b in keys], np.int32)
    for t in [keys.index(x) for x in ((0, 1, 1), (0, 2, 2), (0, 1, 2), (2, 1, 3), (5, 2, nw))] + [7, 30, 47]:
        co = np.zeros(len(keys))
        co[t] = 1.7
        np.testing.assert_array_equal(ctx.ypot(nya, co), ctx.ypot(nya[t:t + 1], co[t:t + 1]), err_msg=str(keys[t]))
