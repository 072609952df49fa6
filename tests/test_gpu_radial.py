"""GPU parity: grid, R^k table (GENINTRK), SLATER, RKINTC, RINTI, I(ab) table
against the CPU oracle on identical inputs.

Tolerances: the R^k contraction sums in a different order than QUAD (tiled
FP64 GEMM), so R^k agrees to <= 1e-12 relative with an absolute floor of
1e-14 (integrals whose value is below the floor are compared absolutely).
Single SLATER/RINTI evaluations follow the reference's sequential sums and
agree to 1e-14 relative (they differ only through log() in QUAD's head).
Index tables (INDTEIRK, KSTART) are bit-exact.
"""
import numpy as np
import pytest

from tests.common import hydrogenic_case, oracle_for

pytestmark = pytest.mark.gpu

RK_RTOL, RK_ATOL = 1e-12, 1e-14


def gpu_ctx(case):
    from grasp_gb300 import Context
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ob = case["orb"]
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    return ctx


def test_grid_bit_exact(gpu_ready, oracle_mod):
    case = hydrogenic_case(nmax=2, lmax=1, z=10.0)
    o = oracle_for(case)
    ctx = gpu_ctx(case)
    for a, b in zip(o.grid(), ctx.grid()):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("nmax,lmax,z,sig", [(3, 2, 10.0, None), (4, 3, 10.0, None), (5, 3, 26.0, "random")])
def test_genintrk_parity(gpu_ready, oracle_mod, nmax, lmax, z, sig):
    case = hydrogenic_case(nmax=nmax, lmax=lmax, z=z, sigma=sig, seed=7)
    o = oracle_for(case)
    ind0, val0, ks0, j20 = o.genintrk(nthreads=8)
    ctx = gpu_ctx(case)
    n, j2 = ctx.genintrk()
    ind, val, ks = ctx.rk_table()
    assert j2 == j20 and n == len(ind0)
    np.testing.assert_array_equal(ind, ind0)
    np.testing.assert_array_equal(ks, ks0)
    err = np.abs(val - val0)
    bad = err > RK_RTOL * np.abs(val0) + RK_ATOL
    assert not bad.any(), (int(bad.sum()), float(err.max()), val0[bad][:5], val[bad][:5])


def test_genintrk_kmax8_40orbitals(gpu_ready, oracle_mod):
    """The R^k table workload: n <= 7, |kappa| <= 4 (40 orbitals), Z = 26,
    seeded screening U[0, Z-1], k = 0..8."""
    case = hydrogenic_case(nmax=7, lmax=4, z=26.0, sigma="random", seed=2024, kappa_max=4)
    assert len(case["orbs"]) == 40
    o = oracle_for(case)
    ind0, val0, ks0, _ = o.genintrk(kmax=8, nthreads=16)
    ctx = gpu_ctx(case)
    n, _ = ctx.genintrk(kmax=8)
    # entries whose QUAD head index is above 2 take the warp-parallel general
    # QUAD (k_quad_table); this workload has thousands of them
    assert ctx.stage_stat(20) > 1000
    ind, val, ks = ctx.rk_table()
    np.testing.assert_array_equal(ind, ind0)
    err = np.abs(val - val0)
    rel = err / np.maximum(np.abs(val0), RK_ATOL / RK_RTOL)
    assert rel.max() <= RK_RTOL, (float(rel.max()), int(np.argmax(rel)))


@pytest.mark.parametrize("nmax,lmax,z,sig,kmax,kapmax", [(4, 3, 10.0, None, -1, None),
                                                         (5, 3, 26.0, "random", -1, None),
                                                         (7, 4, 26.0, "random", 8, 4)])
def test_genintrk_tensor_core_split(gpu_ready, oracle_mod, nmax, lmax, z, sig, kmax, kapmax):
    """GG_SPLIT: the contraction on int8 slices with int32 tensor-core sums
    (Ozaki split, 10 slices of 7 bits per row) meets the same bar as FP64:
    <= 1e-12 relative with a 1e-14 absolute floor; indices bit-exact."""
    case = hydrogenic_case(nmax=nmax, lmax=lmax, z=z, sigma=sig, seed=2024, kappa_max=kapmax)
    o = oracle_for(case)
    ind0, val0, ks0, _ = o.genintrk(kmax=kmax, nthreads=16)
    ctx = gpu_ctx(case)
    ctx.genintrk(kmax=kmax, precision=1)
    ind, val, ks = ctx.rk_table()
    np.testing.assert_array_equal(ind, ind0)
    np.testing.assert_array_equal(ks, ks0)
    err = np.abs(val - val0)
    bad = err > RK_RTOL * np.abs(val0) + RK_ATOL
    assert not bad.any(), (int(bad.sum()), float((err / np.maximum(np.abs(val0), 1e-300)).max()))


def test_slater_rkintc_rinti(gpu_ready, oracle_mod):
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    o = oracle_for(case)
    ctx = gpu_ctx(case)
    ctx.genintrk()
    ind, val, ks = ctx.rk_table()
    key = case["orb"].nw + 1
    rng = np.random.default_rng(5)
    for t in rng.integers(0, len(ind), size=25):
        k = int(np.searchsorted(ks, t + 1, side="right") - 1)
        p = int(ind[t])
        a, b, c, d = p // key ** 3, (p // key ** 2) % key, (p // key) % key, p % key
        s_gpu = ctx.slater(a, b, c, d, k)
        s_cpu = o.slater(a, b, c, d, k)
        assert abs(s_gpu - s_cpu) <= 1e-14 * abs(s_cpu) + 1e-16
        assert ctx.rkintc(c, d, a, b, k) == val[t]
    nw = case["orb"].nw
    nak = case["orb"].nak
    tab = ctx.iabint_table()
    for j in range(1, nw + 1):
        for k in range(1, nw + 1):
            if nak[j - 1] != nak[k - 1]:
                assert np.isnan(tab[j - 1, k - 1])
                continue
            ref = o.rinti(j, k, 0)
            assert abs(tab[j - 1, k - 1] - ref) <= 1e-13 * abs(ref) + 1e-15
            assert abs(ctx.rinti(j, k, 0) - ref) <= 1e-13 * abs(ref) + 1e-15
    from grasp_gb300 import GGError
    with pytest.raises(GGError):
        ctx.rinti(1, 3)  # 1s / 2p-: different kappa (rinti.f90:48-51 STOPs)
    with pytest.raises(GGError):
        ctx.rkintc(1, 1, 1, 3, 0)  # not in the table (rkintc.f90 STOPs)


def test_genintrk_structure_reused_and_rebuilt(gpu_ready, oracle_mod):
    """gg_genintrk keeps its index structure between calls: the same orbital
    set with other radial functions reuses it, another set rebuilds it. Every
    table, FP64 and tensor-core, matches the oracle."""
    from grasp_gb300 import Context
    cases = [hydrogenic_case(nmax=4, lmax=3, z=10.0),
             hydrogenic_case(nmax=4, lmax=3, z=26.0, sigma="random", seed=3),  # same set, other functions
             hydrogenic_case(nmax=3, lmax=2, z=10.0),                          # another set
             hydrogenic_case(nmax=4, lmax=3, z=10.0)]
    ctx = Context(0)
    for case in cases:
        ob = case["orb"]
        ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
        ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
        ind0, val0, ks0, _ = oracle_for(case).genintrk(nthreads=8)
        for precision in (0, 1):
            ctx.genintrk(precision=precision)
            ind, val, ks = ctx.rk_table()
            np.testing.assert_array_equal(ind, ind0)
            np.testing.assert_array_equal(ks, ks0)
            rel = np.abs(val - val0) / np.maximum(np.abs(val0), RK_ATOL / RK_RTOL)
            assert rel.max() <= RK_RTOL, (precision, float(rel.max()))
