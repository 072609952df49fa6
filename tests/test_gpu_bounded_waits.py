"""The bounded device waits of the tensor-core R^k contraction (k_rk_tc):
a tile that never receives its first copy (the copy is withheld through
gg_test_stall_rk_tile, so its barrier is one that nothing completes) must
give up after its poll limit, drain, free its tensor memory and report
GG_ERR_TIMEOUT through the host; no trap, no fault, no hang. The context
then still works: no stale table is used, and the next table is right."""
import numpy as np
import pytest

from tests.common import hydrogenic_case

pytestmark = pytest.mark.gpu


def test_rk_tensor_core_wait_times_out_and_context_recovers(gpu_ready, oracle_mod):
    from grasp_gb300 import SPLIT, Context, GGError, _lib
    case = hydrogenic_case(nmax=5, lmax=3, z=26.0, sigma="random", seed=5)
    ob = case["orb"]
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    o = oracle_mod.Oracle(n=case["n"], rnt=case["rnt"], h=case["h"], c=case["c"], zz=case["zz"])
    o.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    ind0, val0, _, _ = o.genintrk()
    ctx.genintrk(precision=SPLIT)   # a valid table first
    for tile in (0, 3):
        assert _lib.gpu().gg_test_stall_rk_tile(ctx._h, tile) == 0
        with pytest.raises(GGError) as e:
            ctx.genintrk(precision=SPLIT)
        assert e.value.status == -9, e.value
        assert "timed out" in str(e.value) and "drained" in str(e.value)
        # the failed call left no table: a lookup is refused, not answered
        # from the earlier one
        with pytest.raises(GGError):
            ctx.rkintc(1, 1, 1, 1, 0)
        # the hook is one-shot: the next call computes the right table
        n, _ = ctx.genintrk(precision=SPLIT)
        ind, val, _ = ctx.rk_table()
        np.testing.assert_array_equal(ind, ind0)
        assert np.abs(val - val0).max() <= 1e-12 * np.abs(val0).max()
