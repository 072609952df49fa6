"""gg_slater_noalloc: the SLATER entry point for callers that cannot allocate
device memory when they need an integral. It must give gg_slater's result
while allocating nothing; its working arrays live in one fixed device array.

Collected last on purpose: it runs after every other test in a full run, and
also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from tests.common import hydrogenic_case

pytestmark = pytest.mark.gpu


def test_slater_noalloc_matches_slater_twice(gpu_ready):
    from grasp_gb300 import Context, _lib
    case = hydrogenic_case(nmax=4, lmax=3, z=26.0, sigma="random", seed=17)
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ob = case["orb"]
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    lib = _lib.gpu()
    # two different integrals in a row (k = 0 with b = d, then an exchange-type k = 2)
    idx = {o: j + 1 for j, o in enumerate(case["orbs"])}
    calls = [(idx[(2, -1)], idx[(3, -2)], idx[(2, -1)], idx[(3, -2)], 0),
             (idx[(1, -1)], idx[(3, 2)], idx[(3, 2)], idx[(1, -1)], 2)]
    refs = [ctx.slater(a, b, c, d, k) for a, b, c, d, k in calls]
    # the property the entry point exists for: the library makes no device
    # (or pinned host) allocation during these calls, the first included
    allocs = lib.gg_alloc_count()
    for (a, b, c, d, k), ref in zip(calls, refs):
        v = C.c_double(np.nan)
        st = lib.gg_slater_noalloc(ctx._h, a, b, c, d, k, C.byref(v))
        assert st == 0, lib.gg_last_error()
        assert abs(v.value - ref) <= 1e-14 * abs(ref) + 1e-16, (a, b, c, d, k, v.value, ref)
    assert lib.gg_alloc_count() == allocs
    # a grid beyond the fixed scratch is rejected with a clear error
    big = Context(0)
    n = 2100
    big.set_grid(n, 2.0e-6, 0.05 * 590 / n, case["c"], np.full(n, 26.0))
    pf = np.zeros((1, n)); qf = np.zeros((1, n))
    pf[0, 1:100] = 1e-3; qf[0, 1:100] = 1e-5
    big.set_orbitals([-1], [99], pf, qf)
    v = C.c_double()
    st = lib.gg_slater_noalloc(big._h, 1, 1, 1, 1, 0, C.byref(v))
    assert st != 0 and b"exceeds the fixed scratch" in lib.gg_last_error()
