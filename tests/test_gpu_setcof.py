"""SETCOF on the device (gg_setcof_prepare, gg_setcof; rmcdhf90/setcof.f90)
against the oracle's loop-by-loop restatement, on two synthetic Ne VII
blocks (J = 0 even, J = 1 odd), in both DSUBRS modes (EOL: two levels per
block with weights; EAL: CSF weights):

- the three lists' labels are the oracle's, entry for entry (order and the
  merging of labels repeated in the second block);
- the values agree to 1e-14 of the largest: the label sums add the same
  products in the same order on the device;
- COFPOT on the device (gg_cofpot) from those lists equals the oracle's
  COFPOT from its own lists (1e-14), so SETCOF -> YPOT/XPOT/DACON runs on
  the GPU end to end."""
import numpy as np
import pytest

from tests.common import hydrogenic_case, oracle_for
from tests.test_setcof_oracle import _blocks

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("eol", [True, False])
def test_setcof_matches_oracle(gpu_ready, oracle_mod, eol):
    from grasp_gb300 import Context, HMatrix
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    o = oracle_for(case)
    ob = case["orb"]
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    ctx.genintrk()
    ctx.iabint_table()
    orbs, blocks = _blocks(two_js=(0, 2))
    if not eol:
        rng = np.random.default_rng(4)
        blocks = [dict(b, wt=rng.uniform(0.1, 1.0, b["ncf"])) for b in blocks]
    hs = []
    for b in blocks:
        H = HMatrix(ctx, b["ncf"], b["iendc"], b["irow"])
        H.setham_upload(b["iq"], b["tlist"], b["vlists"])
        hs.append(H)
    ctx.setcof_prepare(hs, [b["wt"] for b in blocks], [b["evec"] for b in blocks] if eol else None, eol=eol)
    nw = len(ob.nak)
    for j in range(1, nw + 1):
        ucf = 1.0 + 0.1 * j
        got = ctx.setcof(j, ucf)
        ref = o.setcof(blocks, eol, j, ucf)
        for key in ("nya", "nxa", "nda"):
            np.testing.assert_array_equal(got[key], ref[key])
        for key in ("ya", "xa", "da"):
            scale = max(1e-300, np.abs(ref[key]).max()) if ref[key].size else 1.0
            assert np.abs(got[key] - ref[key]).max(initial=0.0) <= 1e-14 * scale, (j, key)
        if j in (2, 5):
            yp, xp, xq = ctx.cofpot(j, ucf, got)
            yp0, xp0, xq0 = o.cofpot(j, ucf, ref)
            for a, b in ((yp, yp0), (xp, xp0), (xq, xq0)):
                assert np.abs(a - b).max() <= 1e-14 * max(1e-300, np.abs(b).max())


def test_setcof_needs_prepare_and_lists(gpu_ready):
    from grasp_gb300 import Context, GGError, HMatrix
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    ob = case["orb"]
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    with pytest.raises(GGError):
        ctx.setcof(1, 1.0)
    orbs, blocks = _blocks()
    b = blocks[0]
    H = HMatrix(ctx, b["ncf"], b["iendc"], b["irow"])  # no lists uploaded
    with pytest.raises(GGError):
        ctx.setcof_prepare([H], [b["wt"]], [b["evec"]], eol=True)
