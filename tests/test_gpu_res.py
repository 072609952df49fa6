"""rci restarted from rci.res: the stored rows (rci's element filter applied
to an assembled block) read back, loaded as rci's MANEIG loads them
(diagonal shifted by EAV, rci90/maneig.f90:318-330) into a device matrix,
and solved on the GPU. Bar: eigenvalues within 1e-9 Eh and eigenvectors
within 1e-7 after the sign fix of the oracle's MANEIG on the same rows."""
import numpy as np
import pytest

from grasp_gb300 import formats as F
from tests.common import hydrogenic_case, ne7_block, oracle_for

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_res_restart_maneig(gpu_ready, oracle_mod, tmp_path, precision):
    from grasp_gb300 import Context, HMatrix
    _, blk = ne7_block()
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    o = oracle_for(case)
    o.genintrk()
    emt = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    iendc, irow, emtf = F.rci_filter(blk.iendc, blk.irow, emt)
    hd = F.ResHeader(nelec=4, ncf=blk.ncf, nw=0, z=10.0, emn=20.18, parm=np.zeros(0), zz=case["zz"].copy(), nnuc=1,
                     c=case["c"], lfordr=False, iccut=[0], ltrans=False, wfact=1e-6, lvp=False, lnms=False, lsms=False,
                     rnt=case["rnt"], h=case["h"], hp=0.0, r=np.zeros(case["zz"].size + 10),
                     rp=np.zeros(case["zz"].size + 10), rpor=np.zeros(case["zz"].size + 10), orbitals=[])
    F.write_res(tmp_path / "rci.res", hd, [F.ResBlock(blk.ncf, 0, iendc, irow, emtf, elsto=-1.25)])
    _, (b,) = F.read_res(tmp_path / "rci.res")
    eav = F.res_eav(b)
    i2, r2, e2 = F.res_to_hmat(b, eav)
    ctx = Context(0)
    H = HMatrix(ctx, b.ncf, i2, r2)
    H.set_emt(e2)
    np.testing.assert_array_equal(H.emt(), e2)
    nvec = 3
    ev, vec, info = H.maneig(nvec, flavour=0, precision=precision)
    ev0, vec0, _ = oracle_mod.maneig(0, b.ncf, nvec, i2, r2, e2)
    assert info["ierr"] == 0
    assert np.abs(ev - ev0).max() <= 1e-9, (ev, ev0)
    assert np.abs(vec - vec0).max() <= 1e-7
