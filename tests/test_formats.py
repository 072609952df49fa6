"""GRASP file formats (grasp_gb300/formats.py): round trips of mcp.30/31/32+k,
rwfn and .cm, and checks against the reference's own example data
(src/appl/rhfszeeman95/examples: rwfn and mixing files written by GRASP runs,
and their text summaries), copied into tests/golden/grasp_examples by
tests/golden/copy_grasp_examples.py.

The reference-data checks also pin the oracle's grid and quadrature on
orbitals GRASP produced: RADGRD reproduces the stored grid, QUAD finds the
orbitals normalised, and the moments <r^-1>, <r>, <r^2> agree with the
values the reference printed (6 digits)."""
import glob
import os
import re

import numpy as np
import pytest

from grasp_gb300 import formats as F
from tests.common import hydrogenic_case, ne7_block, oracle_for

REF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "grasp_examples")
ref_data = pytest.mark.skipif(not os.path.isdir(REF), reason="GRASP example data not present")


def test_mcp_round_trip_and_setham(tmp_path, oracle_mod):
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    _, blk = ne7_block()
    s = F.McpSet(ncore=0, nelec=4, ncf=blk.ncf, nw=case["orb"].nw, kmaxf=len(blk.vlists) - 1, idblk=["  0+    "],
                 blocks=[F.McpBlock(blk.ncf, blk.iendc, blk.irow, blk.tlist, list(blk.vlists))])
    head = str(tmp_path / "mcp")
    F.write_mcp(head, s)
    assert sorted(os.listdir(tmp_path)) == sorted(f"mcp.{k}" for k in range(30, 33 + s.kmaxf))
    r = F.read_mcp(head)
    assert (r.ncore, r.nelec, r.nw, r.kmaxf, r.idblk) == (0, 4, s.nw, s.kmaxf, s.idblk)
    b = r.blocks[0]
    np.testing.assert_array_equal(b.iendc, blk.iendc)
    np.testing.assert_array_equal(b.irow, blk.irow)
    for got, want in zip([b.tlist] + b.vlists, [blk.tlist] + list(blk.vlists)):
        for key in ("lab", "start", "loc", "coeff"):
            np.testing.assert_array_equal(got[key], want[key])
    # SETHAM from the lists read back is the SETHAM of the originals
    o = oracle_for(case)
    o.genintrk()
    e0 = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    e1 = o.setham(b.ncf, int(b.iendc[-1]), b.iendc, blk.iq, b.tlist, b.vlists)
    np.testing.assert_array_equal(e0, e1)


def test_mcp_record_framing(tmp_path):
    """Each record is framed by its byte length (int32) on both sides."""
    p = tmp_path / "x.bin"
    with F.FortranFile(p, "wb") as ff:
        ff.write_record(np.array([1, 2, 3], "<i4"))
    raw = p.read_bytes()
    assert raw[:4] == (12).to_bytes(4, "little") and raw[-4:] == (12).to_bytes(4, "little") and len(raw) == 20


def test_rwfn_round_trip(tmp_path):
    case = hydrogenic_case(nmax=2, lmax=1, z=10.0)
    ob = case["orb"]
    r = np.arange(case["n"]) * 0.01
    orbs = [F.Orbital(n, k, -e, 1.5, ob.pf[j, :ob.mf[j]], ob.qf[j, :ob.mf[j]], r[:ob.mf[j]])
            for j, ((n, k), e) in enumerate(zip(case["orbs"], ob.e))]
    F.write_rwfn(tmp_path / "w", orbs)
    back = F.read_rwfn(tmp_path / "w")
    assert [(o.np, o.nak, o.e, o.pz) for o in back] == [(o.np, o.nak, o.e, o.pz) for o in orbs]
    for a, b in zip(back, orbs):
        np.testing.assert_array_equal(a.p, b.p)
        np.testing.assert_array_equal(a.q, b.q)


def test_mix_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    blocks = [F.MixBlock(1, 5, 2, 1, -1, np.array([1, 2], np.int32), -3.5, np.array([-1.0, -0.5]),
                         rng.normal(size=(5, 2))),
              F.MixBlock(2, 3, 0, 999, 999, np.zeros(0, np.int32), 0.0, np.zeros(0), np.zeros((3, 0)))]
    m = F.MixFile(2, 8, 4, 2, 5, blocks)
    F.write_mix(tmp_path / "cm", m)
    back = F.read_mix(tmp_path / "cm")
    assert (back.nelec, back.ncftot, back.nw, back.nvectot, back.nvecsiz) == (2, 8, 4, 2, 5)
    np.testing.assert_array_equal(back.blocks[0].evec, blocks[0].evec)
    assert back.blocks[0].eav == -3.5 and back.blocks[1].nvec == 0


def _grid_from_rwfn(orbs):
    r = max((o.r for o in orbs), key=len)
    h = round(float(np.log(r[2] / r[1] - 1.0)), 10)   # the run's H, printed with 13 digits
    rnt = r[1] / (np.exp(h) - 1.0)
    return r, h, rnt


@ref_data
@pytest.mark.parametrize("name", ["data_He/3Pn6", "data_Ge/2Fn5"])
def test_reference_rwfn_grid_and_norms(oracle_mod, name):
    orbs = F.read_rwfn(f"{REF}/{name}.w")
    r, h, rnt = _grid_from_rwfn(orbs)
    n = len(r)
    o = oracle_mod.Oracle(n=n, rnt=rnt, h=h, zz=np.ones(n))
    R, RP, _ = o.grid()
    assert np.max(np.abs(R[1:n] - r[1:]) / r[1:]) < 1e-13       # RADGRD
    for orb in orbs:
        my = orb.p.size
        ta = np.zeros(n + 10)
        ta[:my] = RP[:my] * (orb.p ** 2 + orb.q ** 2)
        assert abs(o.quad(ta, my) - 1.0) < 1e-12                # QUAD: GRASP's orbitals are normalised


@ref_data
def test_reference_rwfn_moments_match_summary(oracle_mod):
    name = "data_He/3Pn6"
    orbs = F.read_rwfn(f"{REF}/{name}.w")
    r, h, rnt = _grid_from_rwfn(orbs)
    n = len(r)
    o = oracle_mod.Oracle(n=n, rnt=rnt, h=h, zz=np.ones(n))
    R, RP, _ = o.grid()
    text = open(f"{REF}/{name}.sum").read()
    block = text.split("Generalised")[1].split("Eigenenergies")[0]
    rows = re.findall(r"^\s+(\d+[a-z]-?)\s+(\S+)\s+(\S+)\s+(\S+)\s+\S+$", block, re.M)
    assert len(rows) == len(orbs)
    for orb, (lab, m1, p1, p2) in zip(orbs, rows):
        my = orb.p.size
        rho = orb.p ** 2 + orb.q ** 2
        got = []
        for k in (-1, 1, 2):
            ta = np.zeros(n + 10)
            ta[:my] = RP[:my] * rho * R[:my] ** k if k > 0 else 0.0
            if k < 0:
                ta[1:my] = RP[1:my] * rho[1:] / R[1:my]
            got.append(o.quad(ta, my))
        want = [float(x.replace("D", "E")) for x in (m1, p1, p2)]
        for g, w in zip(got, want):
            assert abs(g - w) <= 6e-6 * abs(w), (lab, got, want)


@ref_data
@pytest.mark.parametrize("name", ["data_He/3Pn6", "data_Ge/2Fn5"])
def test_reference_mix_energies_match_summary(name):
    """EAV + EVAL of the rci mixing file equal the energies rci printed in
    its summary (.csum, one 'Eigenenergies' table per block)."""
    m = F.read_mix(f"{REF}/{name}.cm")
    text = open(f"{REF}/{name}.csum").read()
    hartrees = []
    for part in text.split("Eigenenergies:")[1:]:
        hartrees += [float(x.replace("D", "E")) for x in
                     re.findall(r"^\s+\d+\s+\S+\s+[+-]\s+(\S+)", part.split("Weights")[0], re.M)]
    mine = [b.eav + e for b in m.blocks for e in b.eval]
    # the summary also prints excitation energies and a combined table:
    # every level of the mixing file must appear among its numbers
    for e in mine:
        assert min(abs(e - h) for h in hartrees) <= 1e-11, (e, hartrees)
    for b in m.blocks:
        np.testing.assert_allclose(np.linalg.norm(b.evec, axis=0), 1.0, atol=1e-12)


@ref_data
def test_reference_files_round_trip_bytes(tmp_path):
    """Reading then writing a GRASP-written file gives back the same bytes."""
    for path in sorted(glob.glob(f"{REF}/data_*/*.w")) + sorted(glob.glob(f"{REF}/data_*/*.cm")):
        out = tmp_path / os.path.basename(path)
        if path.endswith(".w"):
            F.write_rwfn(out, F.read_rwfn(path))
        else:
            F.write_mix(out, F.read_mix(path))
        assert out.read_bytes() == open(path, "rb").read(), path


# ---------------------------------------------------------------------------
# rci.res
# ---------------------------------------------------------------------------

def _res_header(case, nblock, nw):
    n = case["n"]
    ob = case["orb"]
    pad = np.linspace(1.0, 2.0, 10)
    r = np.concatenate([np.exp(np.arange(n) * case["h"]) - 1.0, pad])
    orbs = [F.ResOrbital(-float(ob.e[j]), 1.0, 2.5 + j, ob.pf[j, :ob.mf[j]].copy(), ob.qf[j, :ob.mf[j]].copy())
            for j in range(nw)]
    return F.ResHeader(nelec=4, ncf=0, nw=nw, z=10.0, emn=20.18, parm=np.array([2.9, 0.52]), zz=case["zz"][:n].copy(),
                       nnuc=1, c=case["c"], lfordr=False, iccut=[0] * nblock, ltrans=False, wfact=1e-6, lvp=False,
                       lnms=False, lsms=False, rnt=case["rnt"], h=case["h"], hp=0.0, r=r, rp=r + 1.0, rpor=r * 0.5,
                       orbitals=orbs)


def _row_loop_filter(iendc, irow, emt, cutoff):
    """rci90/setham_gg.f90:364-368, row by row: an element is stored if it is
    on the diagonal or |ELEMNT| > CUTOFF."""
    out_iendc, out_irow, out_emt = [0], [], []
    for ic in range(1, iendc.size):
        for p in range(iendc[ic - 1], iendc[ic]):
            if irow[p] == ic or abs(emt[p]) > cutoff:
                out_irow.append(irow[p])
                out_emt.append(emt[p])
        out_iendc.append(len(out_irow))
    return np.array(out_iendc, np.int64), np.array(out_irow, np.int32), np.array(out_emt)


def test_rci_filter_matches_row_loop(oracle_mod):
    """The element filter on an assembled Ne VII block with planted small
    elements: exactly CUTOFF (dropped), just above it (kept), tiny negative
    values, zeros, and a zero diagonal (always kept). Bit-exact."""
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    _, blk = ne7_block()
    o = oracle_for(case)
    o.genintrk()
    emt = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    rng = np.random.default_rng(5)
    off = np.setdiff1d(np.arange(blk.nnz), blk.iendc[1:] - 1)
    pick = rng.choice(off, size=min(40, off.size), replace=False)
    emt[pick[:8]] = F.RCI_CUTOFF
    emt[pick[8:16]] = -F.RCI_CUTOFF
    emt[pick[16:24]] = np.nextafter(F.RCI_CUTOFF, 1.0)
    emt[pick[24:32]] = -3e-13
    emt[pick[32:]] = 0.0
    emt[blk.iendc[3] - 1] = 0.0
    got = F.rci_filter(blk.iendc, blk.irow, emt)
    want = _row_loop_filter(np.asarray(blk.iendc), np.asarray(blk.irow), emt, F.RCI_CUTOFF)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)
    assert got[0][-1] == blk.nnz - np.count_nonzero(np.abs(emt[off]) <= F.RCI_CUTOFF)
    assert np.count_nonzero(np.abs(emt[off]) <= F.RCI_CUTOFF) >= 8 + 8 + 8 + len(pick[32:])
    # every row keeps its diagonal, last
    assert np.all(got[1][got[0][1:] - 1] == np.arange(1, blk.ncf + 1))
    assert np.count_nonzero(np.abs(got[2][np.setdiff1d(np.arange(got[0][-1]), got[0][1:] - 1)]) <= F.RCI_CUTOFF) == 0


def test_res_round_trip_and_record_layout(tmp_path, oracle_mod):
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    _, blk = ne7_block()
    o = oracle_for(case)
    o.genintrk()
    emt = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    iendc, irow, emtf = F.rci_filter(blk.iendc, blk.irow, emt)
    hd = _res_header(case, 2, case["orb"].nw)
    hd.ncf = blk.ncf + 3
    small = F.ResBlock(3, 0, np.array([0, 1, 3, 6], np.int64), np.array([1, 1, 2, 1, 2, 3], np.int32),
                       np.array([-1.0, 0.5, -2.0, 0.25, 0.125, -3.0]), elsto=-7.5)
    blocks = [F.ResBlock(blk.ncf, 0, iendc, irow, emtf, elsto=-7.5), small]
    p = tmp_path / "rci.res"
    F.write_res(p, hd, blocks)
    hd2, back = F.read_res(p)
    for key in ("nelec", "ncf", "nw", "z", "emn", "nnuc", "c", "lfordr", "iccut", "ltrans", "wfact", "lvp", "lnms",
                "lsms", "rnt", "h", "hp"):
        assert getattr(hd2, key) == getattr(hd, key), key
    for key in ("parm", "zz", "r", "rp", "rpor"):
        np.testing.assert_array_equal(getattr(hd2, key), getattr(hd, key))
    for a, b in zip(hd2.orbitals, hd.orbitals):
        assert (a.e, a.gama, a.pz) == (b.e, b.gama, b.pz)
        np.testing.assert_array_equal(a.p, b.p)
        np.testing.assert_array_equal(a.q, b.q)
    for a, b in zip(back, blocks):
        assert (a.ncf, a.iccut, a.myid, a.nprocs, a.elsto) == (b.ncf, b.iccut, b.myid, b.nprocs, b.elsto)
        np.testing.assert_array_equal(a.iendc, b.iendc)
        np.testing.assert_array_equal(a.irow, b.irow)
        np.testing.assert_array_equal(a.emt, b.emt)
    # the bytes of the file again, and the small block's records at its end:
    # (NCF, ICCUT, MYID, NPROCS), then (NELC, ELSTO, EMT(1:NELC), IROW(1:NELC)) per row
    F.write_res(tmp_path / "again", hd2, back)
    raw = p.read_bytes()
    assert (tmp_path / "again").read_bytes() == raw
    row3 = (np.array([3], "<i4").tobytes() + np.array([-7.5, 0.25, 0.125, -3.0], "<f8").tobytes()
            + np.array([1, 2, 3], "<i4").tobytes())
    framed = len(row3).to_bytes(4, "little") + row3 + len(row3).to_bytes(4, "little")
    assert raw.endswith(framed)
    head = np.array([3, 0, 0, 1], "<i4").tobytes()
    assert (len(head).to_bytes(4, "little") + head + len(head).to_bytes(4, "little")) in raw


def test_res_eav_and_shifted_matrix(oracle_mod):
    """EAV = diagonal mean + ELSTO (rci90/genmat2.f90:36) and the in-core
    matrix with its diagonal shifted by EAV (rci90/maneig.f90:318-330): its
    eigenvalues + EAV are those of the unfiltered H + ELSTO to rounding (the
    dropped elements are at most 1e-12 each)."""
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    _, blk = ne7_block()
    o = oracle_for(case)
    o.genintrk()
    emt = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    iendc, irow, emtf = F.rci_filter(blk.iendc, blk.irow, emt)
    b = F.ResBlock(blk.ncf, 0, iendc, irow, emtf, elsto=-2.0)
    eav = F.res_eav(b)
    diag = emt[np.asarray(blk.iendc)[1:] - 1]
    assert eav == pytest.approx(diag.mean() - 2.0, abs=1e-12)
    i2, r2, e2 = F.res_to_hmat(b, eav)

    def dense(iendc_, irow_, v):
        a = np.zeros((blk.ncf, blk.ncf))
        for ic in range(blk.ncf):
            for p in range(iendc_[ic], iendc_[ic + 1]):
                a[ic, irow_[p] - 1] = a[irow_[p] - 1, ic] = v[p]
        return a

    w_shift = np.linalg.eigvalsh(dense(i2, r2, e2))[:5] + eav + b.elsto  # rci90/matrix.f90:197-201
    w_full = np.linalg.eigvalsh(dense(np.asarray(blk.iendc), np.asarray(blk.irow), emt))[:5] - 2.0
    assert np.abs(w_shift - w_full).max() <= 1e-10
    with pytest.raises(ValueError):
        F.res_to_hmat(F.ResBlock(3, 0, np.array([0, 1], np.int64), np.array([1], np.int32), np.array([1.0])), 0.0)


def test_res_rank_rows_and_interrupted_file(tmp_path):
    """Rows per rank (rci90/genmat.f90:97-98) and a file that ends inside a
    block's rows, as an interrupted rci run leaves it: the rows present are
    read and the block is short."""
    assert [F.res_rows(10, r, 3) for r in range(3)] == [4, 3, 3]
    # fewer CSFs than ranks: each rank wrote the rows of its own stride only
    assert [F.res_rows(2, r, 4) for r in range(4)] == [1, 1, 0, 0]
    case = hydrogenic_case(nmax=2, lmax=1, z=10.0)
    hd = _res_header(case, 1, case["orb"].nw)
    iendc = np.array([0, 1, 3, 5, 8], np.int64)
    irow = np.array([1, 1, 2, 2, 3, 1, 3, 4], np.int32)
    emt = np.arange(1.0, 9.0)
    p = tmp_path / "rci.res"
    F.write_res(p, hd, [F.ResBlock(4, 0, iendc, irow, emt)])
    raw = p.read_bytes()
    last = 4 + 4 + 8 + 3 * 12 + 4
    (tmp_path / "cut.res").write_bytes(raw[:-last])
    _, blocks = F.read_res(tmp_path / "cut.res")
    np.testing.assert_array_equal(blocks[0].iendc, iendc[:4])
    np.testing.assert_array_equal(blocks[0].emt, emt[:5])
    with pytest.raises(ValueError):
        F.write_res(tmp_path / "x", hd, [F.ResBlock(4, 0, iendc, irow, emt, myid=1, nprocs=2)])


def test_mcp_two_blocks_with_empty_lists(tmp_path):
    """Two blocks, the second with no T contributions and an empty V^1 list
    (only the (0, 0) terminator record): everything reads back, and a file
    whose blocks are out of order is rejected as MATRX rejects it."""
    def lst(labs, sizes, seed):
        rng = np.random.default_rng(seed)
        start = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        return dict(lab=np.array(labs, np.int32), start=start,
                    loc=rng.integers(1, 6, size=start[-1]).astype(np.int32), coeff=rng.normal(size=start[-1]),
                    iclmn=rng.integers(1, 4, size=start[-1]).astype(np.int32))
    empty = lst([], [], 0)
    b1 = F.McpBlock(3, np.array([0, 1, 3, 6], np.int64), np.array([1, 1, 2, 1, 2, 3], np.int32),
                    lst([216, 217], [2, 3], 1), [lst([46226 * 215 + 216], [4], 2), lst([216 * 46225 + 217], [1], 3)])
    b2 = F.McpBlock(2, np.array([0, 1, 3], np.int64), np.array([1, 1, 2], np.int32), empty,
                    [lst([46226 * 215 + 216], [2], 4), empty])
    s = F.McpSet(ncore=1, nelec=2, ncf=5, nw=2, kmaxf=1, idblk=["  1/2-  ", "  3/2-  "], blocks=[b1, b2])
    head = str(tmp_path / "m")
    F.write_mcp(head, s)
    r = F.read_mcp(head)
    assert [b.ncf for b in r.blocks] == [3, 2] and r.idblk == s.idblk and r.ncore == 1
    for got, want in zip(r.blocks, s.blocks):
        np.testing.assert_array_equal(got.iendc, want.iendc)
        np.testing.assert_array_equal(got.irow, want.irow)
        for g, w in zip([got.tlist] + got.vlists, [want.tlist] + want.vlists):
            for key in ("lab", "start", "loc", "coeff", "iclmn"):
                np.testing.assert_array_equal(g[key], w[key])
    assert r.blocks[1].tlist["lab"].size == 0 and r.blocks[1].vlists[1]["start"].tolist() == [0]
    s.blocks = [b2, b1]
    s.idblk = s.idblk[::-1]
    F.write_mcp(head, s)
    raw = bytearray(open(f"{head}.30", "rb").read())
    # renumber the first structure block as block 2: MATRX's consistency check
    i = raw.find(b"MCP" + np.array([1, 2], "<i4").tobytes())
    assert i > 0
    raw[i + 3:i + 7] = np.array([2], "<i4").tobytes()
    open(f"{head}.30", "wb").write(bytes(raw))
    with pytest.raises(ValueError):
        F.read_mcp(head)


def test_res_merge_ranks(tmp_path):
    """rci.res files of a 3-rank run (rows dealt round-robin, as rci_mpi
    writes them) merge into the single-rank block; a missing rank or a
    short rank file is an error."""
    rng = np.random.default_rng(11)
    ncf, nprocs = 10, 3
    lens = rng.integers(1, 5, size=ncf)
    lens = np.minimum(lens, np.arange(1, ncf + 1))
    iendc = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    irow = np.concatenate([np.concatenate([np.sort(rng.choice(np.arange(1, i + 1), n - 1, replace=False)), [i + 1]])
                           if n > 1 else [i + 1] for i, n in enumerate(lens)]).astype(np.int32)
    emt = rng.normal(size=iendc[-1])
    full = F.ResBlock(ncf, 0, iendc, irow, emt, elsto=-0.5)
    case = hydrogenic_case(nmax=2, lmax=1, z=10.0)
    parts = []
    for r in range(nprocs):
        rows = range(r, ncf, nprocs)
        sub_i = np.concatenate([[0], np.cumsum([lens[i] for i in rows])]).astype(np.int64)
        sub_r = np.concatenate([irow[iendc[i]:iendc[i + 1]] for i in rows])
        sub_e = np.concatenate([emt[iendc[i]:iendc[i + 1]] for i in rows])
        p = tmp_path / f"rci{r}.res"
        F.write_res(p, _res_header(case, 1, case["orb"].nw), [F.ResBlock(ncf, 0, sub_i, sub_r, sub_e, -0.5, r, nprocs)])
        parts.append(F.read_res(p)[1][0])
    m = F.merge_res_ranks(parts[::-1])
    np.testing.assert_array_equal(m.iendc, full.iendc)
    np.testing.assert_array_equal(m.irow, full.irow)
    np.testing.assert_array_equal(m.emt, full.emt)
    assert (m.myid, m.nprocs, m.elsto) == (0, 1, -0.5)
    with pytest.raises(ValueError):
        F.merge_res_ranks(parts[:2])
    short = F.ResBlock(ncf, 0, parts[1].iendc[:-1], parts[1].irow, parts[1].emt, -0.5, 1, nprocs)
    with pytest.raises(ValueError):
        F.merge_res_ranks([parts[0], short, parts[2]])


def _random_lower_rows(rng, ncf):
    lens = np.minimum(rng.integers(1, 5, size=ncf), np.arange(1, ncf + 1))
    iendc = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    irow = np.concatenate([np.concatenate([np.sort(rng.choice(np.arange(1, i + 1), n - 1, replace=False)), [i + 1]])
                           if n > 1 else [i + 1] for i, n in enumerate(lens)]).astype(np.int32)
    return iendc, irow, rng.normal(size=iendc[-1])


def _rank_rows(iendc, irow, emt, r, nprocs):
    rows = list(range(r, iendc.size - 1, nprocs))
    sub_i = np.concatenate([[0], np.cumsum([iendc[i + 1] - iendc[i] for i in rows])]).astype(np.int64)
    sub_r = np.concatenate([irow[iendc[i]:iendc[i + 1]] for i in rows] + [np.zeros(0, np.int32)]).astype(np.int32)
    sub_e = np.concatenate([emt[iendc[i]:iendc[i + 1]] for i in rows] + [np.zeros(0)])
    return sub_i, sub_r, sub_e


def test_res_block_with_fewer_csfs_than_ranks(tmp_path):
    """A 2-CSF block between two larger ones, written by 3 ranks: rank 2
    owns no row of it (setham_gg.f90:160 deals rows MYID+1, MYID+1+NPROCS,
    ...). Every rank's file reads back block by block (the small block does
    not swallow the next block's header record) and the blocks merge."""
    rng = np.random.default_rng(5)
    sizes, nprocs = [10, 2, 7], 3
    blocks = [_random_lower_rows(rng, n) for n in sizes]
    case = hydrogenic_case(nmax=2, lmax=1, z=10.0)
    hd = _res_header(case, len(sizes), case["orb"].nw)
    read = []
    for r in range(nprocs):
        p = tmp_path / f"rci{r}.res"
        F.write_res(p, hd, [F.ResBlock(n, 0, *_rank_rows(*blk, r, nprocs), 0.25, r, nprocs)
                            for n, blk in zip(sizes, blocks)])
        _, got = F.read_res(p)
        assert [b.ncf for b in got] == sizes
        assert [b.iendc.size - 1 for b in got] == [len(range(r, n, nprocs)) for n in sizes]
        read.append(got)
    for j, (iendc, irow, emt) in enumerate(blocks):
        m = F.merge_res_ranks([read[r][j] for r in range(nprocs)])
        np.testing.assert_array_equal(m.iendc, iendc)
        np.testing.assert_array_equal(m.irow, irow)
        np.testing.assert_array_equal(m.emt, emt)
