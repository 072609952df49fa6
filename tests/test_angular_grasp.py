"""The angular engine (grasp_gb300.angular, libgraspangular) on GRASP-written
CSF lists, with the oracle's R^k/I(ab) tables, SETHAM and MANEIG on
GRASP's own orbitals: the Dirac-Coulomb energies must be the ones rmcdhf
printed for the same CSF lists and orbitals (tests/golden/grasp_examples),
and for Ge II the mixing coefficients the ones rmcdhf wrote (.m).

This pins the whole chain — radial integrals on GRASP's orbitals, the T/V
lists, SETHAM, the eigensolver — against the reference's own outputs."""
import numpy as np

from grasp_gb300 import angular as A
from grasp_gb300 import formats as F
from tests import grasp_examples as G


def _chain(oracle_mod, run):
    d = G.load(run, oracle_mod)
    csl = F.read_csl(f"{G.ROOT}/{G.RUNS[run]}.c")
    o = oracle_mod.Oracle(n=d["n"], rnt=d["rnt"], h=d["h"], c=d["c"], zz=d["zz"])
    o.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    o.genintrk()
    return d, csl, o


def _solve(oracle_mod, o, ab, nvec):
    emt = o.setham(ab.ncf, ab.nnz, ab.iendc, ab.iq, ab.tlist, ab.vlists)
    eav = oracle_mod.shift_eav(ab.ncf, ab.iendc, emt)
    ev, vec, _ = oracle_mod.maneig(0, ab.ncf, nvec, ab.iendc, ab.irow, emt)
    return eav, ev, vec


def test_csl_reader_blocks():
    he = F.read_csl(f"{G.ROOT}/{G.RUNS['He']}.c")
    assert [(b.two_j, b.parity, b.ncsf) for b in he.blocks] == [(0, -1, 70), (2, -1, 180), (4, -1, 222)]
    ge = F.read_csl(f"{G.ROOT}/{G.RUNS['Ge']}.c")
    assert ge.ncore == 9 and len(ge.subshells) == 25
    assert [(b.two_j, b.parity, b.ncsf) for b in ge.blocks] == [(5, -1, 922), (7, -1, 928)]
    # "4s ( 1)  4p ( 1)  4d ( 1)" with J 1/2 3/2 5/2, X = 1, J = 5/2
    b = ge.blocks[0]
    i4s, i4p, i4d = (ge.labels.index(s) for s in ("4s", "4p", "4d"))
    assert (b.iq[2, i4s], b.iq[2, i4p], b.iq[2, i4d]) == (1, 1, 1)
    assert (b.jqs[2, i4s], b.jqs[2, i4p], b.jqs[2, i4d]) == (1, 3, 5)
    assert (b.xj[2, i4s], b.xj[2, i4p], b.xj[2, i4d]) == (1, 2, 5)


def test_fermi_nucleus_parameters_match_summary():
    """c and a of the Fermi distribution, converted from isodata (fm) with
    the run's constants, are the Bohr-radius values rmcdhf printed."""
    text = open(f"{G.ROOT}/{G.RUNS['Ge']}.sum").read()
    c_pr = float(text.split("c =")[1].split("Bohr")[0].replace("D", "E"))
    a_pr = float(text.split("a =")[1].split("Bohr")[0].replace("D", "E"))
    iso = G.read_isodata(f"{G.ROOT}/data_Ge/isodata")
    fmtoau = 1.0e-13 / G.AINFCM_1986
    assert abs(iso["c_fm"] * fmtoau - c_pr) <= 1e-12 * c_pr
    assert abs(iso["a_fm"] * fmtoau - a_pr) <= 1e-12 * a_pr


def test_he_energies_match_rmcdhf(oracle_mod):
    """He, 472 CSFs in J = 0, 1, 2 odd blocks, 36 subshells up to 6h: the
    four levels rmcdhf optimised, to the 13 digits it printed."""
    d, csl, o = _chain(oracle_mod, "He")
    checked = 0
    for bi, blk in enumerate(csl.blocks):
        levels = [lv for lv in d["levels"] if lv[1] == blk.two_j]
        ab = A.block_lists(csl, bi)
        eav, ev, _ = _solve(oracle_mod, o, ab, max(lv[0] for lv in levels))
        for lv in levels:
            assert abs(eav + ev[lv[0] - 1] - lv[3]) <= 1e-12, (blk.two_j, lv)
            checked += 1
    assert checked == 4


def test_ge_energies_and_mixing_match_rmcdhf(oracle_mod):
    """Ge II, 31 electrons (28 in the core), Fermi nucleus, 1850 CSFs in the
    J = 5/2- and 7/2- blocks: the level energies rmcdhf printed (13
    significant digits), the EAV it wrote, and its mixing coefficients,
    sign included, CSF by CSF."""
    d, csl, o = _chain(oracle_mod, "Ge")
    mix = F.read_mix(f"{G.ROOT}/{G.RUNS['Ge']}.m")
    for bi, blk in enumerate(csl.blocks):
        ab = A.block_lists(csl, bi)
        mb = mix.blocks[bi]
        assert (mb.ncf, mb.two_j_plus_1) == (ab.ncf, blk.two_j + 1)
        eav, ev, vec = _solve(oracle_mod, o, ab, mb.nvec)
        (lv,) = [lv for lv in d["levels"] if lv[1] == blk.two_j]
        assert abs(eav + ev[0] - lv[3]) <= 1e-9, (eav + ev[0], lv)
        assert abs(eav - mb.eav) <= 1e-10
        assert abs(ev[0] - mb.eval[0]) <= 1e-9
        np.testing.assert_allclose(vec[:, 0], mb.evec[:, 0], atol=1e-9)


def test_lists_structure_and_labels(oracle_mod):
    """The block's lists are well formed: IENDC/IROW lower triangle by rows
    with the diagonal last, every LOC inside its row's range, labels sorted
    and decodable (T: kappa_a = kappa_b; V^k: triangle and parity rules),
    and the matrix they assemble is the one the oracle's SETHAM builds from
    them twice in a row (deterministic)."""
    _, csl, o = _chain(oracle_mod, "He")
    ab = A.block_lists(csl, 1)
    nak = [k for _, k in csl.subshells]
    lv = [k if k > 0 else -k - 1 for k in nak]
    rows = np.repeat(np.arange(1, ab.ncf + 1), np.diff(ab.iendc))
    assert np.all(ab.irow <= rows) and np.all(ab.irow[ab.iendc[1:] - 1] == np.arange(1, ab.ncf + 1))
    for i in range(ab.ncf):
        assert np.all(np.diff(ab.irow[ab.iendc[i]:ab.iendc[i + 1]]) > 0)
    for k, lst in enumerate([ab.tlist] + ab.vlists):
        assert np.all(np.diff(lst["lab"]) > 0)
        assert lst["loc"].min() >= 1 and lst["loc"].max() <= ab.nnz
        for lab in lst["lab"]:
            if k == 0:
                a, b = divmod(int(lab), 215)
                assert nak[a - 1] == nak[b - 1]
            else:
                kk = k - 1
                ac, bd = divmod(int(lab), 215 * 215)
                a, c = divmod(ac, 215)
                b, d = divmod(bd, 215)
                for x, y in ((a, c), (b, d)):
                    assert oracle_mod.triangrk(lv[x - 1], kk, lv[y - 1])
    e1 = o.setham(ab.ncf, ab.nnz, ab.iendc, ab.iq, ab.tlist, ab.vlists)
    e2 = o.setham(ab.ncf, ab.nnz, ab.iendc, ab.iq, ab.tlist, ab.vlists)
    np.testing.assert_array_equal(e1, e2)


def test_diagonal_one_body_coefficients_count_electrons():
    """Every diagonal element's I(aa) coefficients add up to the number of
    electrons (He: 2), whatever the CSF's couplings."""
    csl = F.read_csl(f"{G.ROOT}/{G.RUNS['He']}.c")
    ab = A.block_lists(csl, 0)
    nw = len(csl.subshells)
    diag_loc = ab.iendc[1:]
    tot = np.zeros(ab.ncf)
    t = ab.tlist
    for li, lab in enumerate(t["lab"]):
        a, b = divmod(int(lab), 215)
        if a != b:
            continue
        for p in range(t["start"][li], t["start"][li + 1]):
            r = np.searchsorted(diag_loc, t["loc"][p])
            if diag_loc[r] == t["loc"][p]:
                tot[r] += t["coeff"][p]
    np.testing.assert_allclose(tot, 2.0, atol=1e-13)
    assert nw == 36


def test_average_split_lists_give_the_same_matrix(oracle_mod):
    """rangular's convention for rmcdhf: the lists without the diagonal
    pieces SETHAM adds from the occupations (FCO/GCO), assembled with the
    CSFs' IQ, give the same Hamiltonian as the whole-H lists with zero IQ;
    closed-subshell terms are then absent from the lists, which are
    shorter."""
    for run in ("He", "Ge"):
        d, csl, o = _chain(oracle_mod, run)
        ab = A.block_lists(csl, 0)
        sp = A.block_lists(csl, 0, average_split=True)
        np.testing.assert_array_equal(sp.iendc, ab.iendc)
        np.testing.assert_array_equal(sp.irow, ab.irow)
        assert sp.iq.any() and not ab.iq.any()
        e_full = o.setham(ab.ncf, ab.nnz, ab.iendc, ab.iq, ab.tlist, ab.vlists)
        e_split = o.setham(sp.ncf, sp.nnz, sp.iendc, sp.iq, sp.tlist, sp.vlists)
        assert np.abs(e_split - e_full).max() <= 1e-12 * np.abs(e_full).max(), run
        assert sp.ncontr < ab.ncontr


def test_mcp_files_from_the_engine(tmp_path, oracle_mod):
    """The engine's lists written as mcp.30/31/32+k (rangular's files for
    rmcdhf) and read back give the same SETHAM."""
    d, csl, o = _chain(oracle_mod, "He")
    s = A.mcp_set(csl, nelec=2)
    head = str(tmp_path / "mcp")
    F.write_mcp(head, s)
    r = F.read_mcp(head)
    assert [b.ncf for b in r.blocks] == [70, 180, 222] and r.kmaxf == s.kmaxf
    for bi, b in enumerate(r.blocks):
        ab = A.block_lists(csl, bi, average_split=True)
        e0 = o.setham(ab.ncf, ab.nnz, ab.iendc, ab.iq, ab.tlist, ab.vlists)
        e1 = o.setham(b.ncf, int(b.iendc[-1]), b.iendc, ab.iq, b.tlist, b.vlists)
        np.testing.assert_array_equal(e0, e1)
