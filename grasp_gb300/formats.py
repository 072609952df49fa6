"""GRASP's file formats at the boundary of the CI stage, read and written
byte-compatibly (Fortran unformatted sequential records: each record framed
by its int32 byte length before and after; little-endian; default INTEGER is
int32, REAL*8 is float64, LOGICAL is 4 bytes).

  mcp.30        angular structure: file header, then per block the CSR-lower
                structure MATRIX reads (rmcdhf90/matrix.f90:123-140)
  mcp.31        one-body (T) coefficient lists, sorted by label
  mcp.32+k      two-body (V^k) coefficient lists, k = 0..KMAXF
                (record layouts: rangular90/setmcp.f90:80-82, setmcp2.f90:49-50,
                sortmem.f90:232-284; read by rmcdhf90/setmcp.f90:78-137 and
                rmcdhf90/setham.f90:223-341)
  rwfn          radial wavefunctions (lib9290/lodrwf.f90:100-108)
  .cm / .mix    mixing coefficients (rci90/matrix.f90:209-212, lodmix.f90:75)
  rci.res       rci's run parameters and stored Hamiltonian rows, with rci's
                element filter (rci90/setres.f90:105, getcid.f90:284-314,
                genmat.f90:117, setham_gg.f90:364-378; lodres.f90:58-101)

The coefficient lists convert to and from the label-grouped arrays that
:meth:`grasp_gb300.HMatrix.setham` takes (dicts of lab/start/loc/coeff).
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass, field

import numpy as np

_I4 = np.dtype("<i4")
_F8 = np.dtype("<f8")


class FortranFile:
    """Sequential unformatted records with 4-byte length markers."""

    def __init__(self, path, mode="rb"):
        self.f = open(path, mode)

    def close(self):
        self.f.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def read_record(self) -> bytes:
        head = self.f.read(4)
        if len(head) < 4:
            raise EOFError
        (n,) = struct.unpack("<i", head)
        data = self.f.read(n)
        (m,) = struct.unpack("<i", self.f.read(4))
        if m != n or len(data) != n:
            raise ValueError("corrupt record markers")
        return data

    def write_record(self, *parts):
        data = b"".join(p if isinstance(p, (bytes, bytearray)) else np.ascontiguousarray(p).tobytes()
                        for p in parts)
        self.f.write(struct.pack("<i", len(data)))
        self.f.write(data)
        self.f.write(struct.pack("<i", len(data)))


def _i4(*v):
    return np.array(v, dtype=_I4)


def _chars(s, n):
    b = s.encode("ascii")
    return b[:n].ljust(n, b" ")


# ---------------------------------------------------------------------------
# mcp files
# ---------------------------------------------------------------------------

@dataclass
class McpBlock:
    """One J/parity block: structure (mcp.30) and coefficient lists."""
    ncf: int
    iendc: np.ndarray                   # int64 [ncf + 1], IENDC(0) = 0
    irow: np.ndarray                    # int32 [nnz], 1-based
    tlist: dict = None                  # lab/start/loc/coeff (+ iclmn)
    vlists: list = field(default_factory=list)


@dataclass
class McpSet:
    ncore: int
    nelec: int
    ncf: int                            # NCF of the file header (all blocks)
    nw: int
    kmaxf: int
    idblk: list
    blocks: list
    diag: bool = False
    iccut: int = 0
    lfordr: bool = False
    myid: int = 0
    nprocs: int = 1


def _write_common_header(ff, s: McpSet):
    ff.write_record(_chars("MCP", 3), _i4(len(s.blocks), s.myid, s.nprocs))
    ff.write_record(_i4(s.nelec, s.ncf, s.nw))
    ff.write_record(_i4(int(s.diag), s.iccut, int(s.lfordr)))


def _read_common_header(ff):
    r = ff.read_record()
    lab = r[:3].decode("ascii")
    nb, myid, nprocs = np.frombuffer(r[3:15], _I4)
    if lab != "MCP":
        raise ValueError("not a sorted GRASP92 MCP file")
    nelec, ncf, nw = np.frombuffer(ff.read_record(), _I4)
    diag, iccut, lfordr = np.frombuffer(ff.read_record(), _I4)
    return int(nb), int(myid), int(nprocs), int(nelec), int(ncf), int(nw), bool(diag), int(iccut), bool(lfordr)


def _write_list(ff, jblock, ncf, lst):
    lab = np.asarray(lst["lab"], _I4)
    start = np.asarray(lst["start"], np.int64)
    loc = np.asarray(lst["loc"], _I4)
    coeff = np.asarray(lst["coeff"], _F8)
    iclmn = np.asarray(lst.get("iclmn", np.zeros(loc.size, _I4)), _I4)
    ff.write_record(_chars("MCP", 3), _i4(jblock, ncf, loc.size))
    rec = np.dtype([("iclmn", _I4), ("index", _I4), ("coeff", _F8)])
    for l in range(lab.size):
        a, b = int(start[l]), int(start[l + 1])
        ff.write_record(_i4(lab[l], b - a))
        data = np.empty(b - a, rec)
        data["iclmn"], data["index"], data["coeff"] = iclmn[a:b], loc[a:b], coeff[a:b]
        ff.write_record(data)
    ff.write_record(_i4(0, 0))


def _read_list(ff, jblock, ncf):
    r = ff.read_record()
    if r[:3].decode("ascii") != "MCP":
        raise ValueError("list block header missing")
    jb, ncft, ncoeff = np.frombuffer(r[3:15], _I4)
    if jb != jblock or ncft != ncf:
        raise ValueError(f"list block {jb}/{ncft} where block {jblock}/{ncf} expected")
    rec = np.dtype([("iclmn", _I4), ("index", _I4), ("coeff", _F8)])
    labs, starts, parts = [], [0], []
    while True:
        lab, ncontr = np.frombuffer(ff.read_record(), _I4)
        if lab == 0 and ncontr == 0:
            break
        d = np.frombuffer(ff.read_record(), rec)
        if d.size != ncontr:
            raise ValueError("contribution record of the wrong length")
        labs.append(int(lab))
        parts.append(d)
        starts.append(starts[-1] + int(ncontr))
    d = np.concatenate(parts) if parts else np.zeros(0, rec)
    return dict(lab=np.array(labs, np.int32), start=np.array(starts, np.int64),
                loc=np.ascontiguousarray(d["index"]), coeff=np.ascontiguousarray(d["coeff"]),
                iclmn=np.ascontiguousarray(d["iclmn"]))


def write_mcp(filehead, s: McpSet):
    """Writes filehead.30, filehead.31 and filehead.32 .. filehead.(32+kmaxf)."""
    nb = len(s.blocks)
    with FortranFile(f"{filehead}.30", "wb") as ff:
        ff.write_record(_i4(s.ncore, nb, s.kmaxf))
        ff.write_record(np.array([b.ncf for b in s.blocks], _I4))
        ff.write_record(b"".join(_chars(x, 8) for x in s.idblk))
        _write_common_header(ff, s)
        for j, b in enumerate(s.blocks, start=1):
            nnz = int(b.iendc[-1])
            ff.write_record(_chars("MCP", 3), _i4(j, b.ncf))
            ff.write_record(_i4(nnz))
            ff.write_record(np.asarray(b.iendc[1:], _I4), np.asarray(b.irow, _I4))
    for k in range(31, 33 + s.kmaxf):
        with FortranFile(f"{filehead}.{k}", "wb") as ff:
            _write_common_header(ff, s)
            for j, b in enumerate(s.blocks, start=1):
                lst = b.tlist if k == 31 else b.vlists[k - 32]
                _write_list(ff, j, b.ncf, lst)


def read_mcp(filehead) -> McpSet:
    """Reads the mcp files the way SETMCP, MATRIX and SETHAM do (one process)."""
    with FortranFile(f"{filehead}.30") as ff:
        ncore, nblock, kmaxf = (int(x) for x in np.frombuffer(ff.read_record(), _I4))
        ncfblk = np.frombuffer(ff.read_record(), _I4).copy()
        raw = ff.read_record()
        idblk = [raw[8 * i:8 * i + 8].decode("ascii") for i in range(nblock)]
        nb, myid, nprocs, nelec, ncf, nw, diag, iccut, lfordr = _read_common_header(ff)
        if nprocs != 1:
            raise ValueError("mcp files written for several processes")
        blocks = []
        for j in range(1, nblock + 1):
            r = ff.read_record()
            jb, ncfb = np.frombuffer(r[3:11], _I4)
            if jb != j or ncfb != ncfblk[j - 1]:
                raise ValueError("matrx: jblockt .NE. jblock .OR. ncf1 .NE. ncf2")
            (nnz,) = np.frombuffer(ff.read_record(), _I4)
            d = np.frombuffer(ff.read_record(), _I4)
            iendc = np.concatenate([[0], d[:ncfb]]).astype(np.int64)
            irow = d[ncfb:ncfb + nnz].copy()
            blocks.append(McpBlock(int(ncfb), iendc, irow))
    for k in range(31, 33 + kmaxf):
        with FortranFile(f"{filehead}.{k}") as ff:
            _read_common_header(ff)
            for j, b in enumerate(blocks, start=1):
                lst = _read_list(ff, j, b.ncf)
                if k == 31:
                    b.tlist = lst
                else:
                    b.vlists.append(lst)
    return McpSet(ncore, nelec, ncf, nw, kmaxf, idblk, blocks, diag, iccut, lfordr, myid, nprocs)


# ---------------------------------------------------------------------------
# rwfn (radial wavefunctions)
# ---------------------------------------------------------------------------

@dataclass
class Orbital:
    np: int
    nak: int
    e: float
    pz: float
    p: np.ndarray
    q: np.ndarray
    r: np.ndarray


def read_rwfn(path) -> list:
    out = []
    with FortranFile(path) as ff:
        if ff.read_record()[:6] != b"G92RWF":
            raise ValueError("not a G92RWF file")
        while True:
            try:
                r = ff.read_record()
            except EOFError:
                break
            npy, naky = np.frombuffer(r[:8], _I4)
            (ey,) = np.frombuffer(r[8:16], _F8)
            (my,) = np.frombuffer(r[16:20], _I4)
            d = np.frombuffer(ff.read_record(), _F8)
            rr = np.frombuffer(ff.read_record(), _F8)
            out.append(Orbital(int(npy), int(naky), float(ey), float(d[0]), d[1:1 + my].copy(),
                               d[1 + my:1 + 2 * my].copy(), rr[:my].copy()))
    return out


def write_rwfn(path, orbitals):
    with FortranFile(path, "wb") as ff:
        ff.write_record(b"G92RWF")
        for o in orbitals:
            my = o.p.size
            ff.write_record(_i4(o.np, o.nak), np.array([o.e], _F8), _i4(my))
            ff.write_record(np.array([o.pz], _F8), np.asarray(o.p, _F8), np.asarray(o.q, _F8))
            ff.write_record(np.asarray(o.r, _F8))


def orbitals_on_grid(orbitals, n, ld=None):
    """PF/QF [ld x nw] (column-major, zero beyond MF) and NAK/MF as the C ABI
    takes them, from rwfn records (the orbitals' grid must be the run's)."""
    nw = len(orbitals)
    ld = ld or n
    pf = np.zeros((nw, ld))
    qf = np.zeros((nw, ld))
    mf = np.zeros(nw, np.int32)
    nak = np.array([o.nak for o in orbitals], np.int32)
    for j, o in enumerate(orbitals):
        m = min(o.p.size, n)
        pf[j, :m], qf[j, :m] = o.p[:m], o.q[:m]
        mf[j] = m
    return nak, mf, pf, qf


# ---------------------------------------------------------------------------
# mixing coefficients (.cm)
# ---------------------------------------------------------------------------

@dataclass
class MixBlock:
    jblock: int
    ncf: int
    nvec: int
    two_j_plus_1: int
    parity: int
    ivec: np.ndarray
    eav: float
    eval: np.ndarray
    evec: np.ndarray                    # [ncf x nvec], column j = vector j


@dataclass
class MixFile:
    nelec: int
    ncftot: int
    nw: int
    nvectot: int
    nvecsiz: int
    blocks: list


def read_mix(path) -> MixFile:
    with FortranFile(path) as ff:
        if ff.read_record()[:6] != b"G92MIX":
            raise ValueError("not a G92MIX file")
        nelec, ncftot, nw, nvectot, nvecsiz, nblock = (int(x) for x in np.frombuffer(ff.read_record(), _I4))
        blocks = []
        for _ in range(nblock):
            jb, ncf, nvec, jj, par = (int(x) for x in np.frombuffer(ff.read_record(), _I4))
            if nvec <= 0:  # a block without vectors: its header only (rci90/matrix.f90:164-165)
                blocks.append(MixBlock(jb, ncf, nvec, jj, par, np.zeros(0, np.int32), 0.0, np.zeros(0),
                                       np.zeros((ncf, 0))))
                continue
            ivec = np.frombuffer(ff.read_record(), _I4).copy()
            d = np.frombuffer(ff.read_record(), _F8)
            ev = np.frombuffer(ff.read_record(), _F8).reshape(nvec, ncf).T.copy()
            blocks.append(MixBlock(jb, ncf, nvec, jj, par, ivec, float(d[0]), d[1:1 + nvec].copy(), ev))
    return MixFile(nelec, ncftot, nw, nvectot, nvecsiz, blocks)


def write_mix(path, m: MixFile):
    with FortranFile(path, "wb") as ff:
        ff.write_record(b"G92MIX")
        ff.write_record(_i4(m.nelec, m.ncftot, m.nw, m.nvectot, m.nvecsiz, len(m.blocks)))
        for b in m.blocks:
            ff.write_record(_i4(b.jblock, b.ncf, b.nvec, b.two_j_plus_1, b.parity))
            if b.nvec <= 0:
                continue
            ff.write_record(np.asarray(b.ivec, _I4))
            ff.write_record(np.concatenate([[b.eav], np.asarray(b.eval, _F8)]).astype(_F8))
            ff.write_record(np.asarray(b.evec, _F8).T.copy())


# ---------------------------------------------------------------------------
# rci.res (rci's run parameters and Hamiltonian rows)
# ---------------------------------------------------------------------------

# rci stores an off-diagonal element only if |H| > CUTOFF (rci90/setham_gg.f90:364)
RCI_CUTOFF = 1.0e-12


@dataclass
class ResOrbital:
    e: float
    gama: float
    pz: float
    p: np.ndarray                       # PF(1:MF)
    q: np.ndarray                       # QF(1:MF)


@dataclass
class ResHeader:
    """Records 1-7 + 2 NW of rci.res (rci90/setres.f90:105, getcid.f90:284-314;
    read back by rci90/lodres.f90:58-101)."""
    nelec: int
    ncf: int                            # all blocks
    nw: int
    z: float
    emn: float
    parm: np.ndarray                    # PARM(1:NPARM)
    zz: np.ndarray                      # ZZ(1:N)
    nnuc: int
    c: float
    lfordr: bool
    iccut: list                         # ICCUTblk, one per block
    ltrans: bool
    wfact: float
    lvp: bool
    lnms: bool
    lsms: bool
    rnt: float
    h: float
    hp: float
    r: np.ndarray                       # R, RP, RPOR: N + 10 points each
    rp: np.ndarray
    rpor: np.ndarray
    orbitals: list                      # ResOrbital, NW of them


@dataclass
class ResBlock:
    """One block's rows as rci writes them (rci90/genmat.f90:117,
    setham_gg.f90:378): the rows held by rank myid of nprocs (rows myid+1,
    myid+1+nprocs, ...), each lower-triangle row with its diagonal last.
    iendc/irow/emt are those rows in the CSR-lower layout of hmat_C; an
    interrupted run leaves fewer rows than res_rows(ncf, myid, nprocs)."""
    ncf: int
    iccut: int
    iendc: np.ndarray                   # int64 [rows + 1]
    irow: np.ndarray                    # int32, 1-based
    emt: np.ndarray                     # float64, without ELSTO
    elsto: float = 0.0
    myid: int = 0
    nprocs: int = 1


def res_rows(ncf, myid=0, nprocs=1):
    """Rows of a block that rank myid writes to rci.res: rows myid+1,
    myid+1+nprocs, ... up to NCF (the row loop of rci90/setham_gg.f90:160).
    genmat.f90:97-99 counts NCF/(MYID+1) rows where NCF < NPROCS, which is
    more than the rank wrote (ncf = 2, nprocs = 3: rank 0 wrote one row);
    the rows actually written are what a reader must take."""
    return max(0, (ncf - myid + nprocs - 1) // nprocs)


def rci_filter(iendc, irow, emt, cutoff=RCI_CUTOFF):
    """The rows rci stores for an assembled block: every diagonal element and
    the off-diagonal ones with |H| > cutoff (rci90/setham_gg.f90:364-368).
    Takes and returns the CSR-lower layout (IENDC with IENDC(0) = 0, 1-based
    IROW, diagonal last in each row); order within a row is kept."""
    iendc = np.asarray(iendc, np.int64)
    irow = np.asarray(irow, np.int32)
    emt = np.asarray(emt, np.float64)
    ncf = iendc.size - 1
    row_of = np.repeat(np.arange(1, ncf + 1, dtype=np.int64), np.diff(iendc))
    keep = (irow == row_of) | (np.abs(emt) > cutoff)
    kept_before = np.concatenate([[0], np.cumsum(keep, dtype=np.int64)])
    return kept_before[iendc], irow[keep].copy(), emt[keep].copy()


def res_eav(block: ResBlock):
    """EAV of a block whose rows are all present: the diagonal mean plus
    ELSTO (rci90/setham_gg.f90:382, genmat2.f90:36)."""
    diag = block.emt[block.iendc[1:] - 1]
    return float(diag.sum()) / block.ncf + block.elsto


def res_to_hmat(block: ResBlock, eav):
    """(iendc, irow, emt) with the diagonal shifted by -EAV, as rci's MANEIG
    loads rci.res into core (rci90/maneig.f90:318-330): the arrays
    HMatrix(ctx, ncf, iendc, irow) and HMatrix.set_emt take. The eigenvalues
    of that matrix plus EAV are rci's; plus ELSTO once more where rci adds it
    (rci90/matrix.f90:197-201)."""
    if block.nprocs != 1 or block.iendc.size - 1 != block.ncf:
        raise ValueError("a block's rows are all needed (one rank, no interrupted rows)")
    emt = block.emt.copy()
    emt[block.iendc[1:] - 1] -= eav
    return block.iendc.copy(), block.irow.copy(), emt


def merge_res_ranks(parts):
    """One block's rows from the rci.res files of all ranks of an MPI run
    (rank myid holds rows myid+1, myid+1+nprocs, ...; rci90/genmat.f90:77,
    setham_gg.f90:162) merged into a single-rank block, rows in order."""
    parts = sorted(parts, key=lambda b: b.myid)
    if not parts:
        raise ValueError("no rank files")
    ncf, nprocs = parts[0].ncf, parts[0].nprocs
    if [b.myid for b in parts] != list(range(nprocs)) or any(b.ncf != ncf or b.nprocs != nprocs for b in parts):
        raise ValueError("one block from every rank of the same run expected")
    for b in parts:
        if b.iendc.size - 1 != res_rows(ncf, b.myid, nprocs):
            raise ValueError(f"rank {b.myid} holds {b.iendc.size - 1} rows, not all of its own")
    lens = np.zeros(ncf, np.int64)
    for b in parts:
        lens[b.myid::nprocs] = np.diff(b.iendc)
    iendc = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    irow = np.zeros(iendc[-1], np.int32)
    emt = np.zeros(iendc[-1])
    for b in parts:
        for r in range(b.iendc.size - 1):
            i = b.myid + r * nprocs
            s, e = int(b.iendc[r]), int(b.iendc[r + 1])
            irow[iendc[i]:iendc[i + 1]] = b.irow[s:e]
            emt[iendc[i]:iendc[i + 1]] = b.emt[s:e]
    return ResBlock(ncf, parts[0].iccut, iendc, irow, emt, parts[0].elsto)


def _write_res_header(ff, hd: ResHeader):
    n = hd.zz.size
    ff.write_record(b"R92RES")
    ff.write_record(_i4(hd.nelec, hd.ncf, hd.nw, len(hd.iccut)))
    ff.write_record(np.array([hd.z, hd.emn], _F8))
    ff.write_record(_i4(len(hd.parm)), np.asarray(hd.parm, _F8))
    ff.write_record(_i4(n), np.asarray(hd.zz, _F8), _i4(hd.nnuc))
    ff.write_record(np.array([hd.c], _F8), _i4(int(hd.lfordr)), np.asarray(hd.iccut, _I4), _i4(int(hd.ltrans)),
                    np.array([hd.wfact], _F8), _i4(int(hd.lvp), int(hd.lnms), int(hd.lsms)))
    for a in (hd.r, hd.rp, hd.rpor):
        if np.asarray(a).size != n + 10:
            raise ValueError("R, RP and RPOR hold N + 10 points")
    ff.write_record(np.array([hd.rnt, hd.h, hd.hp], _F8), np.asarray(hd.r, _F8), np.asarray(hd.rp, _F8),
                    np.asarray(hd.rpor, _F8))
    if len(hd.orbitals) != hd.nw:
        raise ValueError("NW orbitals expected")
    for o in hd.orbitals:
        ff.write_record(np.array([o.e, o.gama, o.pz], _F8), _i4(np.asarray(o.p).size))
        ff.write_record(np.asarray(o.p, _F8), np.asarray(o.q, _F8))


def _read_res_header(ff) -> ResHeader:
    if ff.read_record()[:6] != b"R92RES":
        raise ValueError("not an RCI92 .res file")
    nelec, ncf, nw, nblock = (int(x) for x in np.frombuffer(ff.read_record(), _I4))
    z, emn = np.frombuffer(ff.read_record(), _F8)
    r = ff.read_record()
    (nparm,) = np.frombuffer(r[:4], _I4)
    parm = np.frombuffer(r[4:4 + 8 * nparm], _F8).copy()
    r = ff.read_record()
    (n,) = np.frombuffer(r[:4], _I4)
    zz = np.frombuffer(r[4:4 + 8 * n], _F8).copy()
    (nnuc,) = np.frombuffer(r[4 + 8 * n:8 + 8 * n], _I4)
    r = ff.read_record()
    (c,) = np.frombuffer(r[:8], _F8)
    (lfordr,) = np.frombuffer(r[8:12], _I4)
    iccut = [int(x) for x in np.frombuffer(r[12:12 + 4 * nblock], _I4)]
    o = 12 + 4 * nblock
    (ltrans,) = np.frombuffer(r[o:o + 4], _I4)
    (wfact,) = np.frombuffer(r[o + 4:o + 12], _F8)
    lvp, lnms, lsms = np.frombuffer(r[o + 12:o + 24], _I4)
    d = np.frombuffer(ff.read_record(), _F8)
    np10 = n + 10
    rnt, h, hp = d[:3]
    grid = [d[3 + i * np10:3 + (i + 1) * np10].copy() for i in range(3)]
    orbs = []
    for _ in range(nw):
        r = ff.read_record()
        e, gama, pz = np.frombuffer(r[:24], _F8)
        (mf,) = np.frombuffer(r[24:28], _I4)
        pq = np.frombuffer(ff.read_record(), _F8)
        orbs.append(ResOrbital(float(e), float(gama), float(pz), pq[:mf].copy(), pq[mf:2 * mf].copy()))
    return ResHeader(nelec, ncf, nw, float(z), float(emn), parm, zz, int(nnuc), float(c), bool(lfordr), iccut,
                     bool(ltrans), float(wfact), bool(lvp), bool(lnms), bool(lsms), float(rnt), float(h), float(hp),
                     grid[0], grid[1], grid[2], orbs)


def write_res(path, header: ResHeader, blocks):
    """rci.res: the header records, then per block its (NCF, ICCUT, MYID,
    NPROCS) record and one record (NELC, ELSTO, EMT(1:NELC), IROW(1:NELC))
    per row held (rci90/genmat.f90:117, setham_gg.f90:378)."""
    if len(blocks) != len(header.iccut):
        raise ValueError("one ICCUT per block")
    with FortranFile(path, "wb") as ff:
        _write_res_header(ff, header)
        for b in blocks:
            ff.write_record(_i4(b.ncf, b.iccut, b.myid, b.nprocs))
            iendc = np.asarray(b.iendc, np.int64)
            if iendc.size - 1 > res_rows(b.ncf, b.myid, b.nprocs):
                raise ValueError("more rows than the rank owns")
            for i in range(iendc.size - 1):
                s, e = int(iendc[i]), int(iendc[i + 1])
                ff.write_record(_i4(e - s), np.array([b.elsto], _F8), np.asarray(b.emt[s:e], _F8),
                                np.asarray(b.irow[s:e], _I4))


def read_res(path):
    """(ResHeader, [ResBlock]) from rci.res. A block's rows end where its
    rank's rows end or where the file ends (an interrupted run, which rci
    resumes from, rci90/genmat.f90:65-90)."""
    with FortranFile(path) as ff:
        hd = _read_res_header(ff)
        blocks = []
        for _ in range(len(hd.iccut)):
            try:
                r = ff.read_record()
            except EOFError:
                break
            ncf, iccut, myid, nprocs = (int(x) for x in np.frombuffer(r, _I4))
            lens, irows, emts, elsto = [0], [], [], 0.0
            for _ in range(res_rows(ncf, myid, nprocs)):
                try:
                    r = ff.read_record()
                except EOFError:
                    break
                (nelc,) = np.frombuffer(r[:4], _I4)
                (elsto,) = np.frombuffer(r[4:12], _F8)
                emts.append(np.frombuffer(r[12:12 + 8 * nelc], _F8))
                irows.append(np.frombuffer(r[12 + 8 * nelc:12 + 12 * nelc], _I4))
                lens.append(int(nelc))
            blocks.append(ResBlock(ncf, iccut, np.cumsum(lens).astype(np.int64),
                                   np.concatenate(irows).astype(np.int32) if irows else np.zeros(0, np.int32),
                                   np.concatenate(emts) if emts else np.zeros(0), float(elsto), myid, nprocs))
    return hd, blocks


def exists(path):
    return os.path.exists(path)


# ---------------------------------------------------------------------------
# CSF lists (.c)
# ---------------------------------------------------------------------------

@dataclass
class CslBlock:
    """One J/parity block of a CSF list, as LODCSH2 reads it
    (lib9290/lodcsh2.f90:150-330): per CSF the occupation of every subshell,
    the 2J and seniority of the open ones and the intermediate couplings."""
    two_j: int
    parity: int           # +1 even, -1 odd
    iq: np.ndarray        # uint8 [ncsf, nw]: electrons per subshell (IQ)
    jqs: np.ndarray       # int32 [ncsf, nw]: 2J of each open subshell, 0 for empty and closed ones
    nu: np.ndarray        # int32 [ncsf, nw]: seniority where the list gives it, else 0
    xj: np.ndarray        # int32 [ncsf, nw]: 2X after each open subshell (JCUP), -1 elsewhere

    @property
    def ncsf(self):
        return self.iq.shape[0]


@dataclass
class CslFile:
    subshells: list       # (n, kappa) in list order: core subshells, then peel subshells
    labels: list
    ncore: int
    blocks: list


_SHELL_L = "spdfghiklmn"


def subshell_kappa(label):
    """'4p-' -> (4, 1), '4p' -> (4, -2): j = l - 1/2 for a trailing '-'."""
    label = label.strip()
    neg = label.endswith("-")
    body = label[:-1] if neg else label
    n, l = int(body[:-1]), _SHELL_L.index(body[-1])
    return n, (l if neg else -(l + 1))


def _two_j(tok):
    tok = tok.strip().rstrip("+-")
    return int(tok[:-2]) if tok.endswith("/2") else 2 * int(tok)


def read_csl(path) -> CslFile:
    """A GRASP CSF list (rcsfgenerate's .c file, read by LODCSH/LODCSH2):
    the core and peel subshell records, then three lines per CSF — the
    occupied peel subshells with their occupations, the 2J (and, where
    ambiguous, seniority 'nu;J') of each open subshell, the intermediate
    couplings of the open subshells after the first whose J is not zero,
    and the final J with the parity sign — blocks separated by ' *'."""
    lines = open(path).read().splitlines()
    core = lines[lines.index("Core subshells:") + 1].split()
    peel = lines[lines.index("Peel subshells:") + 1].split()
    labels = core + peel
    shells = [subshell_kappa(s) for s in labels]
    index = {s: i for i, s in enumerate(labels)}
    nw = len(shells)
    cap = [2 * abs(k) for _, k in shells]
    body = lines[lines.index("CSF(s):") + 1:]
    blocks, cur = [], []

    def flush():
        if not cur:
            return
        iq = np.array([c[0] for c in cur], np.uint8)
        jqs = np.array([c[1] for c in cur], np.int32)
        nu = np.array([c[2] for c in cur], np.int32)
        xj = np.array([c[3] for c in cur], np.int32)
        tj = {c[4] for c in cur}
        par = {c[5] for c in cur}
        if len(tj) != 1 or len(par) != 1:
            raise ValueError("a block holds CSFs of one J and parity")
        blocks.append(CslBlock(tj.pop(), par.pop(), iq, jqs, nu, xj))
        cur.clear()

    i = 0
    import re
    pat = re.compile(r"(\d+[a-z]-?)\s*\(\s*(\d+)\)")
    while i < len(body):
        if body[i].strip() == "*":
            flush()
            i += 1
            continue
        if not body[i].strip():
            i += 1
            continue
        occ_line, j_line, x_line = body[i], body[i + 1], body[i + 2]
        i += 3
        iq = [cap[a] if a < len(core) else 0 for a in range(nw)]
        for lab, q in pat.findall(occ_line):
            iq[index[lab]] = int(q)
        jtoks = j_line.split()
        xtoks = x_line.split()
        parity = 1 if xtoks[-1].endswith("+") else -1
        jqs = [0] * nw
        nu = [0] * nw
        xj = [-1] * nw
        jl = xl = 0
        jlast = None
        for a in range(len(core), nw):
            if iq[a] == 0 or iq[a] == cap[a]:
                continue
            tok = jtoks[jl]
            jl += 1
            if ";" in tok:
                s, t = tok.split(";")
                nu[a] = int(s)
                jqs[a] = _two_j(t)
            else:
                jqs[a] = _two_j(tok)
            if jlast is None:
                jlast = jqs[a]
            elif jqs[a] == 0:
                pass
            else:
                jlast = _two_j(xtoks[xl])
                xl += 1
            xj[a] = jlast
        final = _two_j(xtoks[-1])
        if jlast is None:
            jlast = 0
        if final != jlast:
            raise ValueError(f"{path}: final J does not match the couplings of CSF {len(cur) + 1}")
        cur.append((iq, jqs, nu, xj, final, parity))
    flush()
    return CslFile(shells, labels, len(core), blocks)
